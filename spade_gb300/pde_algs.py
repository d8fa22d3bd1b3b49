"""pde_algs::flux_div and its traits (pde-algs/flux-div/flux_div.h:16-56,
pde-algs/pde_traits.h:5-20, pde-algs/flux-div/tags.h:5-33), source_term and
boundary_flux, lowered onto libgbns.so."""
import ctypes

from . import _abi, _native, convective, viscous, omni
from .grid import _stream, refined_layout_t


class _trait:
    def __init__(self, label, name, **kw):
        self.trait_label = label
        self.name = name
        self.__dict__.update(kw)

    def __repr__(self):
        return "pde_algs.%s" % self.name


# pde_increment trait (pde_traits.h:13-20)
overwrite = _trait("pde_increment", "overwrite", increment_mode=False)
increment = _trait("pde_increment", "increment", increment_mode=True)
# flux_div algorithm tag: the GB300 fused tile kernel
gb300 = _trait("flux_div", "gb300")
basic = gb300   # the reference's default tag maps to the same kernel here
# flux arithmetic precision
fp64 = _trait("flux_precision", "fp64", precision=_abi.PREC_FP64)
fp32_flux = _trait("flux_precision", "fp32_flux", precision=_abi.PREC_FP32_FLUX)
fp64_fma = _trait("flux_precision", "fp64_fma", precision=_abi.PREC_FP64_FMA)


def lower(flux_func, precision=_abi.PREC_FP64):
    """Lowers a flux functor (or omni.compose of functors) to the C ABI's
    gbns_scheme_desc.  Raises for anything the GB300 kernels do not
    implement (there is no CPU fallback)."""
    kernels = flux_func.kernels if isinstance(flux_func, omni.composite_kernel_t) else (flux_func,)
    s = _abi.SchemeDesc()
    s.order = 2
    s.weno_smooth = 1
    s.precision = int(precision)
    s.prandtl = 1.0
    s.T_ref = 1.0
    gas = None
    order = []   # canonical order: convective, dissipation, viscous
    for k in kernels:
        if isinstance(k, (convective.cent_keep_scheme_t, convective.totani_lr, convective.fweno_t, convective.weno5_t,
                          convective.hybrid_scheme_t)):
            if s.convective != _abi.CONV_NONE:
                raise _native.SpadeError(_abi.ERR_UNSUPPORTED, "at most one convective functor per composite")
            s.convective = k.kind
            s.order = k.order
            s.weno_smooth = getattr(k, "smooth", 1)
            if k.kind == _abi.CONV_HYBRID:
                s.hybrid_flux = k.tag.kind
                s.hybrid_sensor = k.blender.kind
                s.hybrid_param = k.blender.alpha
            order.append(0)
        elif isinstance(k, convective.pressure_diss_lr):
            if s.dissipation:
                raise _native.SpadeError(_abi.ERR_UNSUPPORTED, "at most one pressure_diss_lr per composite")
            s.dissipation = _abi.DISS_PRESSURE
            s.sensor = k.sensor.kind
            s.sensor_alpha = k.sensor.alpha
            s.eps_p = k.eps_p
            s.eps_T = k.eps_T
            order.append(1)
        elif isinstance(k, viscous.visc_lr):
            if s.viscous:
                raise _native.SpadeError(_abi.ERR_UNSUPPORTED, "at most one visc_lr per composite")
            s.viscous = _abi.VISC_LR
            law = k.vlaw
            s.visc_law = law.law
            s.mu = law.mu
            s.prandtl = law.prandtl
            s.T_ref = law.T_ref
            s.power = law.power
            s.S = law.S
            order.append(2)
        else:
            raise _native.SpadeError(_abi.ERR_UNSUPPORTED, "flux functor %r cannot be lowered to the GB300 kernels" % (k,))
        g = k.gas
        if gas is not None and (g.gamma != gas.gamma or g.R != gas.R):
            raise _native.SpadeError(_abi.ERR_UNSUPPORTED, "all functors of a composite must share one gas")
        gas = g
    # compose(a, b, c) = a + (b + c); a two-term sum commutes exactly, a
    # three-term sum is lowered only in the canonical order.
    if len(order) == 3 and order != [0, 1, 2]:
        raise _native.SpadeError(_abi.ERR_UNSUPPORTED, "three-term composites must be compose(convective, dissipation, viscous)")
    s.gas.gamma = gas.gamma
    s.gas.R = gas.R
    return s


def _traits(traits):
    inc, prec = True, _abi.PREC_FP64
    for t in traits or ():
        lab = getattr(t, "trait_label", None)
        if lab == "pde_increment":
            inc = t.increment_mode
        elif lab == "flux_precision":
            prec = t.precision
        elif lab != "flux_div":
            raise ValueError("unknown trait %r" % (t,))
    return inc, prec


def flux_div_refined(layout, prims, rhs, flux_func, traits=None, stream=None):
    """rhs (+)= div F(prims) on a refined layout (grid.refined_layout_t):
    pde_algs::flux_div on an amr_blocks_t grid, every block with its own
    spacing (gbns_flux_div_blocks; gbns_flux_div_blocks_host for CPU
    tensors, which returns with rhs updated).  prims must hold the ghost
    values of the layout's exchange (grid.exchange_plan_t)."""
    if not isinstance(layout, refined_layout_t):
        raise TypeError("layout must be a grid.refined_layout_t")
    inc, prec = _traits(traits)
    layout.check(prims)
    layout.check(rhs)
    scheme = flux_func if isinstance(flux_func, _abi.SchemeDesc) else lower(flux_func, prec)
    args = (layout.desc(), scheme, layout.boxes_ptr(), ctypes.c_void_p(prims.data_ptr()), ctypes.c_void_p(rhs.data_ptr()),
            int(inc))
    if prims.device.type == "cpu" and rhs.device.type == "cpu":
        _native.check(_native.lib().gbns_flux_div_blocks_host(*args, None))
    elif prims.is_cuda and rhs.is_cuda:
        _native.check(_native.lib().gbns_flux_div_blocks(*args, _stream(stream)))
    else:
        raise ValueError("prims and rhs must both be on the CPU or both on the GPU")


def flux_div(prims, rhs, flux_func, traits=None, stream=None, variant=0):
    """rhs (+)= div F(prims): pde_algs::flux_div(prims, rhs, flux_func[, traits]).
    Default increment mode like the reference; pass
    make_traits(pde_algs.overwrite) to overwrite.  Asynchronous on the
    current torch stream for device arrays; arrays on the CPU are staged
    through the GPU (gbns_flux_div_host) and the call returns with rhs
    updated."""
    inc, prec = _traits(traits)
    if prims.shape != rhs.shape or prims.grid is not rhs.grid and prims.shape != rhs.shape:
        raise ValueError("prims and rhs must live on the same grid")
    scheme = flux_func if isinstance(flux_func, _abi.SchemeDesc) else lower(flux_func, prec)
    on_cpu = prims.data.device.type == "cpu", rhs.data.device.type == "cpu"
    if any(on_cpu):
        if not all(on_cpu):
            raise ValueError("prims and rhs must both be on the CPU or both on the GPU")
        if variant:
            raise ValueError("tile variants select kernels for device arrays")
        if not (prims.data.is_contiguous() and rhs.data.is_contiguous()):
            raise ValueError("host arrays must be contiguous")
        _native.check(_native.lib().gbns_flux_div_host(prims.desc(), scheme, prims.ptr(), rhs.ptr(), int(inc), None))
        return
    if variant:
        rc = _native.lib().gbns_flux_div_variant(prims.desc(), scheme, prims.ptr(), rhs.ptr(), int(inc), int(variant), _stream(stream))
    else:
        rc = _native.lib().gbns_flux_div(prims.desc(), scheme, prims.ptr(), rhs.ptr(), int(inc), _stream(stream))
    _native.check(rc)


# ---------------------------------------------------------------- source_term

class const_source_t:
    """A constant point source: the flux_t (rho, rhoE, rhou, rhov, rhow)."""

    def __init__(self, values):
        values = [float(x) for x in values]
        if len(values) != 5:
            raise ValueError("a source is a flux_t of 5 values")
        self.kind = _abi.SOURCE_CONST
        self.c = values
        self.R = 0.0


class body_force_t:
    """Body force per unit volume f: S = (0, f.u, f_x, f_y, f_z)."""

    def __init__(self, fx, fy=0.0, fz=0.0):
        self.kind = _abi.SOURCE_BODY_FORCE
        self.c = [0.0, 0.0, float(fx), float(fy), float(fz)]
        self.R = 0.0


class body_accel_t:
    """Acceleration g (force per unit mass): S = rho (0, g.u, g_x, g_y, g_z),
    rho = p/(R T) from the gas."""

    def __init__(self, gas, gx, gy=0.0, gz=0.0):
        self.kind = _abi.SOURCE_BODY_ACCEL
        self.c = [0.0, 0.0, float(gx), float(gy), float(gz)]
        self.R = float(gas.R)


def lower_source(src):
    if not isinstance(src, (const_source_t, body_force_t, body_accel_t)):
        raise _native.SpadeError(_abi.ERR_UNSUPPORTED, "source %r cannot be lowered to the GB300 kernels" % (src,))
    d = _abi.SourceDesc()
    d.kind = src.kind
    for v in range(5):
        d.c[v] = src.c[v]
    d.gas.gamma = 1.4
    d.gas.R = src.R
    return d


def source_term(q, rhs, source_func, stream=None):
    """rhs += S(q)/jac on every interior cell: pde_algs::source_term(q, rhs,
    source_func) (pde-algs/source_term.h:19-51) for the lowered point
    sources const_source_t, body_force_t and body_accel_t.  Asynchronous on
    the current torch stream."""
    if q.shape != rhs.shape:
        raise ValueError("q and rhs must live on the same grid")
    d = lower_source(source_func)
    _native.check(_native.lib().gbns_source_term(q.desc(), d, q.ptr(), rhs.ptr(), _stream(stream)))


# -------------------------------------------------------------- boundary_flux

class bound_box_t:
    """bound_box_t<bool, 3>: one flag per domain boundary, min(i) / max(i)."""

    def __init__(self, value=False):
        self._min = [bool(value)] * 3
        self._max = [bool(value)] * 3

    def min(self, i, value=None):
        if value is None:
            return self._min[i]
        self._min[i] = bool(value)

    def max(self, i, value=None):
        if value is None:
            return self._max[i]
        self._max[i] = bool(value)

    def __invert__(self):
        out = bound_box_t()
        out._min = [not v for v in self._min]
        out._max = [not v for v in self._max]
        return out

    def flags(self):
        """The six flags in the order xmin, xmax, ymin, ymax, zmin, zmax."""
        return [f for i in range(3) for f in (self._min[i], self._max[i])]


def boundary_flux(prims, rhs, apply_to_boundary, flux_func, stream=None):
    """pde_algs::boundary_flux(prims, rhs, apply_to_boundary, flux_func)
    (pde-algs/boundary_flux.h:16-105): for each selected domain boundary the
    faces of the boundary plane (transverse indices -1 .. n-1) add their flux
    F to the two cells they separate, rhs(il) -= F/dx and rhs(ir) += F/dx.
    apply_to_boundary is a bound_box_t or six flags (xmin, xmax, ymin, ymax,
    zmin, zmax).  FP64 without FMA contraction; identity coordinates.
    Asynchronous on the current torch stream."""
    if prims.shape != rhs.shape:
        raise ValueError("prims and rhs must live on the same grid")
    flags = apply_to_boundary.flags() if isinstance(apply_to_boundary, bound_box_t) else list(apply_to_boundary)
    if len(flags) != 6:
        raise ValueError("apply_to_boundary needs six flags")
    scheme = flux_func if isinstance(flux_func, _abi.SchemeDesc) else lower(flux_func, _abi.PREC_FP64)
    arr = (ctypes.c_int * 6)(*[int(bool(f)) for f in flags])
    _native.check(_native.lib().gbns_boundary_flux(prims.desc(), scheme, prims.ptr(), rhs.ptr(), arr, _stream(stream)))
