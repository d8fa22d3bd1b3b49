"""Convective flux functors (navier-stokes/convective.h)."""
from . import _abi


class cent_keep_scheme_t:
    """convective::cent_keep_scheme_t<gas, order> (convective.h:96-192)."""

    def __init__(self, gas, order):
        if order not in (2, 4, 6, 8):
            raise ValueError("cent_keep order must be 2, 4, 6 or 8")
        self.gas = gas
        self.order = int(order)
        self.kind = _abi.CONV_CENT_KEEP


def cent_keep(order, gas):
    """convective::cent_keep<order>(gas) (convective.h:187-192)."""
    if order % 2:
        raise ValueError("nominal order for centered scheme must be even")
    return cent_keep_scheme_t(gas, order)


class totani_lr:
    """convective::totani_lr(gas) (convective.h:54-94): 2-point KEEP."""

    def __init__(self, gas):
        self.gas = gas
        self.order = 2
        self.kind = _abi.CONV_TOTANI


enable_smooth = 1
disable_smooth = 0


class fweno_t:
    """convective::fweno_t<gas, smooth> (convective.h:335-497): 4-point,
    3rd-order WENO on a per-point Rusanov split."""

    def __init__(self, gas, smooth=enable_smooth):
        self.gas = gas
        self.order = 2
        self.smooth = int(smooth)
        self.kind = _abi.CONV_FWENO


class weno5_t:
    """5th-order WENO-JS on fweno_t's Rusanov split (6-point stencil, three
    ghost layers).  No reference counterpart."""

    def __init__(self, gas, smooth=enable_smooth):
        self.gas = gas
        self.order = 2
        self.smooth = int(smooth)
        self.kind = _abi.CONV_WENO5


class pressure_diss_lr:
    """convective::pressure_diss_lr(gas, sensor, eps_p[, eps_T])
    (convective.h:194-246)."""

    def __init__(self, gas, sensor, eps_p, eps_T=None):
        self.gas = gas
        self.sensor = sensor
        self.eps_p = float(eps_p)
        self.eps_T = float(eps_p if eps_T is None else eps_T)


class hybrid_secheme_tag_t:
    """convective::hybrid_secheme_tag_t<full> (hybrid_scheme.h:5-12)."""

    def __init__(self, full):
        self.value = bool(full)
        self.kind = _abi.HYBRID_FULL_FLUX if full else _abi.HYBRID_DISS_FLUX


full_flux = hybrid_secheme_tag_t(True)
diss_flux = hybrid_secheme_tag_t(False)


class hybrid_scheme_t:
    """convective::hybrid_scheme_t(scheme0, scheme1, blender, tag)
    (hybrid_scheme.h:14-47): the face flux (1 - s) F0 + s F1 (full_flux) or
    F0 + s F1 (diss_flux), s = blender.get_sensor at the face.  Lowered for
    scheme0 = cent_keep<2|4>, scheme1 = fweno_t and a const_sensor_t or
    ducros_t blender."""

    def __init__(self, scheme0, scheme1, blender, tag):
        if not isinstance(scheme0, cent_keep_scheme_t) or scheme0.order not in (2, 4):
            raise ValueError("hybrid_scheme_t is lowered with scheme0 = cent_keep<2> or cent_keep<4>")
        if not isinstance(scheme1, fweno_t):
            raise ValueError("hybrid_scheme_t is lowered with scheme1 = fweno_t")
        g0, g1 = scheme0.gas, scheme1.gas
        if g0.gamma != g1.gamma or g0.R != g1.R:
            raise ValueError("hybrid_scheme_t schemes must share one gas")
        self.scheme0 = scheme0
        self.scheme1 = scheme1
        self.blender = blender
        self.tag = tag
        self.gas = g0
        self.order = scheme0.order
        self.smooth = scheme1.smooth
        self.kind = _abi.CONV_HYBRID
