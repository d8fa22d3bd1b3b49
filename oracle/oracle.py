"""Python access to the CPU oracle.  TEST INFRASTRUCTURE ONLY.

Two back ends:
  * ``port`` — oracle/_build/libgbns_oracle.so, the plain-C restatement of
    the reference's algorithm (oracle/gbns_oracle.c).  Built by
    ``make -C oracle`` (and by ``__graft_entry__.build()``).
  * ``ref``  — oracle/_ref/libspade_ref.so, the reference's own CPU path
    (oracle/ref_harness.cc compiled against the reference headers).  Only
    available where the reference sources exist; used to pin the port and
    to generate tests/golden/.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
import this module.  Arrays are numpy float64 in the AoS5 layout with ghosts,
shape (nblocks, nz+2ng, ny+2ng, nx+2ng, 5).
"""
import ctypes
import os
import numpy as np

from spade_gb300 import _abi

_HERE = os.path.dirname(os.path.abspath(__file__))
PORT_PATH = os.path.join(_HERE, "_build", "libgbns_oracle.so")
REF_PATH = os.path.join(_HERE, "_ref", "libspade_ref.so")

_port = None
_ref = None


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.c_void_p)


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_PATH):
            raise RuntimeError("oracle port not built: run `make -C oracle` (missing %s)" % PORT_PATH)
        lib = ctypes.CDLL(PORT_PATH)
        P = ctypes.POINTER
        lib.oracle_flux_div.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        lib.oracle_fill_ghosts.argtypes = [P(_abi.GridDesc), P(_abi.BcDesc), ctypes.c_void_p]
        lib.oracle_rk_stage.argtypes = [P(_abi.GridDesc), P(_abi.GasDesc), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
        lib.oracle_reduce.argtypes = [P(_abi.GridDesc), P(_abi.GasDesc), ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.oracle_ssprk3_step.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), P(_abi.BcDesc), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
        lib.oracle_max_threads.restype = ctypes.c_int
        lib.oracle_source_term.argtypes = [P(_abi.GridDesc), P(_abi.SourceDesc), ctypes.c_void_p, ctypes.c_void_p]
        lib.oracle_boundary_flux.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), ctypes.c_void_p, ctypes.c_void_p, P(ctypes.c_int)]
        lib.oracle_exchange_patches.argtypes = [ctypes.c_int] * 5 + [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p]
        lib.oracle_flux_div_blocks.argtypes = [P(_abi.GridDesc), P(_abi.SchemeDesc), ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        _port = lib
    return _port


def ref_available():
    return os.path.exists(REF_PATH)


def ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference harness not built (missing %s)" % REF_PATH)
        lib = ctypes.CDLL(REF_PATH)
        lib.spade_ref_flux_div.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.spade_ref_fill_ghosts.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.spade_ref_ssprk3.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.spade_ref_source_term.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.spade_ref_amr_exchange.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong, ctypes.c_void_p,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                               ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.spade_ref_amr_flux_div.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_longlong,
                                               ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        lib.spade_ref_amr_ssprk3.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_longlong, ctypes.c_void_p, ctypes.c_int]
        lib.spade_ref_amr_fill.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_longlong, ctypes.c_void_p]
        _ref = lib
    return _ref


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("%s failed with code %d" % (what, rc))


# ---------------------------------------------------------------- port API

def flux_div(grid, scheme, prims, rhs, increment=True, nthreads=0):
    _check(port().oracle_flux_div(ctypes.byref(grid), ctypes.byref(scheme), _ptr(prims), _ptr(rhs), int(increment), int(nthreads)), "oracle_flux_div")


def flux_div_blocks(grid, scheme, boxes, prims, rhs, increment=True, nthreads=0):
    """flux_div on a refined layout: grid.nblk = (blocks, 1, 1), identity
    coordinates, boxes (blocks, 6) the per-block min/max per direction."""
    b = np.ascontiguousarray(boxes, dtype=np.float64)
    _check(port().oracle_flux_div_blocks(ctypes.byref(grid), ctypes.byref(scheme), _ptr(b), _ptr(prims), _ptr(rhs),
                                         int(increment), int(nthreads)), "oracle_flux_div_blocks")


def fill_ghosts(grid, bc, prims):
    _check(port().oracle_fill_ghosts(ctypes.byref(grid), ctypes.byref(bc), _ptr(prims)), "oracle_fill_ghosts")


def rk_stage(grid, gas, prims, residuals, coeffs):
    ptrs = (ctypes.c_void_p * len(residuals))(*[r.ctypes.data for r in residuals])
    c = np.ascontiguousarray(coeffs, dtype=np.float64)
    _check(port().oracle_rk_stage(ctypes.byref(grid), ctypes.byref(gas), _ptr(prims), ptrs, _ptr(c), len(residuals)), "oracle_rk_stage")


def reduce(grid, gas, prims, kind):
    out = np.zeros(5)
    _check(port().oracle_reduce(ctypes.byref(grid), ctypes.byref(gas), _ptr(prims), int(kind), _ptr(out)), "oracle_reduce")
    return out if kind == _abi.RED_CONSERVED else float(out[0])


def ssprk3_step(grid, scheme, bc, prims, work, dt, nthreads=0):
    _check(port().oracle_ssprk3_step(ctypes.byref(grid), ctypes.byref(scheme), ctypes.byref(bc), _ptr(prims), _ptr(work), float(dt), int(nthreads)), "oracle_ssprk3_step")


def source_term(grid, src, prims, rhs):
    _check(port().oracle_source_term(ctypes.byref(grid), ctypes.byref(src), _ptr(prims), _ptr(rhs)), "oracle_source_term")


def boundary_flux(grid, scheme, prims, rhs, apply):
    """apply: six flags in the order xmin, xmax, ymin, ymax, zmin, zmax."""
    flags = (ctypes.c_int * 6)(*[int(bool(a)) for a in apply])
    _check(port().oracle_boundary_flux(ctypes.byref(grid), ctypes.byref(scheme), _ptr(prims), _ptr(rhs), flags),
           "oracle_boundary_flux")


def exchange_patches(ncell, ng, nblocks, plan, prims):
    """Executes an exchange plan ((n, 18) int32 gbns_patch records) on prims in place."""
    plan = np.ascontiguousarray(plan, dtype=np.int32)
    _check(port().oracle_exchange_patches(int(ncell[0]), int(ncell[1]), int(ncell[2]), int(ng), int(nblocks),
                                          plan.ctypes.data, int(plan.shape[0]), _ptr(prims)), "oracle_exchange_patches")


def max_threads():
    return int(port().oracle_max_threads())


# ---------------------------------------------------------- reference API

# Scheme ids understood by oracle/ref_harness.cc
REF_CK2_VISC = 0
REF_TOTANI_VISC = 1
REF_CK4_VISC = 2
REF_CK2 = 3
REF_VISC = 4
REF_FWENO_DISS_VISC = 5
REF_FWENO = 6
REF_DISS = 7
REF_TOTANI = 8
REF_CK6 = 9
REF_CK8 = 10
REF_FWENO_NOSMOOTH = 11
REF_CK2_DISS_VISC = 12
REF_DUCROS_DISS = 13
REF_FWENO_DUCROS_VISC = 14
REF_HYB_CK2_FULL = 15
REF_HYB_CK4_DISS_VISC = 16
REF_HYB_CK2_CONST_DISS_VISC = 17


def _ref_problem(grid, scheme, bc=None):
    """Flat int/real arrays for ref_harness.cc:make_problem."""
    periodic = [1, 1, 1]
    wall_y = 0
    t_wall = 0.0
    if bc is not None:
        periodic = [int(bc.kind[2 * d] == _abi.BC_PERIODIC) for d in range(3)]
        if bc.kind[2] == _abi.BC_ISOTHERMAL_NOSLIP:
            wall_y = 1
            t_wall = bc.t_wall[2]
    ints = np.array(list(grid.nblk) + list(grid.ncell) + [grid.ng] + periodic + [wall_y], dtype=np.int32)
    reals = np.array(list(grid.bounds) + [scheme.gas.gamma, scheme.gas.R, scheme.mu, scheme.prandtl,
                                          scheme.eps_p, scheme.eps_T, scheme.sensor_alpha, t_wall,
                                          scheme.hybrid_param], dtype=np.float64)
    return ints, reals


def ref_flux_div(ref_scheme, grid, scheme, prims, rhs, increment=True):
    ints, reals = _ref_problem(grid, scheme)
    _check(ref().spade_ref_flux_div(int(ref_scheme), ints.ctypes.data, reals.ctypes.data, int(not increment), _ptr(prims), _ptr(rhs)), "spade_ref_flux_div")


def ref_fill_ghosts(grid, scheme, bc, prims):
    ints, reals = _ref_problem(grid, scheme, bc)
    _check(ref().spade_ref_fill_ghosts(ints.ctypes.data, reals.ctypes.data, _ptr(prims)), "spade_ref_fill_ghosts")


def ref_ssprk3(ref_scheme, grid, scheme, bc, prims, dt, nsteps):
    ints, reals = _ref_problem(grid, scheme, bc)
    ke = np.zeros(nsteps + 1)
    _check(ref().spade_ref_ssprk3(int(ref_scheme), ints.ctypes.data, reals.ctypes.data, float(dt), int(nsteps), _ptr(prims), _ptr(ke)), "spade_ref_ssprk3")
    return ke


def ref_source_term(grid, scheme, src, prims, rhs):
    """source_term through the reference (kind and c of `src`; the gas
    constant comes from `scheme`)."""
    ints, reals = _ref_problem(grid, scheme)
    c = np.ascontiguousarray(np.array(list(src.c), dtype=np.float64))
    _check(ref().spade_ref_source_term(int(src.kind), ints.ctypes.data, reals.ctypes.data, c.ctypes.data, _ptr(prims), _ptr(rhs)),
           "spade_ref_source_term")


def ref_amr_exchange(nb, nc, ng, periodic, passes, bounds=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), cap_blocks=512, cap_plan=1 << 16):
    """The reference's AMR exchange on a grid refined in place pass by pass
    (oracle/ref_harness.cc spade_ref_amr_exchange).  Returns the array before
    and after the exchange (nblocks, nz+2ng, ny+2ng, nx+2ng, 5), the block
    boxes (nblocks, 6) and levels, and the plan: (ntransactions, 18) int32
    records, injections first (count `ninject`)."""
    ints = [nb[0], nb[1], nb[2], nc[0], nc[1], nc[2], ng] + [int(bool(p)) for p in periodic] + [len(passes)]
    for ps in passes:
        ints += [len(ps)] + list(ps)
    ints = np.array(ints, dtype=np.int32)
    b = np.array(bounds, dtype=np.float64)
    per_block = (nc[0] + 2 * ng) * (nc[1] + 2 * ng) * (nc[2] + 2 * ng) * 5
    cap = per_block * cap_blocks
    before = np.zeros(cap)
    after = np.zeros(cap)
    boxes = np.zeros(6 * cap_blocks)
    levels = np.zeros(cap_blocks, dtype=np.int32)
    plan = np.zeros(18 * cap_plan, dtype=np.int32)
    nblk, nplan, ninj = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_int(0)
    _check(ref().spade_ref_amr_exchange(ints.ctypes.data, b.ctypes.data, cap, before.ctypes.data, after.ctypes.data,
                                        ctypes.byref(nblk), boxes.ctypes.data, levels.ctypes.data, cap_blocks,
                                        plan.ctypes.data, cap_plan, ctypes.byref(nplan), ctypes.byref(ninj)),
           "spade_ref_amr_exchange")
    n = nblk.value
    shape = (n, nc[2] + 2 * ng, nc[1] + 2 * ng, nc[0] + 2 * ng, 5)
    return {"before": before[:n * per_block].reshape(shape), "after": after[:n * per_block].reshape(shape),
            "boxes": boxes[:6 * n].reshape(n, 6), "levels": levels[:n].copy(),
            "plan": plan[:18 * nplan.value].reshape(-1, 18).copy(), "ninject": ninj.value}


def ref_amr_flux_div(ref_scheme, nb, nc, ng, periodic, passes, scheme, prims, bounds=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)):
    """The reference's flux_div (overwrite mode) on the refined layout of
    ref_amr_exchange(nb, nc, ng, periodic, passes, bounds), with the state
    `prims` (its full array, ghosts included) copied in
    (oracle/ref_harness.cc spade_ref_amr_flux_div).  The scheme constants
    come from `scheme` as for ref_flux_div.  Returns the residual array."""
    ints = [nb[0], nb[1], nb[2], nc[0], nc[1], nc[2], ng] + [int(bool(p)) for p in periodic] + [len(passes)]
    for ps in passes:
        ints += [len(ps)] + list(ps)
    ints = np.array(ints, dtype=np.int32)
    grid = _abi.grid_desc(nb, nc, ng, bounds)
    _, reals = _ref_problem(grid, scheme)
    q = np.ascontiguousarray(prims, dtype=np.float64)
    rhs = np.zeros_like(q)
    nblk = ctypes.c_int(0)
    _check(ref().spade_ref_amr_flux_div(int(ref_scheme), ints.ctypes.data, reals.ctypes.data, q.size, _ptr(q), _ptr(rhs),
                                        ctypes.byref(nblk)), "spade_ref_amr_flux_div")
    assert nblk.value == q.shape[0]
    return rhs


def _amr_ints(nb, nc, ng, periodic, passes):
    ints = [nb[0], nb[1], nb[2], nc[0], nc[1], nc[2], ng] + [int(bool(p)) for p in periodic] + [len(passes)]
    for ps in passes:
        ints += [len(ps)] + list(ps)
    return np.array(ints, dtype=np.int32)


def ref_amr_ssprk3(ref_scheme, nb, nc, ng, periodic, passes, scheme, prims, dt, nsteps,
                   bounds=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), t_wall=None):
    """nsteps of the reference's SSPRK3 (integrator_t, ssprk3_t, state
    transform) on the refined layout of ref_amr_exchange, with the layout's
    exchange as the boundary condition (oracle/ref_harness.cc
    spade_ref_amr_ssprk3).  `prims` (full array) is updated in place.  With
    t_wall, the y faces are isothermal walls filled after each exchange."""
    ints = _amr_ints(nb, nc, ng, periodic, passes)
    grid = _abi.grid_desc(nb, nc, ng, bounds)
    _, reals = _ref_problem(grid, scheme)
    if t_wall is not None:
        reals[13] = float(t_wall)
    assert prims.dtype == np.float64 and prims.flags.c_contiguous
    _check(ref().spade_ref_amr_ssprk3(int(ref_scheme), ints.ctypes.data, reals.ctypes.data, float(dt), int(nsteps),
                                      prims.size, _ptr(prims), int(t_wall is not None)), "spade_ref_amr_ssprk3")



def ref_amr_fill(nb, nc, ng, periodic, passes, prims, t_wall=None, bounds=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0)):
    """The reference's boundary condition on a refined layout: its exchange,
    then with t_wall the isothermal-wall boundary_fill of the y faces
    (oracle/ref_harness.cc spade_ref_amr_fill); prims updated in place."""
    ints = _amr_ints(nb, nc, ng, periodic, passes)
    grid = _abi.grid_desc(nb, nc, ng, bounds)
    sch = _abi.SchemeDesc()
    sch.gas.gamma, sch.gas.R = 1.4, 287.0
    _, reals = _ref_problem(grid, sch)
    reals[13] = 0.0 if t_wall is None else float(t_wall)
    assert prims.dtype == np.float64 and prims.flags.c_contiguous
    _check(ref().spade_ref_amr_fill(ints.ctypes.data, reals.ctypes.data, int(t_wall is not None), prims.size, _ptr(prims)),
           "spade_ref_amr_fill")


def wall_fill_blocks(ncell, ng, boxes, bounds, bc, prims):
    """The wall faces of a refined layout, in place (numpy restatement of
    algs::boundary_fill, grid/boundary_fill.h:31-133, as it runs after the
    exchange): for each face f = 0..5 whose bc kind is a wall, every block
    whose box touches domain face f (boxes[:, f] == bounds[f]) has its ghost
    slab (ng layers, the full padded extent across) set from the mirrored
    cells of the same block: isothermal no-slip T -> 2 T_w - T with the
    velocity negated, slip the normal component negated."""
    boxes = np.asarray(boxes)
    for f in range(6):
        kind = bc.kind[f]
        if kind not in (_abi.BC_ISOTHERMAL_NOSLIP, _abi.BC_SLIP_ADIABATIC):
            continue
        d, hi = f // 2, f % 2
        ax = 3 - d                                     # array axis of direction d: (lb, k, j, i, v)
        for lb in np.nonzero(boxes[:, f] == bounds[f])[0]:
            blk = prims[lb]
            for layer in range(ng):
                c = ncell[d] + layer if hi else layer - ng
                img = 2 * ncell[d] - (c + 1) if hi else -1 - c
                src = np.take(blk, img + ng, axis=ax - 1).copy()
                if kind == _abi.BC_ISOTHERMAL_NOSLIP:
                    src[..., 1] = 2.0 * bc.t_wall[f] - src[..., 1]
                    src[..., 2:] = -src[..., 2:]
                else:
                    src[..., 2 + d] = -src[..., 2 + d]
                idx = [slice(None)] * 4
                idx[ax - 1] = c + ng
                blk[tuple(idx)] = src
