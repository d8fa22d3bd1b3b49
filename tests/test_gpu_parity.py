"""GPU parity: the CUDA path through the C ABI of libgbns.so against the
reference's outputs (tests/golden/) and the CPU oracle on identical inputs.

GBNS_PREC_FP64 (the drop-in) performs every FP64 operation in the
reference's order without FMA contraction, so its results must equal the
reference's BIT FOR BIT (pinned schemes) and the oracle's bit for bit
(features the reference lacks).  GBNS_PREC_FP64_FMA contracts multiply-adds:
tolerance 1e-12 normwise per variable (max|gpu-ref| <= 1e-12 max|ref|).
FP32-flux: 2e-4 normwise.  Ghost fills are copies: bit for bit.
"""
import ctypes
import math
import os

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spade_gb300 import _abi, _native
from oracle import oracle as O
import problems as P
from golden.gen_golden import FLUX_CASES, FLUX_GRID, GHOST_GRID

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
TOL64 = 1e-12


def load(name):
    return np.load(os.path.join(GOLD, name))


def interior(a, ng):
    return a[:, ng:-ng, ng:-ng, ng:-ng, :]


def dev(a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy()


def lib():
    return _native.lib()


def stream():
    return int(torch.cuda.current_stream().cuda_stream)


def gpu_flux(grid, scheme, q, rhs0=None, increment=False, variant=0):
    qd = dev(q)
    rd = dev(rhs0 if rhs0 is not None else np.zeros_like(q))
    if variant:
        rc = lib().gbns_flux_div_variant(grid, scheme, qd.data_ptr(), rd.data_ptr(), int(increment), variant, stream())
    else:
        rc = lib().gbns_flux_div(grid, scheme, qd.data_ptr(), rd.data_ptr(), int(increment), stream())
    _native.check(rc)
    return host(rd)


def gpu_fill(grid, bc, q):
    qd = dev(q)
    _native.check(lib().gbns_fill_ghosts(grid, bc, qd.data_ptr(), stream()))
    return host(qd)


def gpu_status_ok():
    st = ctypes.c_int(0)
    _native.check(lib().gbns_device_status(ctypes.byref(st), 1, stream()))
    return st.value == 0


@pytest.fixture(autouse=True)
def _device_status_clean():
    yield
    assert gpu_status_ok(), "a kernel reported a device-side error"


# ---------------------------------------------------------------- flux_div

def normwise(a, b):
    a = np.asarray(a).reshape(-1, 5)
    b = np.asarray(b).reshape(-1, 5)
    return (np.abs(a - b).max(axis=0) / np.maximum(np.abs(b).max(axis=0), 1e-300)).max()


@pytest.mark.parametrize("name", sorted(FLUX_CASES))
def test_flux_div_fp64_bitwise_equals_reference(name):
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    r = gpu_flux(grid, P.scheme(**FLUX_CASES[name][1]), g["q"])
    assert np.array_equal(interior(r, fg["ng"]), g["rhs_" + name])


@pytest.mark.parametrize("name", sorted(FLUX_CASES))
def test_flux_div_fp64_fma_within_tolerance(name):
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    r = gpu_flux(grid, P.scheme(precision=_abi.PREC_FP64_FMA, **FLUX_CASES[name][1]), g["q"])
    assert normwise(interior(r, fg["ng"]), g["rhs_" + name]) <= TOL64


@pytest.mark.parametrize("name", ["ck2_visc", "fweno_diss_visc", "totani_visc"])
@pytest.mark.parametrize("increment", [False, True])
def test_flux_div_host_arrays_equal_reference(name, increment):
    """gbns_flux_div_host on numpy (host) arrays, staged through the GPU:
    the reference's own result bit for bit, and the ghost layers of rhs kept
    as they were."""
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    q = np.ascontiguousarray(g["q"])
    rhs = np.full_like(q, 0.0) if increment else np.full_like(q, 7.25)
    _native.check(lib().gbns_flux_div_host(grid, P.scheme(**FLUX_CASES[name][1]), q.ctypes.data, rhs.ctypes.data,
                                           int(increment), stream()))
    assert np.array_equal(interior(rhs, fg["ng"]), g["rhs_" + name])
    if not increment:
        n = fg["ng"]
        mask = np.ones(rhs.shape[:-1], bool)
        mask[:, n:-n, n:-n, n:-n] = False
        assert np.all(rhs[mask] == 7.25)


def test_flux_div_python_api_on_cpu_arrays():
    """pde_algs.flux_div on grid_arrays held on the CPU (staged through the
    GPU by gbns_flux_div_host) equals the oracle bit for bit."""
    from spade_gb300 import grid as sg, pde_algs
    blocks = sg.cartesian_blocks_t((2, 1, 1), (0.0, 2.0, 0.0, 1.0, 0.0, 1.0))
    g = sg.cartesian_grid_t((8, 8, 8), blocks)
    ng = 3
    q = P.random_state((2, 1, 1), (8, 8, 8), ng, seed=57)
    qa = sg.grid_array(g, 0.0, ng, device="cpu", data=torch.from_numpy(q.copy()))
    ra = sg.grid_array(g, 0.0, ng, device="cpu")
    s = P.scheme(conv=_abi.CONV_WENO5, diss=1, visc=1)
    pde_algs.flux_div(qa, ra, s)
    ref = np.zeros_like(q)
    O.flux_div(qa.desc(), s, q, ref, increment=True)
    assert np.array_equal(interior(ra.data.numpy(), ng), interior(ref, ng))


def test_flux_div_overwrite_leaves_ghost_layers():
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    sentinel = np.full_like(g["q"], 7.25)
    r = gpu_flux(grid, P.scheme(conv=_abi.CONV_CENT_KEEP, order=2, visc=1), g["q"], rhs0=sentinel, increment=False)
    mask = np.ones(r.shape[:-1], bool)
    n = fg["ng"]
    mask[:, n:-n, n:-n, n:-n] = False
    assert np.all(r[mask] == 7.25)


def test_flux_div_increment_mode():
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    r = gpu_flux(grid, P.scheme(conv=_abi.CONV_CENT_KEEP, order=2, visc=1), g["q"], rhs0=g["rhs0_increment"], increment=True)
    assert np.array_equal(interior(r, fg["ng"]), g["rhs_increment_ck2_visc"])


@pytest.mark.parametrize("name", ["ck2_visc", "totani_visc", "fweno_diss_visc", "ck6"])
def test_flux_div_tma_and_plain_staging_identical(name, monkeypatch):
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    s = P.scheme(**FLUX_CASES[name][1])
    a = gpu_flux(grid, s, g["q"])
    monkeypatch.setenv("GBNS_NO_TMA", "1")
    b = gpu_flux(grid, s, g["q"])
    assert np.array_equal(a, b)


@pytest.mark.parametrize("conv,order", [(_abi.CONV_CENT_KEEP, 2), (_abi.CONV_TOTANI, 2), (_abi.CONV_FWENO, 2), (_abi.CONV_WENO5, 2)])
def test_flux_div_tile_variants_identical(conv, order):
    nblk, ncell, ng = (2, 2, 1), (20, 12, 10), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 2.0, 0.0, 1.0, 0.0, 1.5))
    q = P.random_state(nblk, ncell, ng, seed=31)
    s = P.scheme(conv=conv, order=order, diss=1, visc=1)
    base = gpu_flux(grid, s, q)
    nvar = lib().gbns_flux_variant_count(s)
    assert nvar >= 2
    for v in range(1, nvar):
        assert np.array_equal(gpu_flux(grid, s, q, variant=v), base), v


@pytest.mark.parametrize("coords", [_abi.COORDS_IDENTITY, _abi.COORDS_TANH_Y, _abi.COORDS_INTEGRATED_TANH_Y])
@pytest.mark.parametrize("case", ["weno5_diss_suth", "weno5_nosmooth", "fweno_power", "ck4_suth", "ck8"])
def test_flux_div_fp64_matches_oracle_unpinned_features(coords, case):
    """WENO5, Sutherland, power law with visc_lr and stretched-y metrics have
    no reference implementation: checked against the CPU restatement."""
    kw = {
        "weno5_diss_suth": dict(conv=_abi.CONV_WENO5, diss=1, visc=1, law=_abi.LAW_SUTHERLAND),
        "weno5_nosmooth": dict(conv=_abi.CONV_WENO5, smooth=0),
        "fweno_power": dict(conv=_abi.CONV_FWENO, visc=1, law=_abi.LAW_POWER),
        "ck4_suth": dict(conv=_abi.CONV_CENT_KEEP, order=4, visc=1, law=_abi.LAW_SUTHERLAND),
        "ck8": dict(conv=_abi.CONV_CENT_KEEP, order=8, visc=1),
    }[case]
    ng = 4 if case == "ck8" else 3
    nblk, ncell = (2, 3, 1), (9, 7, 5)
    cp = (2.0, 0, 0, 0) if coords == _abi.COORDS_TANH_Y else ((1.0, -1.0, 0.3, 2.5) if coords == _abi.COORDS_INTEGRATED_TANH_Y else (0, 0, 0, 0))
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 2.0, -1.0, 1.0, 0.0, 1.0), coords, cp)
    q = P.random_state(nblk, ncell, ng, seed=41)
    s = P.scheme(**kw)
    ref = np.zeros_like(q)
    O.flux_div(grid, s, q, ref, increment=False)
    r = gpu_flux(grid, s, q)
    if kw.get("law") == _abi.LAW_POWER:
        # pow() of the GPU math library and of the host libm may differ in the last bit
        assert normwise(interior(r, ng), interior(ref, ng)) <= 1e-14
    else:
        assert np.array_equal(interior(r, ng), interior(ref, ng))


@pytest.mark.parametrize("name", ["ck2_visc", "fweno_diss_visc", "totani_visc", "ducros_diss", "fweno_ducros_visc",
                                  "hyb_ck2_full", "hyb_ck4_diss_visc", "hyb_ck2_const_ducros_diss_visc"])
def test_flux_div_fp32_flux_error_bounded(name):
    """FP32 face arithmetic, FP64 accumulation: normwise error vs the FP64
    reference stays at single-precision level."""
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    s = P.scheme(precision=_abi.PREC_FP32_FLUX, **FLUX_CASES[name][1])
    r = interior(gpu_flux(grid, s, g["q"]), fg["ng"])
    ref = g["rhs_" + name]
    err = np.abs(r - ref).reshape(-1, 5).max(axis=0) / np.abs(ref).reshape(-1, 5).max(axis=0)
    assert np.all(err < 2e-4), err


def test_flux_div_conservation_periodic_tgv():
    """Telescoping: the sum of the residual over a periodic box is round-off."""
    nblk, ncell, ng = (2, 2, 2), (16, 16, 16), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    q = P.tgv_state(nblk, ncell, ng, P.tgv_tables(nblk, ncell, ng), seed=0)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    for prec in (_abi.PREC_FP64, _abi.PREC_FP32_FLUX):
        r = interior(gpu_flux(grid, P.tgv_scheme(precision=prec), q), ng).reshape(-1, 5)
        tot = np.abs(r.sum(axis=0))
        scale = np.abs(r).sum(axis=0)
        assert np.all(tot <= 1e-12 * scale), (prec, tot / scale)


# ------------------------------------------------------------- ghost fill

def test_fill_ghosts_matches_reference_bitwise():
    g = load("ghosts_ref.npz")
    gg = GHOST_GRID
    grid = _abi.grid_desc(gg["nblk"], gg["ncell"], gg["ng"], gg["bounds"])
    assert np.array_equal(gpu_fill(grid, P.periodic_bc(), g["q"]), g["periodic"])
    assert np.array_equal(gpu_fill(grid, P.channel_bc(290.0), g["q"]), g["walls"])


def test_fill_ghosts_slip_and_none_match_oracle():
    nblk, ncell, ng = (3, 2, 2), (5, 4, 3), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    q = P.random_state(nblk, ncell, ng, seed=51)
    bc = _abi.bc_desc([_abi.BC_SLIP_ADIABATIC, _abi.BC_ISOTHERMAL_NOSLIP, _abi.BC_PERIODIC, _abi.BC_PERIODIC,
                       _abi.BC_NONE, _abi.BC_SLIP_ADIABATIC], [0, 310.0, 0, 0, 0, 0])
    a = q.copy()
    O.fill_ghosts(grid, bc, a)
    assert np.array_equal(gpu_fill(grid, bc, q), a)


# -------------------------------------------------------------- RK stage

def test_rk_stage_matches_oracle():
    nblk, ncell, ng = (2, 1, 2), (6, 7, 5), 2
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    q = P.random_state(nblk, ncell, ng, seed=61)
    res = [P.random_state(nblk, ncell, ng, seed=62 + j, p0=1e3, T0=1e2, u0=10.0) for j in range(3)]
    coeffs = [-1.0 / 12.0 * 1e-4, -1.0 / 12.0 * 1e-4, 2.0 / 3.0 * 1e-4]
    a = q.copy()
    O.rk_stage(grid, P.gas_desc(), a, res, coeffs)
    qd = dev(q)
    rd = [dev(r) for r in res]
    ptrs = (ctypes.c_void_p * 3)(*[t.data_ptr() for t in rd])
    cf = (ctypes.c_double * 3)(*coeffs)
    _native.check(lib().gbns_rk_stage(grid, P.gas_desc(), qd.data_ptr(), ptrs, cf, 3, stream()))
    b = host(qd)
    assert np.array_equal(interior(b, ng), interior(a, ng))
    ghost = np.ones(q.shape[:-1], bool)
    ghost[:, ng:-ng, ng:-ng, ng:-ng] = False
    assert np.array_equal(b[ghost], q[ghost])


# ---------------------------------------------------------- time stepping

def gpu_ssprk3(grid, scheme, bc, q, dt, nsteps, ke_every=True):
    qd = dev(q)
    n = qd.numel()
    work = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    ke = []
    out = np.zeros(5)

    def red():
        _native.check(lib().gbns_reduce(grid, scheme.gas, qd.data_ptr(), _abi.RED_KINETIC,
                                        out.ctypes.data_as(ctypes.c_void_p), stream()))
        return float(out[0])

    ke.append(red())
    for _ in range(nsteps):
        _native.check(lib().gbns_ssprk3_step(grid, scheme, bc, qd.data_ptr(), work.data_ptr(), ctypes.c_double(dt), stream()))
        if ke_every:
            ke.append(red())
    return host(qd), np.array(ke)


def test_tgv_c1_flux_div_and_ke_history():
    """C1: 2x2x2 blocks of 16^3, ng=2, cent_keep<2> + visc_lr(constant):
    one flux_div and the 20-step SSPRK3 kinetic-energy history of the
    reference."""
    g = load("tgv_ref.npz")
    nblk, ncell, ng = (2, 2, 2), (16, 16, 16), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    tables = {k[4:]: g[k] for k in g.files if k.startswith("tab_")}
    q = P.tgv_state(nblk, ncell, ng, tables, seed=0)
    q = gpu_fill(grid, P.periodic_bc(), q)
    r = interior(gpu_flux(grid, P.tgv_scheme(), q), ng)
    assert np.array_equal(r[:, ::5, ::5, ::5, :], g["rhs_probe"])
    qf, ke = gpu_ssprk3(grid, P.tgv_scheme(), P.periodic_bc(), q, float(g["dt"]), 20)
    # the state is bit-identical; the KE reduction sums in another order
    np.testing.assert_allclose(ke, g["ke"], rtol=1e-13, atol=0)
    qi = interior(qf, ng)
    assert np.array_equal(qi[:, ::3, ::3, ::3, :], g["q_probe"])


def test_tgv_c1_fp64_fma_and_fp32_flux_ke_error():
    """The faster forms against the reference's 20-step KE history."""
    g = load("tgv_ref.npz")
    nblk, ncell, ng = (2, 2, 2), (16, 16, 16), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    tables = {k[4:]: g[k] for k in g.files if k.startswith("tab_")}
    q = gpu_fill(grid, P.periodic_bc(), P.tgv_state(nblk, ncell, ng, tables, seed=0))
    _, ke = gpu_ssprk3(grid, P.tgv_scheme(precision=_abi.PREC_FP64_FMA), P.periodic_bc(), q, float(g["dt"]), 20)
    np.testing.assert_allclose(ke, g["ke"], rtol=1e-12, atol=0)
    _, ke32 = gpu_ssprk3(grid, P.tgv_scheme(precision=_abi.PREC_FP32_FLUX), P.periodic_bc(), q, float(g["dt"]), 20)
    assert np.abs(ke32 / g["ke"] - 1.0).max() < 1e-5


def test_tgv_small_final_state():
    g = load("tgv_small_ref.npz")
    nblk, ncell, ng = (2, 2, 2), (8, 8, 8), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    tables = {k[4:]: g[k] for k in g.files if k.startswith("tab_")}
    q = P.tgv_state(nblk, ncell, ng, tables, seed=3)
    q = gpu_fill(grid, P.periodic_bc(), q)
    qf, ke = gpu_ssprk3(grid, P.tgv_scheme(), P.periodic_bc(), q, float(g["dt"]), 10)
    assert np.array_equal(interior(qf, ng), g["q_final"])
    np.testing.assert_allclose(ke, g["ke"], rtol=1e-13)


def test_channel_fweno_walls_5_steps():
    g = load("channel_ref.npz")
    nblk, ncell, ng = (2, 2, 2), (8, 8, 8), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 4 * math.pi, -1.0, 1.0, 0.0, 4 * math.pi / 3))
    s = P.scheme(conv=_abi.CONV_FWENO, diss=1, visc=1, mu=float(g["mu"]), eps_p=float(g["eps"]), eps_T=float(g["eps"]), alpha=1.0)
    qf, ke = gpu_ssprk3(grid, s, P.channel_bc(300.0), g["q0"], float(g["dt"]), 5)
    assert np.array_equal(interior(qf, ng), g["q_final"])
    np.testing.assert_allclose(ke, g["ke"], rtol=1e-13)


def test_stretched_channel_weno5_sutherland_matches_oracle_3_steps():
    nblk, ncell, ng = (2, 2, 1), (8, 8, 8), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 2.0, -1.0, 1.0, 0.0, 1.0), _abi.COORDS_TANH_Y, (2.0, 0, 0, 0))
    q = P.random_state(nblk, ncell, ng, seed=71, rel=0.01, u0=5.0)
    bc = P.channel_bc(300.0)
    O.fill_ghosts(grid, bc, q)
    s = P.scheme(conv=_abi.CONV_WENO5, diss=1, visc=1, law=_abi.LAW_SUTHERLAND, mu=0.05, eps_p=3.0, eps_T=3.0, alpha=1.0)
    dt = 2e-6
    a = q.copy()
    work = np.zeros((3,) + q.shape)
    for _ in range(3):
        O.ssprk3_step(grid, s, bc, a, work, dt)
    b, _ = gpu_ssprk3(grid, s, bc, q, dt, 3, ke_every=False)
    assert np.array_equal(interior(b, ng), interior(a, ng))


# ------------------------------------------------------------- reductions

@pytest.mark.parametrize("kind", [_abi.RED_MAX_WAVESPEED, _abi.RED_KINETIC, _abi.RED_CONSERVED, _abi.RED_HEALTH])
@pytest.mark.parametrize("coords", [_abi.COORDS_IDENTITY, _abi.COORDS_TANH_Y])
def test_reductions_match_oracle(kind, coords):
    nblk, ncell, ng = (3, 2, 2), (7, 6, 5), 2
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, -1.0, 1.0, 0.0, 2.0), coords, (2.0, 0, 0, 0))
    q = P.random_state(nblk, ncell, ng, seed=81)
    q[0, ng + 1, ng + 1, ng + 1, 0] = -1.0      # one non-physical cell
    q[1, ng + 2, ng, ng + 3, 4] = np.nan        # and one NaN
    if kind != _abi.RED_HEALTH:
        q = np.nan_to_num(np.abs(q))
    want = O.reduce(grid, P.gas_desc(), q, kind)
    qd = dev(q)
    out = np.zeros(5)
    _native.check(lib().gbns_reduce(grid, P.gas_desc(), qd.data_ptr(), kind, out.ctypes.data_as(ctypes.c_void_p), stream()))
    got = out if kind == _abi.RED_CONSERVED else out[0]
    if kind == _abi.RED_HEALTH:
        assert got == want == 2.0
    else:
        np.testing.assert_allclose(got, want, rtol=1e-13)


@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32_FLUX])
def test_flux_div_rk_equals_flux_div_then_rk_stage(precision):
    """The fused launch (residual + stage update) against the two separate
    launches: bit-identical in FP64; FP32-flux rounds the FP64 stage update
    with FMA contraction, so 1e-14 normwise there."""
    nblk, ncell, ng = (2, 2, 1), (12, 8, 8), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 2.0, -1.0, 1.0, 0.0, 1.0), _abi.COORDS_TANH_Y, (2.0, 0, 0, 0))
    q = P.random_state(nblk, ncell, ng, seed=101, rel=0.01, u0=5.0)
    s = P.scheme(conv=_abi.CONV_WENO5, diss=1, visc=1, law=_abi.LAW_SUTHERLAND, mu=0.05, eps_p=3.0, eps_T=3.0,
                 alpha=1.0, precision=precision)
    r0 = P.random_state(nblk, ncell, ng, seed=102, p0=1e3, T0=1e2, u0=10.0)
    r1 = P.random_state(nblk, ncell, ng, seed=103, p0=1e3, T0=1e2, u0=10.0)
    coeffs = [-1.0 / 12.0 * 1e-6, -1.0 / 12.0 * 1e-6, 2.0 / 3.0 * 1e-6]
    qd, r0d, r1d = dev(q), dev(r0), dev(r1)
    # separate launches
    r2d = torch.zeros_like(qd)
    _native.check(lib().gbns_flux_div(grid, s, qd.data_ptr(), r2d.data_ptr(), 0, stream()))
    qa = qd.clone()
    ptrs = (ctypes.c_void_p * 3)(r0d.data_ptr(), r1d.data_ptr(), r2d.data_ptr())
    cf = (ctypes.c_double * 3)(*coeffs)
    _native.check(lib().gbns_rk_stage(grid, s.gas, qa.data_ptr(), ptrs, cf, 3, stream()))
    # fused
    qb = torch.zeros_like(qd)
    earlier = (ctypes.c_void_p * 2)(r0d.data_ptr(), r1d.data_ptr())
    r2f = torch.zeros_like(qd)
    _native.check(lib().gbns_flux_div_rk(grid, s, qd.data_ptr(), r2f.data_ptr(), 1, 3, earlier, cf, qb.data_ptr(), stream()))
    a, b = interior(host(qa), ng), interior(host(qb), ng)
    assert np.array_equal(host(r2f), host(r2d))
    if precision == _abi.PREC_FP64:
        assert np.array_equal(a, b)
    else:
        assert normwise(b, a) <= 1e-14


@pytest.mark.gpu
def test_resume_from_checkpoint_is_bitwise_identical():
    """gbns_ssprk3_step: 3 steps, checkpoint (io.binary_write of the device
    array), restart from the file into a fresh device array, 4 more steps ==
    7 uninterrupted steps bit for bit, and both equal the oracle."""
    import tempfile
    import torch
    from spade_gb300 import io
    nblk, ncell, ng = (2, 1, 1), (8, 8, 8), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    tables = P.tgv_tables(nblk, ncell, ng)
    q = P.tgv_state(nblk, ncell, ng, tables, seed=4)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    dt = P.tgv_dt(q, grid, ng)
    s = P.tgv_scheme()
    bc = P.periodic_bc()
    L = lib()

    def steps(dq, n):
        work = torch.zeros(3 * dq.numel(), dtype=torch.float64, device="cuda")
        for _ in range(n):
            _native.check(L.gbns_ssprk3_step(grid, s, bc, ctypes.c_void_p(dq.data_ptr()), ctypes.c_void_p(work.data_ptr()),
                                             ctypes.c_double(dt), stream()))
        torch.cuda.synchronize()

    full = dev(q)
    steps(full, 7)
    part = dev(q)
    steps(part, 3)
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "restart.bin")
        io.binary_write(f, part)
        fresh = torch.full_like(part, float("nan"))
        io.binary_read(f, fresh)
    steps(fresh, 4)
    assert torch.equal(fresh, full)
    ref = q.copy()
    work = np.zeros((3,) + q.shape)
    for _ in range(7):
        O.ssprk3_step(grid, s, bc, ref, work, dt)
    assert np.array_equal(interior(host(full), ng), interior(ref, ng))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [_abi.SOURCE_CONST, _abi.SOURCE_BODY_FORCE, _abi.SOURCE_BODY_ACCEL])
def test_source_term_bitwise_equals_reference(kind):
    from golden.gen_golden import source_desc
    g = load("source_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    q = dev(P.random_state(fg["nblk"], fg["ncell"], fg["ng"], seed=11))
    r = dev(g["rhs0"])
    _native.check(lib().gbns_source_term(grid, source_desc(kind), ctypes.c_void_p(q.data_ptr()),
                                         ctypes.c_void_p(r.data_ptr()), stream()))
    assert np.array_equal(host(r), g["rhs_%d" % kind])     # ghosts untouched, interior bit-identical


@pytest.mark.gpu
def test_source_term_stretched_matches_oracle():
    from golden.gen_golden import source_desc
    grid = _abi.grid_desc((2, 3, 1), (8, 6, 4), 2, (0.0, 1.0, -1.0, 1.0, 0.0, 0.5), coords=_abi.COORDS_TANH_Y,
                          coord_param=(2.0, 0.0, 0.0, 0.0))
    q = P.random_state((2, 3, 1), (8, 6, 4), 2, seed=17)
    r0 = P.random_state((2, 3, 1), (8, 6, 4), 2, seed=18, p0=1.0, T0=1.0, u0=1.0)
    src = source_desc(_abi.SOURCE_BODY_ACCEL)
    want = r0.copy()
    O.source_term(grid, src, q, want)
    r = dev(r0)
    qd = dev(q)
    _native.check(lib().gbns_source_term(grid, src, ctypes.c_void_p(qd.data_ptr()), ctypes.c_void_p(r.data_ptr()), stream()))
    assert np.array_equal(host(r), want)


@pytest.mark.gpu
@pytest.mark.parametrize("conv", [_abi.CONV_FWENO, _abi.CONV_WENO5])
def test_fp32_flux_weno_weights_do_not_overflow(conv):
    """Energy fluxes of ~1e11 with order-one jumps between neighbours (p ~ 1e7,
    |u| ~ 3e3) push (beta + eps)^2 past the FP32 range; the FP32 weights are
    computed on scaled smoothness indicators, so the residual stays finite and
    close to FP64 (found as inf/NaN after 38 steps of the 16.8M-cell channel)."""
    nblk, ncell, ng = (2, 1, 1), (8, 8, 8), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    q = P.random_state(nblk, ncell, ng, seed=51, p0=1.0e7, T0=300.0, u0=3.0e3, rel=0.15)
    r64 = interior(gpu_flux(grid, P.scheme(conv=conv, diss=1, visc=1), q), ng)
    r32 = interior(gpu_flux(grid, P.scheme(conv=conv, diss=1, visc=1, precision=_abi.PREC_FP32_FLUX), q), ng)
    assert np.isfinite(r32).all()
    err = np.abs(r32 - r64).reshape(-1, 5).max(axis=0) / np.abs(r64).reshape(-1, 5).max(axis=0)
    assert np.all(err < 1e-3), err


@pytest.mark.gpu
def test_integer_pipe_multiply_matches_hardware():
    """The FP64 multiply, x/2, x/4, division and square root the flux kernels
    run on the integer pipes return the hardware operations' bits on 2^26 generated
    pairs (all bit patterns, exponent bands at the normal-range edges, exact
    products and ties, zeros, subnormals, infinities, NaNs)."""
    bad = ctypes.c_uint64(123)
    _native.check(lib().gbns_selftest_dmul_int(1 << 26, 7, ctypes.byref(bad), stream()))
    assert bad.value == 0


@pytest.mark.gpu
def test_bounded_wait_timeout_sets_status_and_context_survives():
    """Failure detection without a fault: a kernel waits for TMA bytes that
    never arrive, gives up after a bounded poll and flags the device status;
    the host reads the flag, and the context keeps working (a flux_div right
    after is still bit-identical to the reference)."""
    st = ctypes.c_int(-1)
    _native.check(lib().gbns_selftest_wait_timeout(ctypes.byref(st), stream()))
    assert st.value == _abi.DEV_TMA_TIMEOUT
    clean = ctypes.c_int(-1)
    _native.check(lib().gbns_device_status(ctypes.byref(clean), 0, stream()))
    assert clean.value == _abi.DEV_OK
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    r = gpu_flux(grid, P.scheme(**FLUX_CASES["ck2_visc"][1]), g["q"])
    assert np.array_equal(interior(r, fg["ng"]), g["rhs_ck2_visc"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32_FLUX])
def test_ssprk3_stepper_graph_replay_equals_direct_steps(precision):
    """time_integration.ssprk3_stepper(use_graph=True) captures one fused
    step (six launches) in a CUDA graph and replays it; five replays equal
    five direct gbns_ssprk3_step calls bit for bit."""
    from spade_gb300 import workloads
    from spade_gb300.time_integration import ssprk3_stepper
    prob = workloads.taylor_green(nblk=(2, 1, 1), ncell=(16, 16, 16), ng=2, seed=9, rng="torch")
    s = prob.scheme_desc(precision)
    bc = prob.bc_desc()
    q0 = prob.q.data.clone()
    st = ssprk3_stepper(prob.q, s, bc, prob.dt, use_graph=True)
    st.step(5)
    torch.cuda.synchronize()
    graphed = prob.q.data.clone()
    prob.q.data.copy_(q0)
    work = torch.zeros(3 * q0.numel(), dtype=torch.float64, device="cuda")
    for _ in range(5):
        _native.check(lib().gbns_ssprk3_step(prob.q.desc(), s, bc, ctypes.c_void_p(prob.q.ptr()),
                                             ctypes.c_void_p(work.data_ptr()), ctypes.c_double(prob.dt), stream()))
    torch.cuda.synchronize()
    assert torch.equal(prob.q.data, graphed)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", [_abi.RED_MAX_WAVESPEED, _abi.RED_KINETIC, _abi.RED_CONSERVED, _abi.RED_HEALTH])
def test_reduce_async_with_caller_scratch_equals_reduce(kind):
    """gbns_reduce_async (caller-owned device scratch, result left on the
    device) gives exactly gbns_reduce's values (same partition, same order)."""
    nblk, ncell, ng = (3, 2, 2), (7, 6, 5), 2
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, -1.0, 1.0, 0.0, 2.0))
    q = np.abs(P.random_state(nblk, ncell, ng, seed=82))
    qd = dev(q)
    want = np.zeros(5)
    _native.check(lib().gbns_reduce(grid, P.gas_desc(), qd.data_ptr(), kind, want.ctypes.data_as(ctypes.c_void_p), stream()))
    nd, off = ctypes.c_size_t(0), ctypes.c_size_t(0)
    _native.check(lib().gbns_reduce_scratch_size(grid, ctypes.byref(nd), ctypes.byref(off)))
    scratch = torch.zeros(nd.value, dtype=torch.float64, device="cuda")
    _native.check(lib().gbns_reduce_async(grid, P.gas_desc(), qd.data_ptr(), kind, scratch.data_ptr(), nd.value, stream()))
    got = scratch[off.value:off.value + 5].cpu().numpy()
    n = 5 if kind == _abi.RED_CONSERVED else 1
    assert np.array_equal(got[:n], want[:n])
    with pytest.raises(_native.SpadeError):
        _native.check(lib().gbns_reduce_async(grid, P.gas_desc(), qd.data_ptr(), kind, scratch.data_ptr(), 1, stream()))


@pytest.mark.gpu
def test_copy_fill_ghosts_equals_copy_then_fill():
    """gbns_copy_fill_ghosts(dst, src) == (dst = src interior; fill dst's ghosts)
    bit for bit, walls included; src is left untouched."""
    g = load("ghosts_ref.npz")
    gg = GHOST_GRID
    grid = _abi.grid_desc(gg["nblk"], gg["ncell"], gg["ng"], gg["bounds"])
    src = dev(g["q"])
    dst = torch.full_like(src, float("nan"))
    _native.check(lib().gbns_copy_fill_ghosts(grid, P.channel_bc(290.0), ctypes.c_void_p(dst.data_ptr()),
                                              ctypes.c_void_p(src.data_ptr()), stream()))
    assert np.array_equal(host(dst), g["walls"])
    assert np.array_equal(host(src), g["q"])


@pytest.mark.gpu
def test_ssprk3_run_graph_equals_steps():
    """gbns_ssprk3_run (one step captured as a CUDA graph inside the library,
    replayed nsteps times; a second call reuses the graph) equals the same
    number of gbns_ssprk3_step calls bit for bit, and matches the oracle."""
    nblk, ncell, ng = (2, 1, 1), (8, 8, 8), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    q = P.tgv_state(nblk, ncell, ng, P.tgv_tables(nblk, ncell, ng), seed=6)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    dt = P.tgv_dt(q, grid, ng)
    s, bc = P.tgv_scheme(), P.periodic_bc()
    a, b = dev(q), dev(q)
    wa = torch.zeros(3 * a.numel(), dtype=torch.float64, device="cuda")
    wb = torch.zeros_like(wa)
    for _ in range(6):
        _native.check(lib().gbns_ssprk3_step(grid, s, bc, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(wa.data_ptr()),
                                             ctypes.c_double(dt), stream()))
    for n in (2, 4):
        _native.check(lib().gbns_ssprk3_run(grid, s, bc, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(wb.data_ptr()),
                                            ctypes.c_double(dt), n, stream()))
    assert torch.equal(a, b)
    ref = q.copy()
    work = np.zeros((3,) + q.shape)
    for _ in range(6):
        O.ssprk3_step(grid, s, bc, ref, work, dt)
    assert np.array_equal(interior(host(b), ng), interior(ref, ng))


@pytest.mark.gpu
def test_ssprk3_run_graph_cache_eviction():
    """More distinct step configurations than the graph cache holds (eight):
    every call with a new time step captures a new graph and evicts the
    oldest; results still equal gbns_ssprk3_step with the same time steps."""
    nblk, ncell, ng = (1, 1, 1), (8, 8, 8), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    q = P.tgv_state(nblk, ncell, ng, P.tgv_tables(nblk, ncell, ng), seed=9)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    dt0 = P.tgv_dt(q, grid, ng)
    s, bc = P.tgv_scheme(), P.periodic_bc()
    a, b = dev(q), dev(q)
    wa = torch.zeros(3 * a.numel(), dtype=torch.float64, device="cuda")
    wb = torch.zeros_like(wa)
    dts = [dt0 * (0.5 + 0.05 * k) for k in range(10)] + [dt0 * 0.5, dt0 * 0.55]
    for dt in dts:
        _native.check(lib().gbns_ssprk3_step(grid, s, bc, ctypes.c_void_p(a.data_ptr()), ctypes.c_void_p(wa.data_ptr()),
                                             ctypes.c_double(dt), stream()))
        _native.check(lib().gbns_ssprk3_run(grid, s, bc, ctypes.c_void_p(b.data_ptr()), ctypes.c_void_p(wb.data_ptr()),
                                            ctypes.c_double(dt), 1, stream()))
    assert torch.equal(a, b)


# ------------------------------------------------------------ boundary_flux

@pytest.mark.parametrize("case", ["ck2_visc", "ck4", "totani_visc", "fweno_diss_visc", "weno5_diss_suth",
                                  "hyb_ck2_ducros_visc", "diss_ducros"])
@pytest.mark.parametrize("apply", [(1, 1, 1, 1, 1, 1), (0, 1, 1, 0, 0, 1)])
def test_boundary_flux_matches_restatement_bitwise(case, apply):
    """gbns_boundary_flux equals the oracle's restatement of
    pde_algs::boundary_flux bit for bit over the whole array (ghost cells
    included), accumulating into an existing rhs; block sizes that are not
    multiples of the 8x8 face patches."""
    kw = {
        "ck2_visc": dict(conv=_abi.CONV_CENT_KEEP, order=2, visc=1),
        "ck4": dict(conv=_abi.CONV_CENT_KEEP, order=4),
        "totani_visc": dict(conv=_abi.CONV_TOTANI, visc=1),
        "fweno_diss_visc": dict(conv=_abi.CONV_FWENO, diss=1, visc=1),
        "weno5_diss_suth": dict(conv=_abi.CONV_WENO5, diss=1, visc=1, law=_abi.LAW_SUTHERLAND),
        "hyb_ck2_ducros_visc": dict(conv=_abi.CONV_HYBRID, order=2, visc=1, hybrid_sensor=_abi.SENSOR_DUCROS,
                                    hybrid_param=1e-3),
        "diss_ducros": dict(conv=_abi.CONV_NONE, diss=1, sensor=_abi.SENSOR_DUCROS, alpha=1e-3),
    }[case]
    nblk, ncell, ng = (2, 2, 2), (9, 7, 10), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 2.0, 0.0, 1.0, 0.0, 1.5))
    q = P.random_state(nblk, ncell, ng, seed=53)
    r0 = P.random_state(nblk, ncell, ng, seed=54)
    s = P.scheme(**kw)
    ref = r0.copy()
    O.boundary_flux(grid, s, q, ref, apply)
    qd, rd = dev(q), dev(r0)
    flags = (ctypes.c_int * 6)(*apply)
    _native.check(lib().gbns_boundary_flux(grid, s, qd.data_ptr(), rd.data_ptr(), flags, stream()))
    assert np.array_equal(host(rd), ref)


def test_boundary_flux_python_api_and_errors():
    """pde_algs.boundary_flux on grid_arrays with a bound_box_t equals the
    restatement; stretched grids are rejected with GBNS_ERR_UNSUPPORTED and
    leave rhs untouched."""
    from spade_gb300 import grid as sg, pde_algs
    blocks = sg.cartesian_blocks_t((1, 2, 1), (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    g = sg.cartesian_grid_t((8, 8, 8), blocks)
    nblk, ncell, ng = (1, 2, 1), (8, 8, 8), 3
    q = P.random_state(nblk, ncell, ng, seed=55)
    qa = sg.grid_array(g, 0.0, ng, data=dev(q))
    ra = sg.grid_array(g, 0.0, ng)
    s = P.scheme(conv=_abi.CONV_WENO5, diss=1, visc=1)
    bb = pde_algs.bound_box_t(False)
    bb.max(1, True)
    pde_algs.boundary_flux(qa, ra, bb, s)
    ref = np.zeros_like(q)
    O.boundary_flux(qa.desc(), s, q, ref, bb.flags())
    assert np.array_equal(host(ra.data), ref)
    stretched = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, -1.0, 1.0, 0.0, 1.0), _abi.COORDS_TANH_Y, (2.0, 0, 0, 0))
    rd2 = dev(np.zeros_like(q))
    rc = lib().gbns_boundary_flux(stretched, s, qa.ptr(), rd2.data_ptr(), (ctypes.c_int * 6)(*bb.flags()), stream())
    assert rc == _abi.ERR_UNSUPPORTED
    assert not host(rd2).any()
