"""flux_div on refined (AMR) block layouts, on the CPU.

Each block of a layout refined through cartesian_grid_t::refine_blocks takes
1/dx from its own bounding box (flux_div_basic.h:55, grid/grid_geometry.h:
85-89).  tests/golden/amr_flux_ref.npz holds the reference's own flux_div
(overwrite mode) on the exchanged arrays of tests/golden/amr_ref.npz for two
scheme compositions (tests/golden/gen_golden.py).  Here:

* the oracle's per-block-box flux_div reproduces it bit for bit;
* where the reference harness is built, a third composition too;
* three SSPRK3 steps composed from the oracle's exchange, flux_div and stage
  update reproduce the reference's integrator_t run with the exchange as
  boundary condition (the golden holds the SHA-256 of its final interior;
  live, where the harness is built, the whole array), also with y walls
  filled after each exchange (the reference's boundary_fill);
* gbns_flux_div_blocks rejects malformed layouts before any CUDA call.

The GPU side is tests/test_gpu_amr_flux.py."""
import ctypes
import hashlib
import os

import numpy as np
import pytest

from spade_gb300 import _abi, _native
from oracle import oracle as O
import problems as P
from test_amr_exchange import CASES, golden
from golden.gen_golden import AMR_CASES, AMR_FLUX_SCHEMES, AMR_SSPRK3_DT, AMR_SSPRK3_STEPS, AMR_T_WALL, amr_flux_input

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "amr_flux_ref.npz")


def layout(case):
    """(grid descriptor of the refined layout, boxes, the flux input state, ng)"""
    g = golden(case)
    ng = int(g["ng"])
    q = amr_flux_input(g["after"])
    grid = _abi.grid_desc((q.shape[0], 1, 1), tuple(int(n) for n in g["ncell"]), ng, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    return grid, g["boxes"], q, ng


@pytest.mark.parametrize("scheme", sorted(AMR_FLUX_SCHEMES))
@pytest.mark.parametrize("case", CASES)
def test_oracle_flux_div_blocks_equals_reference(case, scheme):
    grid, boxes, q, ng = layout(case)
    s = P.scheme(**AMR_FLUX_SCHEMES[scheme][1])
    r = np.zeros_like(q)
    O.flux_div_blocks(grid, s, boxes, q, r, increment=False)
    want = np.load(GOLD)[case + "_" + scheme]
    assert np.array_equal(r[:, ng:-ng, ng:-ng, ng:-ng], want)
    assert len(np.unique(boxes[:, 1] - boxes[:, 0])) >= 2          # blocks of more than one spacing


@pytest.mark.skipif(not O.ref_available(), reason="reference harness not built")
@pytest.mark.parametrize("case", ["two_levels_walls_y", "anisotropic_blocks"])
def test_oracle_flux_div_blocks_equals_reference_live(case):
    """A composition the goldens do not hold: hybrid cent_keep<2>/fweno_t
    with the Ducros blend."""
    nb, nc, ng, per, passes = AMR_CASES[case]
    grid, boxes, q, ng = layout(case)
    s = P.scheme(conv=_abi.CONV_HYBRID, order=2, hybrid_flux=_abi.HYBRID_FULL_FLUX,
                 hybrid_sensor=_abi.SENSOR_DUCROS, hybrid_param=0.5)
    want = O.ref_amr_flux_div(O.REF_HYB_CK2_FULL, nb, nc, ng, per, passes, s, q)
    r = np.zeros_like(q)
    O.flux_div_blocks(grid, s, boxes, q, r, increment=False)
    inner = (slice(None), slice(ng, -ng), slice(ng, -ng), slice(ng, -ng))
    assert np.all(np.isfinite(want[inner]))
    assert np.array_equal(r[inner], want[inner])


DOMAIN = (0.0, 1.0, 0.0, 1.0, 0.0, 1.0)


def oracle_amr_fill(case, q, bc=None):
    """The boundary condition of a refined layout: the exchange, then with bc
    the wall faces (oracle.wall_fill_blocks), in place."""
    g = golden(case)
    nc = tuple(int(n) for n in g["ncell"])
    ng = int(g["ng"])
    O.exchange_patches(nc, ng, q.shape[0], g["plan"], q)
    if bc is not None:
        O.wall_fill_blocks(nc, ng, g["boxes"], DOMAIN, bc, q)


def oracle_amr_ssprk3(case, s, q, dt, nsteps, bc=None):
    """nsteps of SSPRK3 on a refined layout from the oracle's pieces, after
    one exchange (as the reference's driver refreshes the ghosts first): per
    stage the residual (flux_div_blocks), the stage update (rk_stage, the
    ratio_diff coefficients of ssprk3_t) and the exchange, in place."""
    grid, boxes, _, ng = layout(case)
    oracle_amr_fill(case, q, bc)
    coeffs = ([dt], [(-3.0 / 4.0) * dt, (1.0 / 4.0) * dt], [(-1.0 / 12.0) * dt, (-1.0 / 12.0) * dt, (2.0 / 3.0) * dt])
    for _ in range(nsteps):
        R = [np.zeros_like(q) for _ in range(3)]
        for k, c in enumerate(coeffs):
            O.flux_div_blocks(grid, s, boxes, q, R[k], increment=True)
            O.rk_stage(grid, s.gas, q, R[:k + 1], c)
            oracle_amr_fill(case, q, bc)
    return q


def interior_digest(q, ng):
    return np.frombuffer(hashlib.sha256(np.ascontiguousarray(q[:, ng:-ng, ng:-ng, ng:-ng]).tobytes()).digest(),
                         dtype=np.uint8)


@pytest.mark.parametrize("scheme", sorted(AMR_FLUX_SCHEMES))
@pytest.mark.parametrize("case", CASES)
def test_oracle_amr_ssprk3_equals_reference(case, scheme):
    _, _, q, ng = layout(case)
    s = P.scheme(**AMR_FLUX_SCHEMES[scheme][1])
    a = oracle_amr_ssprk3(case, s, q.copy(), AMR_SSPRK3_DT, AMR_SSPRK3_STEPS)
    assert np.array_equal(interior_digest(a, ng), np.load(GOLD)[case + "_ssprk3_" + scheme])
    assert not np.array_equal(a, q)
    if O.ref_available():
        nb, nc, ng_, per, passes = AMR_CASES[case]
        want = q.copy()
        O.ref_amr_ssprk3(AMR_FLUX_SCHEMES[scheme][0], nb, nc, ng_, per, passes, s, want, AMR_SSPRK3_DT, AMR_SSPRK3_STEPS)
        assert np.array_equal(a, want)                    # ghost cells included


@pytest.mark.parametrize("scheme", sorted(AMR_FLUX_SCHEMES))
def test_oracle_amr_ssprk3_with_walls_equals_reference(scheme):
    """Two levels with y walls, the walls filled after each exchange (the
    reference's boundary_fill with the isothermal wall kernel)."""
    case = "two_levels_walls_y"
    _, _, q, ng = layout(case)
    s = P.scheme(**AMR_FLUX_SCHEMES[scheme][1])
    bc = P.channel_bc(AMR_T_WALL)
    a = oracle_amr_ssprk3(case, s, q.copy(), AMR_SSPRK3_DT, AMR_SSPRK3_STEPS, bc)
    assert np.array_equal(interior_digest(a, ng), np.load(GOLD)[case + "_ssprk3_walls_" + scheme])
    if O.ref_available():
        nb, nc, ng_, per, passes = AMR_CASES[case]
        want = q.copy()
        O.ref_amr_fill(nb, nc, ng_, per, passes, want, t_wall=AMR_T_WALL)
        got = q.copy()
        oracle_amr_fill(case, got, bc)
        assert np.array_equal(got, want)                  # the boundary condition alone, ghosts included
        want = q.copy()
        O.ref_amr_ssprk3(AMR_FLUX_SCHEMES[scheme][0], nb, nc, ng_, per, passes, s, want, AMR_SSPRK3_DT,
                         AMR_SSPRK3_STEPS, t_wall=AMR_T_WALL)
        assert np.array_equal(a, want)


def test_flux_div_blocks_rejects_bad_layouts_before_cuda():
    lib = _native.lib()
    s = P.scheme(conv=_abi.CONV_CENT_KEEP, visc=1)
    boxes = np.array([[0.0, 0.5, 0.0, 0.5, 0.0, 0.5], [0.5, 1.0, 0.0, 0.5, 0.0, 0.5]])
    pq, pr = ctypes.c_void_p(16), ctypes.c_void_p(32)

    def call(grid, b, scheme=s):
        bp = b.ctypes.data_as(ctypes.c_void_p) if b is not None else None
        return lib.gbns_flux_div_blocks(grid, scheme, bp, pq, pr, 0, None)

    g = _abi.grid_desc((2, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1))
    assert call(_abi.grid_desc((1, 2, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1)), boxes) == _abi.ERR_INVALID
    assert call(_abi.grid_desc((2, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1), _abi.COORDS_TANH_Y, (2.0, 0, 0, 0)),
                boxes) == _abi.ERR_UNSUPPORTED
    assert call(g, None) == _abi.ERR_INVALID
    bad = boxes.copy()
    bad[1, 3] = bad[1, 2]
    assert call(g, bad) == _abi.ERR_INVALID and "block 1" in _native.last_error()
    assert call(_abi.grid_desc((2, 1, 1), (4, 4, 4), 1, (0, 1, 0, 1, 0, 1)), boxes,
                P.scheme(conv=_abi.CONV_FWENO)) == _abi.ERR_INVALID
    assert "ghost layers" in _native.last_error()
    # the wall fill: no boundary descriptor; a wall across blocks thinner than the ghost depth
    assert lib.gbns_wall_fill_blocks(g, boxes.ctypes.data_as(ctypes.c_void_p), None, pq, None) == _abi.ERR_INVALID
    thin = _abi.grid_desc((2, 1, 1), (4, 1, 4), 2, (0, 1, 0, 1, 0, 1))
    assert lib.gbns_wall_fill_blocks(thin, boxes.ctypes.data_as(ctypes.c_void_p), P.channel_bc(300.0), pq,
                                     None) == _abi.ERR_UNSUPPORTED
    # the fused step: a missing exchange plan
    assert lib.gbns_ssprk3_step_blocks(g, s, boxes.ctypes.data_as(ctypes.c_void_p), None, None, pq, pr,
                                       ctypes.c_double(1e-4), None) == _abi.ERR_INVALID


def test_refined_layout_python_checks():
    """grid.refined_layout_t: descriptor and array shape of a layout; arrays of
    another shape are refused before any library call."""
    import torch
    from spade_gb300 import grid as G, pde_algs
    _, boxes, q, ng = layout("anisotropic_blocks")
    lay = G.refined_layout_t((8, 4, 4), ng, boxes)
    assert tuple(lay.desc().nblk) == (q.shape[0], 1, 1) and lay.shape() == q.shape
    bad = torch.zeros((q.shape[0] - 1,) + q.shape[1:], dtype=torch.float64)
    with pytest.raises(ValueError):
        pde_algs.flux_div_refined(lay, bad, bad.clone(), P.scheme())
    with pytest.raises(ValueError):
        G.refined_layout_t((8, 4, 4), ng, boxes[:, :4])
