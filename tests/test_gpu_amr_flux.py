"""flux_div on refined (AMR) block layouts on the GPU (gbns_flux_div_blocks):
the reference's own results from tests/golden/amr_flux_ref.npz, bit for bit,
for three layouts refined through cartesian_grid_t::refine_blocks and two
scheme compositions, in every tile variant; increment mode against the
oracle; FP32-flux within its normwise bound; the whole refined-layout
path on the device (the reference's exchange plan run by
gbns_exchange_plan_*, then flux_div) against the reference; and three fused
SSPRK3 steps (gbns_ssprk3_step_blocks) against the reference's integrator
run (the SHA-256 of its final interior) and the oracle's steps (the whole
array, ghost cells included)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spade_gb300 import _abi, _native
from spade_gb300 import grid as _grid
from oracle import oracle as O
import problems as P
from test_amr_exchange import CASES, amr_fill, golden
from test_amr_flux import GOLD, DOMAIN, layout, oracle_amr_fill, oracle_amr_ssprk3, interior_digest
from golden.gen_golden import AMR_FLUX_SCHEMES, AMR_SSPRK3_DT, AMR_SSPRK3_STEPS, AMR_T_WALL

pytestmark = pytest.mark.gpu


def _st():
    return int(torch.cuda.current_stream().cuda_stream)


def _flux(grid, s, boxes, qd, rhs0, increment):
    rd = torch.from_numpy(rhs0.copy()).cuda()
    b = np.ascontiguousarray(boxes)
    _native.check(_native.lib().gbns_flux_div_blocks(grid, s, b.ctypes.data_as(ctypes.c_void_p), qd.data_ptr(),
                                                     rd.data_ptr(), int(increment), _st()))
    torch.cuda.synchronize()
    return rd.cpu().numpy()


@pytest.mark.parametrize("scheme", sorted(AMR_FLUX_SCHEMES))
@pytest.mark.parametrize("case", CASES)
def test_flux_div_blocks_equals_reference_every_variant(case, scheme):
    grid, boxes, q, ng = layout(case)
    want = np.load(GOLD)[case + "_" + scheme]
    qd = torch.from_numpy(q).cuda()
    s = P.scheme(**AMR_FLUX_SCHEMES[scheme][1])
    nvar = _native.lib().gbns_flux_variant_count(s)
    assert nvar >= 2
    for v in range(nvar):
        s.tile_variant = v
        r = _flux(grid, s, boxes, qd, np.zeros_like(q), False)
        assert np.array_equal(r[:, ng:-ng, ng:-ng, ng:-ng], want), v


@pytest.mark.parametrize("case", CASES)
def test_flux_div_blocks_increment_and_fp32_flux(case):
    grid, boxes, q, ng = layout(case)
    qd = torch.from_numpy(q).cuda()
    s = P.scheme(**AMR_FLUX_SCHEMES["fweno_diss_visc"][1])
    r0 = np.random.Generator(np.random.PCG64(5)).standard_normal(q.shape)
    want = r0.copy()
    O.flux_div_blocks(grid, s, boxes, q, want, increment=True)
    assert np.array_equal(_flux(grid, s, boxes, qd, r0, True), want)
    ref = np.load(GOLD)[case + "_fweno_diss_visc"]
    s32 = P.scheme(precision=_abi.PREC_FP32_FLUX, **AMR_FLUX_SCHEMES["fweno_diss_visc"][1])
    r = _flux(grid, s32, boxes, qd, np.zeros_like(q), False)[:, ng:-ng, ng:-ng, ng:-ng]
    err = (np.abs(r - ref).reshape(-1, 5).max(axis=0) / np.abs(ref).reshape(-1, 5).max(axis=0)).max()
    assert err < 2e-4, err


@pytest.mark.parametrize("case", CASES)
def test_refined_layout_exchange_then_flux_on_the_device(case):
    g = golden(case)
    grid, boxes, _, ng = layout(case)
    qd = torch.from_numpy(amr_fill(g["boxes"], g["ncell"], ng)).cuda()
    plan = _grid.exchange_plan_t(g["ncell"], ng, qd.shape[0], g["plan"])
    plan.exchange(qd)
    plan.close()
    hole = qd[..., 1] == 0.0                                  # wall ghosts the exchange leaves unset
    qd[hole] = torch.tensor([3.0, 1.0, 0.0, 0.0, 0.0], dtype=torch.float64, device="cuda")
    s = P.scheme(**AMR_FLUX_SCHEMES["ck2_visc"][1])
    r = _flux(grid, s, boxes, qd, np.zeros(tuple(qd.shape)), False)
    assert np.array_equal(r[:, ng:-ng, ng:-ng, ng:-ng], np.load(GOLD)[case + "_ck2_visc"])



@pytest.mark.parametrize("scheme", sorted(AMR_FLUX_SCHEMES))
@pytest.mark.parametrize("case", CASES)
def test_ssprk3_step_blocks_equals_reference(case, scheme):
    g = golden(case)
    grid, boxes, q, ng = layout(case)
    s = P.scheme(**AMR_FLUX_SCHEMES[scheme][1])
    qd = torch.from_numpy(q.copy()).cuda()
    work = torch.zeros(3 * q.size, dtype=torch.float64, device="cuda")
    plan = _grid.exchange_plan_t(g["ncell"], ng, q.shape[0], g["plan"])
    b = np.ascontiguousarray(boxes)
    plan.exchange(qd)                                          # the ghosts on entry, as the reference's driver
    for _ in range(AMR_SSPRK3_STEPS):
        _native.check(_native.lib().gbns_ssprk3_step_blocks(grid, s, b.ctypes.data_as(ctypes.c_void_p), plan.handle, None,
                                                            qd.data_ptr(), work.data_ptr(),
                                                            ctypes.c_double(AMR_SSPRK3_DT), _st()))
    torch.cuda.synchronize()
    plan.close()
    r = qd.cpu().numpy()
    assert np.array_equal(interior_digest(r, ng), np.load(GOLD)[case + "_ssprk3_" + scheme])
    assert np.array_equal(r, oracle_amr_ssprk3(case, s, q.copy(), AMR_SSPRK3_DT, AMR_SSPRK3_STEPS))


def test_python_api_on_refined_layouts():
    """The Python mirror: pde_algs.flux_div_refined on CUDA and CPU tensors
    (gbns_flux_div_blocks / _host) and time_integration.ssprk3_refined_stepper
    give the reference's results."""
    from spade_gb300 import pde_algs, time_integration
    case = "two_levels_walls_y"
    g = golden(case)
    _, boxes, q, ng = layout(case)
    lay = _grid.refined_layout_t(g["ncell"], ng, boxes)
    s = P.scheme(**AMR_FLUX_SCHEMES["ck2_visc"][1])
    want = np.load(GOLD)[case + "_ck2_visc"]
    for dev in ("cuda", "cpu"):
        qt = torch.from_numpy(q.copy()).to(dev)
        rt = torch.zeros_like(qt)
        pde_algs.flux_div_refined(lay, qt, rt, s, traits=(pde_algs.overwrite,))
        torch.cuda.synchronize()
        assert np.array_equal(rt.cpu().numpy()[:, ng:-ng, ng:-ng, ng:-ng], want), dev
    plan = _grid.exchange_plan_t(g["ncell"], ng, q.shape[0], g["plan"])
    qd = torch.from_numpy(q.copy()).cuda()
    plan.exchange(qd)
    st = time_integration.ssprk3_refined_stepper(lay, qd, s, plan, AMR_SSPRK3_DT)
    st.step(AMR_SSPRK3_STEPS)
    torch.cuda.synchronize()
    assert np.array_equal(interior_digest(qd.cpu().numpy(), ng), np.load(GOLD)[case + "_ssprk3_ck2_visc"])
    # with the y walls: the layout's wall fill, then the walled stepper
    bc = P.channel_bc(AMR_T_WALL)
    qd = torch.from_numpy(q.copy()).cuda()
    plan.exchange(qd)
    lay.fill_walls(qd, bc)
    st = time_integration.ssprk3_refined_stepper(lay, qd, s, plan, AMR_SSPRK3_DT, bc=bc)
    st.step(AMR_SSPRK3_STEPS)
    torch.cuda.synchronize()
    plan.close()
    assert np.array_equal(interior_digest(qd.cpu().numpy(), ng), np.load(GOLD)[case + "_ssprk3_walls_ck2_visc"])



@pytest.mark.parametrize("scheme", sorted(AMR_FLUX_SCHEMES))
def test_wall_fill_and_walled_steps_equal_reference(scheme):
    """Two levels with y walls: the exchange then gbns_wall_fill_blocks equals
    the oracle's boundary condition (ghosts included); three fused steps with
    the walls filled after each exchange give the reference's run."""
    case = "two_levels_walls_y"
    g = golden(case)
    grid, boxes, q, ng = layout(case)
    bc = P.channel_bc(AMR_T_WALL)
    b = np.ascontiguousarray(boxes)
    plan = _grid.exchange_plan_t(g["ncell"], ng, q.shape[0], g["plan"])
    qd = torch.from_numpy(q.copy()).cuda()
    plan.exchange(qd)
    _native.check(_native.lib().gbns_wall_fill_blocks(grid, b.ctypes.data_as(ctypes.c_void_p), bc, qd.data_ptr(), _st()))
    torch.cuda.synchronize()
    want = q.copy()
    oracle_amr_fill(case, want, bc)
    assert np.array_equal(qd.cpu().numpy(), want)
    s = P.scheme(**AMR_FLUX_SCHEMES[scheme][1])
    work = torch.zeros(3 * q.size, dtype=torch.float64, device="cuda")
    for _ in range(AMR_SSPRK3_STEPS):
        _native.check(_native.lib().gbns_ssprk3_step_blocks(grid, s, b.ctypes.data_as(ctypes.c_void_p), plan.handle, bc,
                                                            qd.data_ptr(), work.data_ptr(),
                                                            ctypes.c_double(AMR_SSPRK3_DT), _st()))
    torch.cuda.synchronize()
    plan.close()
    r = qd.cpu().numpy()
    assert np.array_equal(interior_digest(r, ng), np.load(GOLD)[case + "_ssprk3_walls_" + scheme])
    assert np.array_equal(r, oracle_amr_ssprk3(case, s, q.copy(), AMR_SSPRK3_DT, AMR_SSPRK3_STEPS, bc))
