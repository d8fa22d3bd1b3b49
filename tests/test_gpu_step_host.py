"""gbns_ssprk3_step_host: one SSPRK3 step of a state held in page-locked host
memory, with the host/device copies split into block groups and overlapped
with stage 1 (copies in) and stage 3 (ghost fill and copies out).

The step is the same arithmetic as gbns_ssprk3_step on a device copy of the
state, issued group by group, so the new host state must be bit-identical to
copy in -> gbns_ssprk3_step -> copy out, for every group count: one group,
the library's default, uneven groups, one block per group, more groups than
blocks.  The channel (walls in y, periodic x and z: group ranges wrap around
z) and the all-periodic Taylor-Green vortex cover both kinds of ghost donor;
FP64 and FP32-flux both.  Argument checks return before any CUDA call and run
on the CPU."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spade_gb300 import _abi, _native, workloads
from spade_gb300.time_integration import ssprk3_stepper
import problems as P


def _st():
    return int(torch.cuda.current_stream().cuda_stream)


def _device_step(prob, s, q0, nsteps):
    qd = torch.from_numpy(q0).cuda()
    work = torch.zeros(3 * qd.numel(), dtype=torch.float64, device="cuda")
    for _ in range(nsteps):
        _native.check(_native.lib().gbns_ssprk3_step(prob.q.desc(), s, prob.bc_desc(), qd.data_ptr(),
                                                     work.data_ptr(), ctypes.c_double(prob.dt), _st()))
    torch.cuda.synchronize()
    return qd.cpu().numpy()


def _host_step(prob, s, q0, nsteps, ngroups, copy_stream=None):
    host = torch.empty(q0.shape, dtype=torch.float64, pin_memory=True)
    host.copy_(torch.from_numpy(q0))
    stepper = ssprk3_stepper(prob.q, s, prob.bc_desc(), prob.dt)
    prob.q.data.fill_(float("nan"))         # the device copy is overwritten by the call
    for _ in range(nsteps):
        stepper.step_host(host, ngroups=ngroups, copy_stream=copy_stream)
    torch.cuda.current_stream().synchronize()
    return host.numpy().copy()


CHANNEL = dict(nblk=(2, 3, 4), ncell=(8, 8, 8), ng=3)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32_FLUX])
@pytest.mark.parametrize("ngroups", [0, 1, 5, 24, 40])
def test_step_host_channel_bitwise(precision, ngroups):
    prob = workloads.channel(rng="torch", seed=3, **CHANNEL)
    q0 = prob.q.data.cpu().numpy().copy()
    s = prob.scheme_desc(precision)
    want = _device_step(prob, s, q0, 2)
    got = _host_step(prob, s, q0, 2, ngroups)
    assert np.isfinite(want).all()
    diff = np.count_nonzero(got != want)
    assert diff == 0, "%d of %d entries differ" % (diff, got.size)


@pytest.mark.gpu
@pytest.mark.parametrize("ngroups", [3, 7])
def test_step_host_taylor_green_periodic_bitwise_own_copy_stream(ngroups):
    prob = workloads.taylor_green(nblk=(3, 2, 2), ncell=(8, 8, 8), ng=2, rng="torch", seed=5)
    q0 = prob.q.data.cpu().numpy().copy()
    s = prob.scheme_desc(_abi.PREC_FP64)
    want = _device_step(prob, s, q0, 3)
    cs = torch.cuda.Stream()
    got = _host_step(prob, s, q0, 3, ngroups, copy_stream=cs)
    assert np.array_equal(got, want)


def test_step_host_rejects_bad_arguments():
    lib = _native.lib()
    grid = _abi.grid_desc((2, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1))
    s = P.scheme()
    bc = P.periodic_bc()
    vp = ctypes.c_void_p
    # NULL host array, NULL device array, NULL work
    assert lib.gbns_ssprk3_step_host(grid, s, bc, None, vp(64), vp(128), 1e-3, 0, None, None) == _abi.ERR_INVALID
    assert lib.gbns_ssprk3_step_host(grid, s, bc, vp(64), None, vp(128), 1e-3, 0, None, None) == _abi.ERR_INVALID
    assert lib.gbns_ssprk3_step_host(grid, s, bc, vp(64), vp(128), None, 1e-3, 0, None, None) == _abi.ERR_INVALID
    # host and device arrays the same, negative group count, copy stream = stream
    assert lib.gbns_ssprk3_step_host(grid, s, bc, vp(64), vp(64), vp(128), 1e-3, 0, None, None) == _abi.ERR_INVALID
    assert lib.gbns_ssprk3_step_host(grid, s, bc, vp(64), vp(96), vp(128), 1e-3, -1, None, None) == _abi.ERR_INVALID
    assert lib.gbns_ssprk3_step_host(grid, s, bc, vp(64), vp(96), vp(128), 1e-3, 0, vp(8), vp(8)) == _abi.ERR_INVALID
    bad = _abi.grid_desc((2, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1))
    bad.ncell[1] = 0
    assert lib.gbns_ssprk3_step_host(bad, s, bc, vp(64), vp(96), vp(128), 1e-3, 0, None, None) == _abi.ERR_INVALID
