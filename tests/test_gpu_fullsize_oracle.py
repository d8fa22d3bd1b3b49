"""The benchmarked channel at full size against the oracle.

The workload is exactly the bench's: 8x8x8 blocks of 32^3 cells (16.8 M
cells), 3 ghost layers, tanh-stretched y (beta = 2), 5th-order WENO +
pressure dissipation + visc_lr with Sutherland's law, isothermal no-slip walls
at y = +-1, periodic x and z, seeded state from the device generator (seed 0).

* one flux_div in FP64: bit-identical to oracle.flux_div over every interior
  cell (model: flux_div_basic.h:17-76);
* one SSPRK3 step in FP64: bit-identical to oracle.ssprk3_step
  (advance.h:234-280);
* the same step in FP32-flux: per-variable error against the FP64 oracle
  state, printed and bounded (max error below 1e-6 of each variable's field
  maximum);
* a 4x4x4-block channel of 32^3 cells advanced 10 steps: the state after every
  step bit-identical to the oracle's, so the whole time history agrees.

The oracle runs on all host cores (about a minute of CPU time in total)."""
import ctypes

import numpy as np
import pytest
import torch

from spade_gb300 import _abi, _native, workloads
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _st():
    return int(torch.cuda.current_stream().cuda_stream)


def _inner(a, ng):
    return a[:, ng:-ng, ng:-ng, ng:-ng]


@pytest.fixture(scope="module")
def bench_channel():
    prob = workloads.channel(nblk=(8, 8, 8), ncell=(32, 32, 32), ng=3, rng="torch", seed=0)
    q0 = prob.q.data.cpu().numpy().copy()
    yield prob, q0
    del prob
    torch.cuda.empty_cache()


def test_bench_channel_flux_div_fp64_bitwise_vs_oracle(bench_channel):
    prob, q0 = bench_channel
    g = prob.q.desc()
    s = prob.scheme_desc(_abi.PREC_FP64)
    rd = torch.zeros_like(prob.q.data)
    _native.check(_native.lib().gbns_flux_div(g, s, prob.q.ptr(), rd.data_ptr(), 0, _st()))
    torch.cuda.synchronize()
    got = _inner(rd.cpu().numpy(), prob.ng)
    del rd
    want = np.zeros_like(q0)
    O.flux_div(g, s, q0, want, increment=False)
    want = _inner(want, prob.ng)
    assert np.isfinite(want).all()
    diff = np.count_nonzero(got != want)
    assert diff == 0, "%d of %d residual entries differ" % (diff, got.size)


def _gpu_step(prob, q0, precision):
    g = prob.q.desc()
    s = prob.scheme_desc(precision)
    qd = torch.from_numpy(q0).cuda()
    work = torch.zeros(3 * qd.numel(), dtype=torch.float64, device="cuda")
    _native.check(_native.lib().gbns_ssprk3_step(g, s, prob.bc_desc(), qd.data_ptr(), work.data_ptr(),
                                                 ctypes.c_double(prob.dt), _st()))
    torch.cuda.synchronize()
    del work
    return qd.cpu().numpy()


def test_bench_channel_ssprk3_step_fp64_bitwise_and_fp32_flux_error_vs_oracle(bench_channel):
    prob, q0 = bench_channel
    g = prob.q.desc()
    s = prob.scheme_desc(_abi.PREC_FP64)
    ng = prob.ng
    want = q0.copy()
    work = np.zeros((3,) + q0.shape)
    O.ssprk3_step(g, s, prob.bc_desc(), want, work, prob.dt)
    del work
    want_in = _inner(want, ng)
    got64 = _inner(_gpu_step(prob, q0, _abi.PREC_FP64), ng)
    diff = np.count_nonzero(got64 != want_in)
    assert diff == 0, "%d of %d state entries differ" % (diff, got64.size)
    del got64
    # FP32-flux against the FP64 oracle state, per conserved-state primitive
    got32 = _inner(_gpu_step(prob, q0, _abi.PREC_FP32_FLUX), ng)
    names = ("p", "T", "u", "v", "w")
    for v in range(5):
        a, b = want_in[..., v], got32[..., v]
        err = np.abs(b - a)
        scale = np.abs(a).max()
        # v and w: perturbation fields of 5 % U_b, so scale by U_b instead
        if v >= 3:
            scale = prob.u0
        rel_max = err.max() / scale
        rel_l2 = np.sqrt(np.mean(err * err)) / scale
        print("FP32-flux one step, %s: max %.3e, rms %.3e (of %s)" % (names[v], rel_max, rel_l2,
                                                                      "U_b" if v >= 3 else "field max"))
        assert rel_max < 1e-6, (names[v], rel_max)


def test_channel_64_blocks_10_step_history_bitwise_vs_oracle():
    prob = workloads.channel(nblk=(4, 4, 4), ncell=(32, 32, 32), ng=3, rng="torch", seed=7)
    g = prob.q.desc()
    s = prob.scheme_desc(_abi.PREC_FP64)
    bc = prob.bc_desc()
    ng = prob.ng
    q = prob.q.data.cpu().numpy().copy()
    lib = _native.lib()
    qd = prob.q.data
    work_d = torch.zeros(3 * qd.numel(), dtype=torch.float64, device="cuda")
    work = np.zeros((3,) + q.shape)
    for step in range(10):
        O.ssprk3_step(g, s, bc, q, work, prob.dt)
        _native.check(lib.gbns_ssprk3_step(g, s, bc, qd.data_ptr(), work_d.data_ptr(), ctypes.c_double(prob.dt), _st()))
        got = _inner(qd.cpu().numpy(), ng)
        diff = np.count_nonzero(got != _inner(q, ng))
        assert diff == 0, "step %d: %d entries differ" % (step + 1, diff)
        ke_o = O.reduce(g, s.gas, q, _abi.RED_KINETIC)
        out = np.zeros(5)
        _native.check(lib.gbns_reduce(g, s.gas, qd.data_ptr(), _abi.RED_KINETIC, out.ctypes.data_as(ctypes.c_void_p), _st()))
        # identical states; the two reductions sum 2.1M cells in different
        # orders (device tree vs host loop), so agreement to summation error
        np.testing.assert_allclose(out[0], ke_o, rtol=1e-11)
