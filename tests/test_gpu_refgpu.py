"""The reference's own GPU flux_div (basic, bfoct and longf algorithms,
pde-algs/flux-div/flux_div.h:16-56), replayed on this GPU from the launch
scripts recorded where the reference's sources are (oracle/refgpu.py), on the
benchmark-size grids of the two schemes the reference can run: the
Taylor-Green scheme compose(cent_keep<2>, visc_lr) and the channel's
compose(fweno_t, pressure_diss_lr, visc_lr) on a uniform grid, 8x8x8 blocks
of 32^3 cells, 2 ghost layers.

The reference's kernels are compiled with nvcc's default FMA contraction,
so they round differently from its CPU code (which the FP64 drop-in matches
bit for bit): the comparison is to round-off, per conserved variable, and
the three algorithms must agree with each other the same way."""
import ctypes

import numpy as np
import pytest
import torch

from spade_gb300 import _abi, _native, workloads
from oracle import refgpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refgpu.available(),
                                 reason="reference GPU recordings absent (recorded where the reference sources are)")]


def _st():
    return int(torch.cuda.current_stream().cuda_stream)


def problem(case):
    if case == "tgv_ck2_visc":
        return workloads.taylor_green(nblk=(8, 8, 8), ncell=(32, 32, 32), ng=2, rng="torch", seed=0)
    return workloads.channel(nblk=(8, 8, 8), ncell=(32, 32, 32), ng=2, beta=None, weno="fweno", law="constant",
                             rng="torch", seed=0)


def _errors(got, want, ng):
    a = got[:, ng:-ng, ng:-ng, ng:-ng].reshape(-1, 5)
    b = want[:, ng:-ng, ng:-ng, ng:-ng].reshape(-1, 5)
    d = (a - b).abs()
    cell = (d.max(dim=0).values / b.abs().max(dim=0).values).cpu().numpy()
    norm = (d.norm(dim=0) / b.norm(dim=0)).cpu().numpy()
    return cell, norm


@pytest.mark.parametrize("case", refgpu.CASE_NAMES)
def test_reference_gpu_flux_div_agrees_with_gbns(case):
    prob = problem(case)
    ng = prob.ng
    s = prob.scheme_desc(_abi.PREC_FP64)
    ours = torch.zeros_like(prob.q.data)
    _native.check(_native.lib().gbns_flux_div(prob.q.desc(), s, prob.q.ptr(), ours.data_ptr(), 0, _st()))
    rhs = torch.zeros_like(prob.q.data)
    rep = refgpu.Replay(case, prob.q.data, rhs, _st())
    try:
        results = {}
        for alg in ("basic", "bfoct", "longf"):
            rhs.zero_()
            rep.run(alg, _st())
            torch.cuda.synchronize()
            results[alg] = rhs.clone()
    finally:
        rep.close()
    assert torch.isfinite(results["basic"]).all()
    for alg, r in results.items():
        cell, norm = _errors(r, ours, ng)
        print("%s %s vs gbns FP64: max cell error %s, normwise %s (of each variable's max)"
              % (case, alg, np.array2string(cell, precision=2), np.array2string(norm, precision=2)))
        assert np.all(cell < 1e-10), (alg, cell)
        assert np.all(norm < 1e-12), (alg, norm)
