"""Full-size checks (the 16.8M-cell channel: 8x8x8 blocks of 32^3, WENO5 +
pressure dissipation + Sutherland, tanh-stretched walls; a 2.1M-cell periodic
Taylor-Green box) through size-independent properties, where the oracle would
take minutes: every tile variant gives the same residual bit for bit, the
fused stage equals flux_div followed by the stage update, repeated runs are
identical, the FP32-flux residual stays within single-precision error of the
FP64 one, and the periodic residual telescopes to round-off."""
import ctypes

import numpy as np
import pytest
import torch

from spade_gb300 import _abi, _native, workloads

pytestmark = pytest.mark.gpu


def _lib():
    return _native.lib()


def _st():
    return int(torch.cuda.current_stream().cuda_stream)


@pytest.fixture(scope="module")
def channel():
    prob = workloads.channel(nblk=(8, 8, 8), ncell=(32, 32, 32), ng=3, rng="torch", seed=3)
    yield prob
    del prob
    torch.cuda.empty_cache()


def _flux(prob, s, out, variant=0):
    _native.check(_lib().gbns_flux_div_variant(prob.q.desc(), s, ctypes.c_void_p(prob.q.ptr()),
                                               ctypes.c_void_p(out.data_ptr()), 0, variant, _st()))


def test_channel_full_size_variants_identical_and_deterministic(channel):
    s = channel.scheme_desc(_abi.PREC_FP64)
    ref = torch.zeros_like(channel.q.data)
    _flux(channel, s, ref)
    again = torch.zeros_like(ref)
    _flux(channel, s, again)
    assert torch.equal(ref, again)
    for v in range(1, _lib().gbns_flux_variant_count(s)):
        r = torch.zeros_like(ref)
        _flux(channel, s, r, v)
        assert torch.equal(r, ref), v
    assert torch.isfinite(ref).all()


def test_channel_full_size_fused_stage_equals_separate(channel):
    prob = channel
    s = prob.scheme_desc(_abi.PREC_FP64)
    g = prob.q.desc()
    q = prob.q.data
    dt = prob.dt
    r = torch.zeros_like(q)
    _flux(prob, s, r)
    qa = q.clone()
    res = (ctypes.c_void_p * 1)(r.data_ptr())
    cf = (ctypes.c_double * 1)(dt)
    _native.check(_lib().gbns_rk_stage(g, s.gas, ctypes.c_void_p(qa.data_ptr()), res, cf, 1, _st()))
    qb = q.clone()
    rf = torch.zeros_like(q)
    _native.check(_lib().gbns_flux_div_rk(g, s, ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(rf.data_ptr()), 1, 1,
                                          None, cf, ctypes.c_void_p(qb.data_ptr()), _st()))
    ng = prob.ng
    inner = (slice(None), slice(ng, -ng), slice(ng, -ng), slice(ng, -ng))
    assert torch.equal(rf, r)
    assert torch.equal(qb[inner], qa[inner])


def test_channel_full_size_fp32_flux_residual_error(channel):
    r64 = torch.zeros_like(channel.q.data)
    _flux(channel, channel.scheme_desc(_abi.PREC_FP64), r64)
    r32 = torch.zeros_like(r64)
    _flux(channel, channel.scheme_desc(_abi.PREC_FP32_FLUX), r32)
    ng = channel.ng
    a = r64[:, ng:-ng, ng:-ng, ng:-ng].reshape(-1, 5)
    b = r32[:, ng:-ng, ng:-ng, ng:-ng].reshape(-1, 5)
    err = ((b - a).norm(dim=0) / a.norm(dim=0)).cpu().numpy()
    assert np.all(err < 1e-4), err


def test_periodic_tgv_2m_cells_residual_telescopes():
    prob = workloads.taylor_green(nblk=(4, 4, 4), ncell=(32, 32, 32), ng=2, rng="torch", seed=5)
    r = torch.zeros_like(prob.q.data)
    _flux(prob, prob.scheme_desc(_abi.PREC_FP64), r)
    ng = prob.ng
    inner = r[:, ng:-ng, ng:-ng, ng:-ng].reshape(-1, 5)
    total = inner.sum(dim=0)
    scale = inner.abs().sum(dim=0)
    assert torch.all(total.abs() <= 1e-11 * scale), (total, scale)


@pytest.mark.parametrize("nblk,ncell", [((64, 1, 1), (8, 8, 8)), ((1, 1, 1), (96, 96, 96)), ((3, 5, 7), (12, 10, 6))])
def test_extreme_block_shapes_variants_identical(nblk, ncell):
    """Many small blocks (64 along x, the descriptor maximum), one large block
    (96^3), and odd block counts with ragged tiles: every tile variant gives
    the same finite residual (bit for bit)."""
    ng = 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, -1.0, 1.0, 0.0, 1.0), _abi.COORDS_TANH_Y, (2.0, 0, 0, 0))
    import problems as P
    q = torch.from_numpy(P.random_state(nblk, ncell, ng, seed=61, rel=0.01, u0=5.0)).cuda()
    s = P.scheme(conv=_abi.CONV_WENO5, diss=1, visc=1, law=_abi.LAW_SUTHERLAND, mu=0.05, eps_p=3.0, eps_T=3.0, alpha=1.0)
    ref = None
    for v in range(_lib().gbns_flux_variant_count(s)):
        r = torch.zeros_like(q)
        _native.check(_lib().gbns_flux_div_variant(grid, s, ctypes.c_void_p(q.data_ptr()), ctypes.c_void_p(r.data_ptr()),
                                                   0, v, _st()))
        torch.cuda.synchronize()
        if ref is None:
            ref = r
            assert torch.isfinite(r).all()
        else:
            assert torch.equal(r, ref), v
