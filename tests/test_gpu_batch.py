"""Batched form (gbns_batch_*): instances of uneven size advanced by
persistent launches.  Every instance's result is bit-identical alone in a
batch and in the mix, with or without the CUDA graph, while others are added
and removed.  Against the single-grid path (gbns_ssprk3_step): bit-identical
in FP64 (no FMA contraction anywhere); FP32-flux within 1e-6 normwise (the
FP32 face arithmetic is FMA-contracted, and the compiler may contract the
same source differently inside the persistent kernel)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spade_gb300 import _abi, _native
from spade_gb300.batch import batch_t
import problems as P

pytestmark = pytest.mark.gpu


def lib():
    return _native.lib()


def stream():
    return int(torch.cuda.current_stream().cuda_stream)


def tgv_instance(nblk, seed, precision=_abi.PREC_FP64, mach=0.1, re=1600.0):
    ncell, ng = (8, 8, 8), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    q = P.tgv_state(nblk, ncell, ng, P.tgv_tables(nblk, ncell, ng), seed=seed)
    s = P.tgv_scheme(precision=precision)
    s.mu = s.mu * (1600.0 / re)
    bc = P.periodic_bc()
    from oracle import oracle as O
    O.fill_ghosts(grid, bc, q)
    return grid, s, bc, q, P.tgv_dt(q, grid, ng)


def channel_instance(seed, precision=_abi.PREC_FP64):
    nblk, ncell, ng = (2, 2, 1), (8, 8, 8), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 2.0, -1.0, 1.0, 0.0, 1.0), _abi.COORDS_TANH_Y, (2.0, 0, 0, 0))
    q = P.random_state(nblk, ncell, ng, seed=seed, rel=0.01, u0=5.0)
    bc = P.channel_bc(300.0)
    from oracle import oracle as O
    O.fill_ghosts(grid, bc, q)
    s = P.scheme(conv=_abi.CONV_WENO5, diss=1, visc=1, law=_abi.LAW_SUTHERLAND, mu=0.05, eps_p=3.0, eps_T=3.0,
                 alpha=1.0, precision=precision)
    return grid, s, bc, q, 2e-6


def hybrid_instance(seed, precision=_abi.PREC_FP64):
    """Taylor-Green field under hybrid_scheme_t(cent_keep<2>, fweno_t,
    ducros_t, full_flux) + visc_lr."""
    grid, s, bc, q, dt = tgv_instance((2, 1, 1), seed, precision, mach=0.2)
    s.convective = _abi.CONV_HYBRID
    s.order = 2
    s.hybrid_flux = _abi.HYBRID_FULL_FLUX
    s.hybrid_sensor = _abi.SENSOR_DUCROS
    s.hybrid_param = 1e-3
    return grid, s, bc, q, dt


def alone(grid, s, bc, q, dt, nsteps):
    qd = torch.from_numpy(q).cuda()
    work = torch.zeros(3 * qd.numel(), dtype=torch.float64, device="cuda")
    for _ in range(nsteps):
        _native.check(lib().gbns_ssprk3_step(grid, s, bc, qd.data_ptr(), work.data_ptr(), ctypes.c_double(dt), stream()))
    torch.cuda.synchronize()
    return qd.cpu().numpy()


@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32_FLUX])
@pytest.mark.parametrize("use_graph", [True, False])
def test_batch_bitwise_equals_alone(precision, use_graph):
    insts = [tgv_instance((1, 1, 1), 1, precision), tgv_instance((2, 1, 1), 2, precision, mach=0.3, re=300.0),
             tgv_instance((2, 2, 2), 3, precision, re=3000.0), channel_instance(4, precision),
             tgv_instance((2, 2, 1), 5, precision), hybrid_instance(6, precision)]
    b = batch_t(512 << 20, precision, use_graph)
    slots = []
    keep = []
    for grid, s, bc, q, dt in insts:
        qd = torch.from_numpy(q).cuda()
        keep.append(qd)
        slots.append(b.add(grid, s, bc, dt, qd.data_ptr()))
    b.step(3)
    torch.cuda.synchronize()
    for (grid, s, bc, q, dt), sl in zip(insts, slots):
        want = alone(grid, s, bc, q, dt, 3)
        got = b.state(sl).cpu().numpy()
        if precision == _abi.PREC_FP64:
            assert np.array_equal(got, want), sl
        else:
            # velocity components against the largest velocity (a component
            # that is ~0 everywhere, like w of Taylor-Green, has no scale of its own)
            w = np.abs(want).reshape(-1, 5).max(axis=0)
            scale = np.array([w[0], w[1], w[2:].max(), w[2:].max(), w[2:].max()])
            err = np.abs(got - want).reshape(-1, 5).max(axis=0) / scale
            assert np.all(err < 1e-6), (sl, err)
        assert b.steps_done(sl) == 3
    b.close()


def alone_in_batch(inst, precision, nsteps):
    grid, s, bc, q, dt = inst
    b = batch_t(256 << 20, precision, True)
    qd = torch.from_numpy(q).cuda()
    sl = b.add(grid, s, bc, dt, qd.data_ptr())
    b.step(nsteps)
    torch.cuda.synchronize()
    out = b.state(sl).cpu().numpy()
    b.close()
    return out


@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32_FLUX])
def test_batch_alone_and_in_the_mix_bitwise(precision):
    insts = [tgv_instance((2, 1, 1), 41, precision, mach=0.2), channel_instance(42, precision),
             tgv_instance((2, 2, 2), 43, precision, re=150.0), channel_instance(44, precision)]
    b = batch_t(512 << 20, precision, True)
    keep = []
    slots = []
    for grid, s, bc, q, dt in insts:
        qd = torch.from_numpy(q).cuda()
        keep.append(qd)
        slots.append(b.add(grid, s, bc, dt, qd.data_ptr()))
    b.step(4)
    torch.cuda.synchronize()
    for inst, sl in zip(insts, slots):
        assert np.array_equal(b.state(sl).cpu().numpy(), alone_in_batch(inst, precision, 4)), sl
    b.close()


def test_batch_add_remove_between_steps_does_not_disturb_others():
    a = tgv_instance((2, 2, 1), 11)
    c = channel_instance(12)
    d = tgv_instance((1, 1, 1), 13, re=200.0)
    b = batch_t(512 << 20, _abi.PREC_FP64, True)
    qa = torch.from_numpy(a[3]).cuda()
    sa = b.add(*a[:3], a[4], qa.data_ptr())
    b.step(2)
    qc = torch.from_numpy(c[3]).cuda()
    sc = b.add(*c[:3], c[4], qc.data_ptr())          # joins mid-run
    b.step(2)
    qd = torch.from_numpy(d[3]).cuda()
    sd = b.add(*d[:3], d[4], qd.data_ptr())
    b.remove(sc)                                      # leaves mid-run
    b.step(1)
    torch.cuda.synchronize()
    assert np.array_equal(b.state(sa).cpu().numpy(), alone(*a[:3], a[3], a[4], 5))
    assert np.array_equal(b.state(sd).cpu().numpy(), alone(*d[:3], d[3], d[4], 1))
    b.close()


def test_batch_budget_admission():
    grid, s, bc, q, dt = tgv_instance((2, 2, 2), 21)
    need = batch_t.instance_bytes(grid)
    assert need > 0
    b = batch_t(2 * need + need // 2, _abi.PREC_FP64, True)
    qd = torch.from_numpy(q).cuda()
    s1 = b.add(grid, s, bc, dt, qd.data_ptr())
    b.add(grid, s, bc, dt, qd.data_ptr())
    with pytest.raises(_native.SpadeError) as e:
        b.add(grid, s, bc, dt, qd.data_ptr())
    assert e.value.code == _abi.ERR_CAPACITY
    b.remove(s1)
    b.add(grid, s, bc, dt, qd.data_ptr())             # room again after eviction
    assert b.usage()["active"] == 2
    b.close()


def test_batch_rejects_mismatched_precision_and_unbatched_scheme():
    grid, s, bc, q, dt = tgv_instance((1, 1, 1), 31)
    b = batch_t(64 << 20, _abi.PREC_FP32_FLUX, True)
    qd = torch.from_numpy(q).cuda()
    with pytest.raises(_native.SpadeError):
        b.add(grid, s, bc, dt, qd.data_ptr())        # FP64 scheme into an FP32 batch
    s2 = P.scheme(conv=_abi.CONV_CENT_KEEP, order=4, visc=1, precision=_abi.PREC_FP32_FLUX)
    with pytest.raises(_native.SpadeError) as e:
        b.add(grid, s2, bc, dt, qd.data_ptr())
    assert e.value.code in (_abi.ERR_UNSUPPORTED, _abi.ERR_INVALID)
    b.close()


@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32_FLUX])
def test_batch_step_limits_inside_one_chunk_equal_alone(precision):
    """Instances with different step limits advanced by one chunk of 6
    steps: each stops at exactly its own count (counted on the device) and
    idles, and its state is bit-identical to advancing it alone that many
    steps; the host's count of steps done and left agrees."""
    insts = [tgv_instance((2, 1, 1), 71, precision, mach=0.2), channel_instance(72, precision),
             tgv_instance((1, 1, 1), 73, precision, re=400.0)]
    limits = [2, 5, -1]
    b = batch_t(512 << 20, precision, True)
    keep, slots = [], []
    for (grid, s, bc, q, dt), n in zip(insts, limits):
        qd = torch.from_numpy(q).cuda()
        keep.append(qd)
        sl = b.add(grid, s, bc, dt, qd.data_ptr())
        if n >= 0:
            b.set_steps(sl, n)
        slots.append(sl)
    b.step(6)
    torch.cuda.synchronize()
    for inst, sl, n in zip(insts, slots, limits):
        done = 6 if n < 0 else n
        assert b.steps_done(sl) == done
        assert b.steps_left(sl) == (-1 if n < 0 else 0)
        assert np.array_equal(b.state(sl).cpu().numpy(), alone_in_batch(inst, precision, done)), sl
    b.close()


def _close32(a, r):
    """FP32-flux states of two tile variants: the FP32 face arithmetic is
    FMA-contracted per kernel instantiation, so variants agree to single
    precision (velocities against the largest velocity)."""
    w = np.abs(r).reshape(-1, 5).max(axis=0)
    scale = np.array([w[0], w[1], w[2:].max(), w[2:].max(), w[2:].max()])
    err = np.abs(a - r).reshape(-1, 5).max(axis=0) / scale
    return np.all(err < 1e-6), err


@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32_FLUX])
def test_batch_tile_variants_identical_and_autotune(precision):
    """Every tile variant of every class gives the same states: bit for bit
    in FP64, to single-precision rounding in FP32-flux; the autotuner
    reports a valid variant for each class present."""
    insts = [tgv_instance((2, 1, 1), 81, precision), channel_instance(82, precision), hybrid_instance(83, precision)]
    ref = None
    ncls = int(lib().gbns_batch_class_count())
    for v in range(3):
        b = batch_t(512 << 20, precision, True)
        keep, slots = [], []
        for grid, s, bc, q, dt in insts:
            qd = torch.from_numpy(q).cuda()
            keep.append(qd)
            slots.append(b.add(grid, s, bc, dt, qd.data_ptr()))
        for c in range(ncls):
            try:
                b.set_variant(c, v)
            except _native.SpadeError:
                pass                                      # class with fewer variants
        b.step(2)
        torch.cuda.synchronize()
        states = [b.state(sl).cpu().numpy() for sl in slots]
        if ref is None:
            ref = states
            tuned = b.autotune(reps=1)
            assert set(tuned) == {"cent_keep2/identity", "weno5/stretched-y", "hybrid(cent_keep2,fweno)/identity"}
            assert all(t["variant"] >= 0 and t["tile"][0] == 8 for t in tuned.values())
        else:
            for a, r in zip(states, ref):
                if precision == _abi.PREC_FP64:
                    assert np.array_equal(a, r), v
                else:
                    ok, err = _close32(a, r)
                    assert ok, (v, err)
        b.close()
