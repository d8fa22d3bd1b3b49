"""GPU parity at the descriptor's limits.

* 64 blocks along x, the most the kernel-parameter geometry holds, with
  blocks of 4^3 cells (smaller than every tile, so each tile is ragged in all
  three directions), periodic;
* a stretched-y grid whose metric tables are full: 32 blocks along y of 31
  cells, blocks_y*(ny+1) = 1024 face entries, walls in y, the channel scheme
  (WENO5 + pressure_diss_lr + visc_lr with Sutherland).

On both: the ghost fill, one flux_div and three SSPRK3 steps of the FP64
drop-in equal the oracle bit for bit; the FP32-flux flux_div stays within
its normwise bound of the FP64 result.  The one-past-the-limit descriptors are
rejected on the host (tests/test_abi.py)."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spade_gb300 import _abi, _native
from oracle import oracle as O
import problems as P

pytestmark = pytest.mark.gpu

CASES = {
    # blocks, cells per block, ghosts, coordinates, scheme
    "64_blocks_x": ((64, 1, 1), (4, 4, 4), 2, _abi.COORDS_IDENTITY,
                    dict(conv=_abi.CONV_CENT_KEEP, visc=1)),
    "full_metric_table": ((1, 32, 1), (8, 31, 8), 3, _abi.COORDS_TANH_Y,
                          dict(conv=_abi.CONV_WENO5, diss=1, visc=1, law=_abi.LAW_SUTHERLAND,
                               mu=0.05, eps_p=3.0, eps_T=3.0, alpha=1.0)),
}


def _interior(a, ng):
    return a[:, ng:-ng, ng:-ng, ng:-ng, :]


def _normwise(a, b):
    a = np.asarray(a).reshape(-1, 5)
    b = np.asarray(b).reshape(-1, 5)
    return (np.abs(a - b).max(axis=0) / np.maximum(np.abs(b).max(axis=0), 1e-300)).max()


@pytest.mark.parametrize("case", sorted(CASES))
def test_fill_flux_div_and_steps_at_the_limits(case):
    nblk, ncell, ng, coords, kw = CASES[case]
    stretched = coords == _abi.COORDS_TANH_Y
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, -1.0, 1.0, 0.0, 1.0), coords,
                          (2.0, 0, 0, 0) if stretched else (0, 0, 0, 0))
    lib = _native.lib()
    st = int(torch.cuda.current_stream().cuda_stream)
    n = ctypes.c_size_t(0)
    _native.check(lib.gbns_array_size(grid, ctypes.byref(n)))
    bc = P.channel_bc(300.0) if stretched else P.periodic_bc()
    s = P.scheme(**kw)
    q = P.random_state(nblk, ncell, ng, seed=17, rel=0.01, u0=5.0)
    assert q.size == n.value

    want = q.copy()
    O.fill_ghosts(grid, bc, want)
    qd = torch.from_numpy(q.copy()).cuda()
    _native.check(lib.gbns_fill_ghosts(grid, bc, qd.data_ptr(), st))
    torch.cuda.synchronize()
    assert np.array_equal(qd.cpu().numpy(), want)
    q = want

    ref = np.zeros_like(q)
    O.flux_div(grid, s, q, ref, increment=False)
    rd = torch.zeros_like(qd)
    _native.check(lib.gbns_flux_div(grid, s, qd.data_ptr(), rd.data_ptr(), 0, st))
    torch.cuda.synchronize()
    r = rd.cpu().numpy()
    assert np.array_equal(_interior(r, ng), _interior(ref, ng))

    s32 = P.scheme(precision=_abi.PREC_FP32_FLUX, **kw)
    rd.zero_()
    _native.check(lib.gbns_flux_div(grid, s32, qd.data_ptr(), rd.data_ptr(), 0, st))
    torch.cuda.synchronize()
    err = _normwise(_interior(rd.cpu().numpy(), ng), _interior(ref, ng))
    assert err < 2e-4, err

    dt = 1e-7
    a = q.copy()
    work = np.zeros((3,) + q.shape)
    for _ in range(3):
        O.ssprk3_step(grid, s, bc, a, work, dt)
    wd = torch.zeros(3 * q.size, dtype=torch.float64, device="cuda")
    for _ in range(3):
        _native.check(lib.gbns_ssprk3_step(grid, s, bc, qd.data_ptr(), wd.data_ptr(), ctypes.c_double(dt), st))
    torch.cuda.synchronize()
    b = qd.cpu().numpy()
    assert np.all(np.isfinite(b))
    assert np.array_equal(_interior(b, ng), _interior(a, ng))
    st_ = ctypes.c_int(0)
    _native.check(lib.gbns_device_status(ctypes.byref(st_), 1, st))
    assert st_.value == 0
