"""gbns_reduce_noalloc: the reduction entry point that allocates nothing (its
partial sums live in a fixed device array inside the library).  It is for
callers that cannot let the library call cudaMalloc: applications whose
device memory all belongs to their own pool allocator, and solver loops that
must not stall on an allocation.

The GPU test calls it through the C ABI twice in a row for every reduction
kind and checks each result against gbns_reduce (library-allocated scratch)
on the same state.  The arithmetic and partition are gbns_reduce's, so the
results must be bit-identical.  One grid is small (3 partial records) and one
has 4x4x4 blocks of 32^3 cells, which uses the full 1024 partial records the
fixed array holds.  It must pass alone in a fresh process and after the
other tests.  The argument checks return before any CUDA call and run on the
CPU."""
import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spade_gb300 import _abi, _native
import problems as P

CASES = [
    # (blocks, cells per block, ghosts, coordinates, partial records used)
    ((3, 2, 2), (9, 7, 6), 2, _abi.COORDS_IDENTITY, 3),
    ((3, 2, 2), (9, 7, 6), 2, _abi.COORDS_TANH_Y, 3),
    ((4, 4, 4), (32, 32, 32), 3, _abi.COORDS_TANH_Y, 1024),
]


@pytest.mark.gpu
@pytest.mark.parametrize("nblk,ncell,ng,coords,npart", CASES)
def test_reduce_noalloc_matches_reduce_twice_in_a_row(nblk, ncell, ng, coords, npart):
    lib = _native.lib()
    st = int(torch.cuda.current_stream().cuda_stream)
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, -1.0, 1.0, 0.0, 2.0), coords, (2.0, 0, 0, 0))
    need, off = ctypes.c_size_t(0), ctypes.c_size_t(0)
    _native.check(lib.gbns_reduce_scratch_size(grid, ctypes.byref(need), ctypes.byref(off)))
    assert off.value == 6 * npart and need.value <= 6152
    gas = P.gas_desc()
    q = np.abs(P.random_state(nblk, ncell, ng, seed=91))
    q[0, ng + 2, ng + 1, ng + 3, 1] = -5.0          # one cell the health count must see
    qd = torch.from_numpy(q).cuda()
    out_dev = torch.full((5,), -1.0, dtype=torch.float64, device="cuda")
    for kind in (_abi.RED_MAX_WAVESPEED, _abi.RED_KINETIC, _abi.RED_CONSERVED, _abi.RED_HEALTH):
        want = np.zeros(5)
        _native.check(lib.gbns_reduce(grid, gas, qd.data_ptr(), kind, want.ctypes.data_as(ctypes.c_void_p), st))
        n = 5 if kind == _abi.RED_CONSERVED else 1
        for _ in range(2):
            out_dev.fill_(-1.0)
            _native.check(lib.gbns_reduce_noalloc(grid, gas, qd.data_ptr(), kind, out_dev.data_ptr(), st))
            torch.cuda.synchronize()
            got = out_dev.cpu().numpy()[:n]
            assert np.array_equal(got, want[:n]), (kind, got, want[:n])


def test_reduce_noalloc_rejects_bad_arguments():
    lib = _native.lib()
    grid = _abi.grid_desc((1, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1))
    rc = lib.gbns_reduce_noalloc(grid, P.gas_desc(), ctypes.c_void_p(16), 99, ctypes.c_void_p(32), None)
    assert rc == _abi.ERR_INVALID
    rc = lib.gbns_reduce_noalloc(grid, P.gas_desc(), ctypes.c_void_p(16), _abi.RED_KINETIC, None, None)
    assert rc == _abi.ERR_INVALID
    bad = _abi.grid_desc((1, 1, 1), (4, 4, 4), 2, (0, 1, 0, 1, 0, 1))
    bad.ncell[0] = 0
    rc = lib.gbns_reduce_noalloc(bad, P.gas_desc(), ctypes.c_void_p(16), _abi.RED_KINETIC, ctypes.c_void_p(32), None)
    assert rc == _abi.ERR_INVALID
