"""The C++ drop-in executed for real, on a GPU.

tests/cpp/dropin_record.cc calls spade::pde_algs::flux_div with the gb300
traits at a SPADE call site on device::cpu grid_arrays, with no test hook:
the header lowers the scheme and grid and calls gbns_flux_div_host.  Built
against the reference's headers where they are (tests/golden/gen_golden.py),
it is linked with a recording stand-in for libgbns.so
(tests/cpp/gbns_record_stub.c), which stores each C-ABI call exactly as the
header made it, together with the reference's own CPU flux_div result on the
same arrays (tests/golden/dropin_ref.npz).  Here the recorded calls run
through the real library on the GPU:

* compose(cent_keep<2>, visc_lr) in increment mode and compose(fweno_t,
  pressure_diss_lr, visc_lr) in overwrite mode: bit-identical to the
  reference's result;
* the benchmarked channel scheme (gb300::weno5_t, pressure_diss_lr,
  visc_lr(gb300::sutherland_t)) on a gb300::tanh_stretch_1D grid, which the
  reference cannot run: bit-identical to the oracle;
* on a refined (amr_blocks_t) grid (tests/cpp/dropin_amr_record.cc,
  gbns_flux_div_blocks_host): bit-identical to the reference's result."""
import os

import numpy as np
import pytest

from spade_gb300 import _abi, _native
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dropin_ref.npz")


def _call(g, k):
    gb, sb = g["grid%d" % k].tobytes(), g["scheme%d" % k].tobytes()
    assert len(gb) == _abi.ctypes.sizeof(_abi.GridDesc) and len(sb) == _abi.ctypes.sizeof(_abi.SchemeDesc)
    grid = _abi.GridDesc.from_buffer_copy(gb)
    s = _abi.SchemeDesc.from_buffer_copy(sb)
    shape = (grid.nblk[0] * grid.nblk[1] * grid.nblk[2], grid.ncell[2] + 2 * grid.ng, grid.ncell[1] + 2 * grid.ng,
             grid.ncell[0] + 2 * grid.ng, 5)
    return grid, s, int(g["incr%d" % k]), g["q"].reshape(shape).copy(), g["rhs_in%d" % k].reshape(shape).copy()


@pytest.mark.parametrize("k", [0, 1])
def test_dropin_calls_on_the_gpu_equal_the_reference(k):
    g = np.load(GOLD)
    grid, s, incr, q, r = _call(g, k)
    _native.check(_native.lib().gbns_flux_div_host(grid, s, q.ctypes.data, r.ctypes.data, incr, None))
    assert np.array_equal(r.ravel(), g["ref"][k])


def test_dropin_channel_scheme_on_the_gpu_equals_the_oracle():
    g = np.load(GOLD)
    grid, s, incr, q, r = _call(g, 2)
    assert grid.coords == _abi.COORDS_TANH_Y and s.convective == _abi.CONV_WENO5 and s.visc_law == _abi.LAW_SUTHERLAND
    want = r.copy()
    O.flux_div(grid, s, q, want, increment=bool(incr))
    _native.check(_native.lib().gbns_flux_div_host(grid, s, q.ctypes.data, r.ctypes.data, incr, None))
    assert np.isfinite(r).all()
    assert np.array_equal(r, want)


@pytest.mark.parametrize("k", [0, 1])
def test_refined_dropin_calls_on_the_gpu_equal_the_reference(k):
    """The drop-in's calls on a refined grid (tests/cpp/dropin_amr_record.cc,
    gbns_flux_div_blocks_host with the grid's own block boxes) through the
    real library: the reference's CPU flux_div bit for bit."""
    from test_cpp_dropin import refined_dropin_call
    grid, s, boxes, q, r, incr, ng, want = refined_dropin_call(k)
    b = np.ascontiguousarray(boxes)
    _native.check(_native.lib().gbns_flux_div_blocks_host(grid, s, b.ctypes.data, q.ctypes.data, r.ctypes.data, incr, None))
    assert np.array_equal(r[:, ng:-ng, ng:-ng, ng:-ng], want)
