"""AMR coarse/fine exchange on the GPU (gbns_exchange_plan_*): the
reference's own exchange plans from tests/golden/amr_ref.npz, run on the
device from the harness's field, give the reference's exchanged arrays bit
for bit (one level periodic, two levels with y walls, non-cubic blocks).

With y walls some interpolation donors are ghost cells that other
interpolations write, so the result depends on the plan's order (the
reference executes it transaction by transaction) and a second exchange is
not a no-op: the second run is checked against the oracle's second run of
the same plan, bit for bit."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spade_gb300 import grid as _grid
from oracle import oracle as O
from test_amr_exchange import CASES, amr_fill, golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", CASES)
def test_gpu_exchange_plan_equals_reference(case):
    g = golden(case)
    ng = int(g["ng"])
    q0 = amr_fill(g["boxes"], g["ncell"], ng)
    q = torch.from_numpy(q0).cuda()
    plan = _grid.exchange_plan_t(g["ncell"], ng, q.shape[0], g["plan"])
    plan.exchange(q)
    torch.cuda.synchronize()
    assert np.array_equal(q.cpu().numpy(), g["after"])
    want = g["after"].copy()
    O.exchange_patches(g["ncell"], ng, q.shape[0], g["plan"], want)
    plan.exchange(q)
    torch.cuda.synchronize()
    assert np.array_equal(q.cpu().numpy(), want)
    plan.close()
