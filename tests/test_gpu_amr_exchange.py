"""AMR coarse/fine exchange on the GPU (gbns_exchange_plan_*): the
reference's own exchange plans from tests/golden/amr_ref.npz, run on the
device from the harness's field, give the reference's exchanged arrays bit
for bit (one level periodic, two levels with y walls, non-cubic blocks); a
second run changes nothing (ghosts are written from interior donors only)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spade_gb300 import grid as _grid
from test_amr_exchange import CASES, amr_fill, golden

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", CASES)
def test_gpu_exchange_plan_equals_reference(case):
    g = golden(case)
    ng = int(g["ng"])
    q = torch.from_numpy(amr_fill(g["boxes"], g["ncell"], ng)).cuda()
    plan = _grid.exchange_plan_t(g["ncell"], ng, q.shape[0], g["plan"])
    for _ in range(2):
        plan.exchange(q)
        torch.cuda.synchronize()
        assert np.array_equal(q.cpu().numpy(), g["after"])
    plan.close()
