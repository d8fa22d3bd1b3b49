"""Serving form: requests arriving over time are admitted as memory frees
up, batched together, retired at their own step counts; a request whose
state goes non-physical is evicted as failed; every completed result equals
the same solve run alone, bit for bit."""

import numpy as np
import pytest

torch = pytest.importorskip("torch")

from spade_gb300 import _abi, serve
from spade_gb300.batch import batch_t

pytestmark = pytest.mark.gpu


def run_alone(req, precision):
    """The same solve served alone: a batch holding only this request."""
    prob = serve.build_instance(req, precision, seed=req.id)
    q = prob.q
    b = batch_t(batch_t.instance_bytes(q.desc()) + (1 << 20), precision, True)
    sl = b.add(q.desc(), prob.scheme_desc(precision), prob.bc_desc(), prob.dt, q.ptr())
    b.step(req.steps)
    torch.cuda.synchronize()
    out = b.state(sl).cpu().numpy()
    b.close()
    return out


@pytest.mark.parametrize("precision", [_abi.PREC_FP64, _abi.PREC_FP32_FLUX])
def test_serving_results_equal_alone_and_failures_are_isolated(precision):
    reqs = [
        serve.request_t(0, "tgv", 32, 16, 800.0, 0.1, 7, 0.00),
        serve.request_t(1, "channel", 32, 16, 1500.0, 0.2, 5, 0.01),
        serve.request_t(2, "tgv", 16, 16, 200.0, 0.3, 11, 0.02, corrupt=True),
        serve.request_t(3, "tgv", 16, 16, 2500.0, 0.05, 3, 0.03),
        serve.request_t(4, "channel", 16, 16, 300.0, 0.15, 9, 0.04),
        serve.request_t(5, "tgv", 32, 16, 1000.0, 0.25, 6, 0.05),
    ]
    # budget for about two 32^3 instances at a time: later requests wait for memory
    one = batch_t.instance_bytes(_abi.grid_desc((2, 2, 2), (16, 16, 16), 3, (0, 1, 0, 1, 0, 1)))
    srv = serve.server_t(precision, hbm_budget=int(2.2 * one), chunk=4, health_every=1)
    results = {}
    stats = srv.run(reqs, collect=lambda r, t: results.__setitem__(r.id, t.cpu().numpy()))
    srv.close()
    assert stats["completed"] == 5 and stats["failed"] == 1 and stats["unfinished"] == 0
    assert reqs[2].status == "failed"
    assert stats["p50_latency_s"] is not None and stats["p99_latency_s"] >= stats["p50_latency_s"]
    for r in reqs:
        if r.status == "ok":
            assert np.array_equal(results[r.id], run_alone(r, precision)), r.id


def test_poisson_stream_is_seeded_and_shaped():
    a = serve.poisson_requests(200, seed=7)
    b = serve.poisson_requests(200, seed=7)
    assert [(r.kind, r.edge, r.steps) for r in a] == [(r.kind, r.edge, r.steps) for r in b]
    arr = np.array([r.arrival for r in a])
    assert np.all(np.diff(arr) > 0)
    assert 30.0 < len(a) / arr[-1] < 52.0                     # mean 40 req/s
    assert 0.6 < np.mean([r.kind == "tgv" for r in a]) < 0.8
    assert all(100 <= r.steps <= 2000 for r in a)
