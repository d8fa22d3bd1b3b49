"""Serving form: continuous batching of independent solves.

Requests (a grid, a scheme, a step count) arrive over time.  The server keeps
one resident batch (spade_gb300.batch.batch_t, one flux launch per
kernel class per RK stage, replayed from a CUDA graph).  Between chunks of
steps it admits every request that has arrived and fits the HBM budget
(first come, first served), advances all active instances together, and
retires the ones that reached their step count.  A request that went
non-physical (NaN/Inf or p, T <= 0, gbns_reduce GBNS_RED_HEALTH) is evicted
as failed without disturbing the others: every instance's arithmetic is
independent of the mix, so each result equals running it alone.
"""
import collections
import ctypes
import math
import time

import numpy as np
import torch

from . import _abi, _native, workloads
from .batch import batch_t


class request_t:
    def __init__(self, rid, kind, edge, block, reynolds, mach, steps, arrival, corrupt=False):
        self.id = rid
        self.kind = kind            # "tgv" or "channel"
        self.edge = edge            # cells per direction
        self.block = block          # cells per block per direction
        self.reynolds = reynolds
        self.mach = mach
        self.steps = steps
        self.arrival = arrival      # seconds after the start of the run
        self.corrupt = corrupt      # fault injection: a NaN planted in the initial state
        self.slot = None
        self.admitted = None
        self.done = None
        self.status = "queued"
        self.cells = edge ** 3
        self.remaining = steps
        self.grid = None
        self.scheme = None
        self.bc = None
        self.dt = None

    def latency(self):
        return None if self.done is None else self.done - self.arrival


def poisson_requests(n, rate=40.0, seed=0, tgv_frac=0.7, edges=(16, 32, 64, 128), steps=(100, 2000),
                     reynolds=(100.0, 3000.0), mach=(0.05, 0.4)):
    """Seeded synthetic request stream: Poisson arrivals at `rate` per second,
    70 % Taylor-Green / 30 % channel, cube edges drawn from `edges` (16^3
    blocks up to 32^3 cells, 32^3 blocks beyond), step counts uniform in
    `steps`, Re log-uniform and Mach uniform."""
    r = np.random.Generator(np.random.PCG64(seed))
    t = 0.0
    out = []
    for i in range(n):
        t += r.exponential(1.0 / rate)
        kind = "tgv" if r.random() < tgv_frac else "channel"
        edge = int(r.choice(edges))
        block = 16 if edge <= 32 else 32
        re = float(math.exp(r.uniform(math.log(reynolds[0]), math.log(reynolds[1]))))
        ma = float(r.uniform(mach[0], mach[1]))
        st = int(r.integers(steps[0], steps[1] + 1))
        out.append(request_t(i, kind, edge, block, re, ma, st, t))
    return out


def build_instance(req, precision, seed):
    """Initial state of a request on the GPU (a workloads.problem)."""
    nb = req.edge // req.block
    if req.kind == "tgv":
        prob = workloads.taylor_green(nblk=(nb, nb, nb), ncell=(req.block,) * 3, ng=2, mach=req.mach,
                                      reynolds=req.reynolds, seed=seed, rng="torch", p_factor=1.0 / 16.0)
    else:
        prob = workloads.channel(nblk=(nb, nb, nb), ncell=(req.block,) * 3, ng=3, mach_b=req.mach,
                                 re_b=req.reynolds, seed=seed, rng="torch")
    if req.corrupt:
        g = prob.ng
        prob.q.data[0, g + 1, g + 1, g + 1, 0] = float("nan")
    return prob


class server_t:
    """Continuous batching server.  Between chunks of steps (one chunk in
    flight on the GPU at a time) it retires the requests that reached their
    step counts, admits arrived requests whose arrays fit the HBM budget
    (first come, first served) and launches the next chunk.  While a chunk
    runs, the host builds the initial states of arrived requests on a side
    stream and polls the chunk's completion event instead of synchronising.
    Each instance carries a device-side step limit (gbns_batch_set_steps), so
    a request that finishes inside a chunk idles there at exactly its step
    count and chunks keep their length (`chunk_ms` of GPU time, adapted from
    the measured step time)."""

    def __init__(self, precision=_abi.PREC_FP32_FLUX, hbm_budget=150 << 30, chunk=16, use_graph=True,
                 health_every=4, chunk_ms=60.0, prepare_ahead=4):
        self.precision = precision
        self.batch = batch_t(hbm_budget, precision, use_graph)
        self.chunk = int(chunk)               # steps of the first chunk (the cap is 4x this)
        self.chunk_ms = float(chunk_ms)
        self.health_every = int(health_every)
        self.prepare_ahead = int(prepare_ahead)
        self.lib = _native.lib()
        self.stream = self.batch.stream
        self.st = int(self.stream.cuda_stream)
        self.side = torch.cuda.Stream()

    def _healthy(self, req):
        ptr, _ = self.batch.state_ptr(req.slot)
        out = ctypes.c_double(0.0)
        _native.check(self.lib.gbns_reduce(req.grid, req.scheme.gas, ctypes.c_void_p(ptr), _abi.RED_HEALTH,
                                           ctypes.byref(out), self.st))
        return out.value == 0.0

    def _prepare(self, req):
        """Builds the request's initial state on the side stream."""
        with torch.cuda.stream(self.side):
            prob = build_instance(req, self.precision, seed=req.id)
            ev = torch.cuda.Event()
            ev.record(self.side)
        req.grid = prob.q.desc()
        req.scheme = prob.scheme_desc(self.precision)
        req.bc = prob.bc_desc()
        req.dt = prob.dt
        return prob, ev

    def _admit(self, req, prob, ev, now):
        ev.synchronize()
        req.slot = self.batch.add(req.grid, req.scheme, req.bc, req.dt, prob.q.ptr(), shape=prob.q.shape)
        self.batch.set_steps(req.slot, req.steps)
        req.admitted = now
        req.status = "running"

    @staticmethod
    def _need(req):
        nb = req.edge // req.block
        return batch_t.instance_bytes(_abi.grid_desc((nb,) * 3, (req.block,) * 3, 3, (0, 1, 0, 1, 0, 1)))

    def run(self, requests, collect=None, time_limit=None):
        """Serves `requests` (sorted by arrival) to completion, or until
        `time_limit` seconds.  `collect`, if given, is called as
        collect(req, state_tensor) on every completed request before its slot
        is freed.  Returns statistics."""
        queue = collections.deque(sorted(requests, key=lambda r: r.arrival))
        prepared = collections.deque()
        active = {}
        done = []
        t0 = time.perf_counter()
        cell_steps = 0
        chunks = 0
        busy_ms = 0.0
        k = max(1, self.chunk)
        inflight = None          # (start event, end event, steps)
        stopping = False
        while queue or prepared or active or inflight is not None:
            now = time.perf_counter() - t0
            if time_limit is not None and now > time_limit:
                stopping = True
            # build the initial states of arrived requests while the GPU works
            while not stopping and queue and queue[0].arrival <= now and len(prepared) < self.prepare_ahead:
                r = queue.popleft()
                if self._need(r) > self.batch.usage()["bytes_budget"]:
                    r.status = "rejected"
                    r.done = now
                    done.append(r)
                    continue
                prob, ev = self._prepare(r)
                prepared.append((r, prob, ev))
            if inflight is not None:
                if not inflight[1].query():
                    time.sleep(0.0002)
                    continue
                # the chunk has finished: account it, retire, check health
                e0, e1, kk = inflight
                inflight = None
                ms = e0.elapsed_time(e1)
                busy_ms += ms
                chunks += 1
                now = time.perf_counter() - t0
                k = int(min(self.chunk * 4, max(1, round(self.chunk_ms * kk / max(ms, 1e-3)))))
                finished = []
                periodic = self.health_every and chunks % self.health_every == 0
                for slot, r in active.items():
                    left = self.batch.steps_left(slot)
                    if (left == 0 or periodic) and not self._healthy(r):
                        r.status = "failed"
                        finished.append(slot)
                    elif left == 0:
                        r.status = "ok"
                        finished.append(slot)
                for slot in finished:
                    r = active.pop(slot)
                    r.done = now
                    if collect is not None and r.status == "ok":
                        collect(r, self.batch.state(slot))
                    self.batch.remove(slot)
                    done.append(r)
            if stopping:
                break
            # admission between chunks: nothing of this batch is in flight
            while prepared:
                r, prob, ev = prepared[0]
                use = self.batch.usage()
                if use["bytes_used"] + self._need(r) > use["bytes_budget"]:
                    break
                prepared.popleft()
                try:
                    self._admit(r, prob, ev, time.perf_counter() - t0)
                except _native.SpadeError as e:
                    if e.code == _abi.ERR_CAPACITY:
                        prepared.appendleft((r, prob, ev))
                        break
                    r.status = "failed"
                    r.done = time.perf_counter() - t0
                    done.append(r)
                    continue
                active[r.slot] = r
                del prob
            if not active:
                if queue and not prepared:
                    wait = queue[0].arrival - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.01))
                continue
            # launch the next chunk; the cell-steps it does are known now
            for slot, r in active.items():
                left = self.batch.steps_left(slot)
                cell_steps += r.cells * (k if left < 0 else min(k, left))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            self.batch.step(k)
            e1.record(self.stream)
            inflight = (e0, e1, k)
        torch.cuda.synchronize()
        makespan = time.perf_counter() - t0
        lat = [r.latency() for r in done if r.status == "ok"]
        return {
            "offered": len(requests),
            "completed": sum(r.status == "ok" for r in done),
            "failed": sum(r.status == "failed" for r in done),
            "rejected": sum(r.status == "rejected" for r in done),
            "unfinished": len(queue) + len(prepared) + len(active),
            "p50_latency_s": float(np.percentile(lat, 50)) if lat else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if lat else None,
            "cell_steps": cell_steps,
            "makespan_s": makespan,
            "cell_steps_per_s": cell_steps / makespan if makespan > 0 else None,
            "gpu_busy_frac": busy_ms * 1e-3 / makespan if makespan > 0 else None,
            "chunks": chunks,
        }

    def close(self):
        self.batch.close()
