"""Serving form: continuous batching of independent solves.

Requests (a grid, a scheme, a step count) arrive over time.  The server keeps
one resident batch (spade_gb300.batch.batch_t, one persistent launch per
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
    def __init__(self, precision=_abi.PREC_FP32_FLUX, hbm_budget=150 << 30, chunk=16, use_graph=True,
                 health_every=4):
        self.precision = precision
        self.batch = batch_t(hbm_budget, precision, use_graph)
        self.chunk = int(chunk)
        self.health_every = int(health_every)
        self.lib = _native.lib()
        self.st = int(torch.cuda.current_stream().cuda_stream)

    def _healthy(self, req):
        ptr, _ = self.batch.state_ptr(req.slot)
        out = ctypes.c_double(0.0)
        _native.check(self.lib.gbns_reduce(req.grid, req.scheme.gas, ctypes.c_void_p(ptr), _abi.RED_HEALTH,
                                           ctypes.byref(out), self.st))
        return out.value == 0.0

    def _admit(self, req, now):
        prob = build_instance(req, self.precision, seed=req.id)
        req.grid = prob.q.desc()
        req.scheme = prob.scheme_desc(self.precision)
        req.bc = prob.bc_desc()
        req.dt = prob.dt
        req.slot = self.batch.add(req.grid, req.scheme, req.bc, req.dt, prob.q.ptr(), shape=prob.q.shape)
        req.admitted = now
        req.status = "running"
        torch.cuda.synchronize()
        del prob

    def run(self, requests, collect=None, time_limit=None):
        """Serves `requests` (sorted by arrival) to completion.  `collect`, if
        given, is called as collect(req, state_tensor) on every completed
        request before its slot is freed.  Returns statistics."""
        queue = collections.deque(sorted(requests, key=lambda r: r.arrival))
        active = {}
        done = []
        t0 = time.perf_counter()
        cell_steps = 0
        chunks = 0
        while queue or active:
            now = time.perf_counter() - t0
            if time_limit is not None and now > time_limit:
                break
            # admission: everything that has arrived and fits, first come first served
            while queue and queue[0].arrival <= now:
                need = batch_t.instance_bytes(_abi.grid_desc((queue[0].edge // queue[0].block,) * 3,
                                                             (queue[0].block,) * 3, 3, (0, 1, 0, 1, 0, 1)))
                use = self.batch.usage()
                if need > use["bytes_budget"]:
                    r = queue.popleft()
                    r.status = "rejected"
                    r.done = now
                    done.append(r)
                    continue
                if use["bytes_used"] + need > use["bytes_budget"]:
                    break
                r = queue.popleft()
                try:
                    self._admit(r, now)
                except _native.SpadeError as e:
                    if e.code == _abi.ERR_CAPACITY:
                        queue.appendleft(r)
                        break
                    r.status = "failed"
                    r.done = time.perf_counter() - t0
                    done.append(r)
                    continue
                active[r.slot] = r
            if not active:
                if queue:
                    wait = queue[0].arrival - (time.perf_counter() - t0)
                    if wait > 0:
                        time.sleep(min(wait, 0.05))
                continue
            k = min(self.chunk, min(r.remaining for r in active.values()))
            self.batch.step(k)
            torch.cuda.synchronize()
            chunks += 1
            now = time.perf_counter() - t0
            finished = []
            for slot, r in active.items():
                r.remaining -= k
                cell_steps += r.cells * k
                check = r.remaining == 0 or (self.health_every and chunks % self.health_every == 0)
                if check and not self._healthy(r):
                    r.status = "failed"
                    finished.append(slot)
                elif r.remaining == 0:
                    r.status = "ok"
                    finished.append(slot)
            for slot in finished:
                r = active.pop(slot)
                r.done = now
                if collect is not None and r.status == "ok":
                    collect(r, self.batch.state(slot))
                self.batch.remove(slot)
                done.append(r)
        makespan = time.perf_counter() - t0
        lat = [r.latency() for r in done if r.status == "ok"]
        return {
            "completed": sum(r.status == "ok" for r in done),
            "failed": sum(r.status == "failed" for r in done),
            "rejected": sum(r.status == "rejected" for r in done),
            "unfinished": len(queue) + len(active),
            "p50_latency_s": float(np.percentile(lat, 50)) if lat else None,
            "p99_latency_s": float(np.percentile(lat, 99)) if lat else None,
            "cell_steps": cell_steps,
            "makespan_s": makespan,
            "cell_steps_per_s": cell_steps / makespan if makespan > 0 else None,
            "chunks": chunks,
        }

    def close(self):
        self.batch.close()
