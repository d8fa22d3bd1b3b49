"""Benchmark: SSPRK3 cell-steps/s of the explicit Navier–Stokes RHS path on
the plain-FP64 channel at scale (8x8x8 blocks of 32^3 = 16.8M cells, 3 ghost
layers, tanh-stretched y (beta = 2), 5th-order WENO + pressure dissipation +
visc_lr with Sutherland viscosity, isothermal walls, periodic x/z).

One step = one SSPRK3 step over the whole grid: 3 flux_div launches, 3 fused
RK-stage updates, 3 ghost fills.  Inputs (1.1 GB per array) are larger than
the 129 MB L2, so no flush is needed between steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--impl reference` times the CPU restatement of the reference's algorithm
(oracle/, the reference's CPU path cannot be built on the GPU host) on all
host cores over a bounded sample of the same workload.
"""
import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-steps/s"
UNIT = "cell-steps/s"
ALG_BYTES_FLUX = 80          # read 5 + write 5 FP64 per cell per flux_div (overwrite)
ALG_BYTES_STEP = 720         # 3 x 80 + 120 + 160 + 200 per cell per SSPRK3 step (reference structure)
# flux_div with the fused stage update, per launch averaged over the 3 stages:
# (40+40+40) + (40+40+40+40) + (40+80+40) = 440 B/cell per step
ALG_BYTES_FUSED = 440.0 / 3.0


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gbns", choices=["gbns", "reference"])
    p.add_argument("--precision", default="fp64", choices=["fp64", "fp32_flux"])
    p.add_argument("--nblk", type=int, nargs=3, default=[8, 8, 8])
    p.add_argument("--ncell", type=int, nargs=3, default=[32, 32, 32])
    p.add_argument("--e2e-steps", type=int, default=5)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp32", action="store_true", help="skip the FP32-flux side measurement")
    p.add_argument("--no-forms", action="store_true", help="skip the batched and serving measurements")
    p.add_argument("--no-reference-gpu", action="store_true", help="skip the reference's own GPU flux_div leg")
    p.add_argument("--reference-gpu-only", action="store_true",
                   help="print only the reference-GPU comparison (the reference's own flux_div kernels beside gbns)")
    p.add_argument("--batch-instances", type=int, default=96)
    p.add_argument("--batch-steps", type=int, default=200)
    p.add_argument("--serve-requests", type=int, default=200)
    p.add_argument("--serve-time-limit", type=float, default=30.0,
                   help="seconds each precision serves the configured stream")
    p.add_argument("--batch-only", action="store_true",
                   help="instead of the bench line: run only the batched form (--batch-instances, --batch-steps) "
                        "and print its block")
    p.add_argument("--flux-variants", choices=["taylor_green", "channel", "channel_fweno"], default=None,
                   help="instead of the bench line: time one plain flux_div launch of every tile variant on the named "
                        "workload (--nblk blocks of --ncell cells; --precision) and print the times; with --steps 1 it "
                        "is the short, fixed launch sequence (one warm-up and one timed launch per variant) the ncu "
                        "summaries capture")
    p.add_argument("--precision-report", type=int, default=0, metavar="STEPS",
                   help="instead of the bench line: run the channel workload STEPS steps in FP64 and in the "
                        "FP32-flux form from the same state and print their per-variable errors and drifts")
    return p.parse_args()


def config(args):
    return {"workload": "channel_fp64_weno5_sutherland_tanh",
            "blocks": list(args.nblk), "cells_per_block": list(args.ncell), "ghosts": 3,
            "cells": int(math.prod(args.nblk) * math.prod(args.ncell)),
            "scheme": "compose(weno5_t, pressure_diss_lr(const_sensor), visc_lr(sutherland_t))",
            "coords": "diagonal_coords(identity, tanh_stretch(beta=2), identity)",
            "bc": "periodic x/z, isothermal no-slip walls y=+-1",
            "time_integration": "ssprk3_t with state_transform_t",
            "l2": "inputs larger than L2 (1.1 GB per array)"}


# ---------------------------------------------------------------------------
# clocks sampler
# ---------------------------------------------------------------------------
class Clocks:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1"):
                        reasons.add(n)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_gpu(args, rank, world):
    import torch
    from spade_gb300 import _abi, _native, workloads
    from spade_gb300 import build as _b
    if not _b.up_to_date():
        raise SystemExit("libgbns.so is stale or missing: run __graft_entry__.build() first")
    lib = _native.lib()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    st = int(stream.cuda_stream)

    prob = workloads.channel(nblk=tuple(args.nblk), ncell=tuple(args.ncell), ng=3, rng="torch", seed=rank)
    q = prob.q
    g = q.desc()
    prec = _abi.PREC_FP64 if args.precision == "fp64" else _abi.PREC_FP32_FLUX
    s = prob.scheme_desc(prec)
    bc = prob.bc_desc()
    dt = prob.dt
    cells = prob.grid.get_grid_size()
    n = q.data.numel()
    R = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    rptr = [r.data_ptr() for r in R]
    res = (ctypes.c_void_p * 3)(*rptr)
    c1 = (ctypes.c_double * 1)((1.0 / 1.0) * dt)
    c2 = (ctypes.c_double * 2)((-3.0 / 4.0) * dt, (1.0 / 4.0) * dt)
    c3 = (ctypes.c_double * 3)((-1.0 / 12.0) * dt, (-1.0 / 12.0) * dt, (2.0 / 3.0) * dt)
    gas = prob.gas.desc()
    qp = q.ptr()
    chk = _native.check

    from spade_gb300 import autotune
    tuned = {}
    best, times = autotune.tune(g, s, qp, rptr[0], reps=2, use_cache=False)
    tuned[args.precision] = {"variant": best, "ms_per_variant": times}

    Bbuf = torch.zeros(n, dtype=torch.float64, device="cuda")
    bp = Bbuf.data_ptr()
    e1 = (ctypes.c_void_p * 2)(rptr[0], None)
    e2 = (ctypes.c_void_p * 2)(rptr[0], rptr[1])
    stages = ((qp, rptr[0], 1, 1, e1, c1, bp), (bp, rptr[1], 1, 2, e1, c2, qp), (qp, None, 0, 3, e2, c3, bp))

    def step(events=None):
        # SSPRK3 (advance.h:234-280) exactly as gbns_ssprk3_step issues it:
        # per stage one flux_div launch with the fused stage update, then the
        # ghost fill; issued one by one so the flux launches can be timed.
        for i, (src, rhs, wr, nres, earlier, cf, dst) in enumerate(stages):
            if events is not None:
                events[i][0].record(stream)
            chk(lib.gbns_flux_div_rk(g, s, src, rhs, wr, nres, earlier, cf, dst, st))
            if events is not None:
                events[i][1].record(stream)
            if i < 2:
                chk(lib.gbns_fill_ghosts(g, bc, dst, st))
            else:
                chk(lib.gbns_copy_fill_ghosts(g, bc, qp, bp, st))

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    evs = [[[torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)] for _ in range(3)]
           for _ in range(args.steps)]
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    clocks = Clocks(dev)
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    t0.record(stream)
    for k in range(args.steps):
        step(evs[k])
    t1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clk = clocks.stop()
    ms = t0.elapsed_time(t1)
    flux_ms = [e[0].elapsed_time(e[1]) for ev in evs for e in ev]
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())

    health = ctypes.c_double(0.0)
    chk(lib.gbns_reduce(g, gas, qp, _abi.RED_HEALTH, ctypes.byref(health), st))
    launches = 6 * args.steps

    # ---- end to end through the public C-ABI call, host buffers ---------------
    # gbns_ssprk3_step_host: every step copies the whole padded state from
    # page-locked host memory and back, in block groups overlapped with the
    # first and last stage.  The serial form (copy in, gbns_ssprk3_step, copy
    # out on one stream) is timed beside it.
    host_q = torch.empty(q.data.shape, dtype=torch.float64, pin_memory=True)
    host_q.copy_(q.data)
    work = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    ke = max(1, args.e2e_steps)
    hp = host_q.data_ptr()

    def e2e_overlapped():
        chk(lib.gbns_ssprk3_step_host(g, s, bc, hp, qp, work.data_ptr(), ctypes.c_double(dt), 0, st, None))

    def e2e_serial():
        q.data.copy_(host_q, non_blocking=True)
        chk(lib.gbns_ssprk3_step(g, s, bc, qp, work.data_ptr(), ctypes.c_double(dt), st))
        host_q.copy_(q.data, non_blocking=True)

    def time_e2e(fn):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(ke):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / ke

    e2e_ms = time_e2e(e2e_overlapped)
    e2e_serial_ms = time_e2e(e2e_serial)

    # ---- other precision forms on the same workload (side measurements) --------
    def side_form(precision, key, dtype):
        sp = prob.scheme_desc(precision)
        bv, tv = autotune.tune(g, sp, qp, rptr[0], reps=3, use_cache=False)
        tuned[key] = {"variant": bv, "ms_per_variant": tv}
        w = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
        for _ in range(2):
            chk(lib.gbns_ssprk3_step(g, sp, bc, qp, w.data_ptr(), ctypes.c_double(dt), st))
        torch.cuda.synchronize()
        f0 = torch.cuda.Event(enable_timing=True)
        f1 = torch.cuda.Event(enable_timing=True)
        kk = max(3, args.steps)
        f0.record(stream)
        for _ in range(kk):
            chk(lib.gbns_ssprk3_step(g, sp, bc, qp, w.data_ptr(), ctypes.c_double(dt), st))
        f1.record(stream)
        torch.cuda.synchronize()
        fms = f0.elapsed_time(f1) / kk
        return {"value": cells / (fms * 1e-3), "unit": UNIT, "ms_per_step": fms, "dtype": dtype,
                "speedup_vs_fp64": (ms / args.steps) / fms}

    fp32 = None
    fma = None
    if not args.no_fp32 and prec == _abi.PREC_FP64:
        fp32 = side_form(_abi.PREC_FP32_FLUX, "fp32_flux", "f32-flux/f64-state")
        fma = side_form(_abi.PREC_FP64_FMA, "fp64_fma", "f64 with FMA contraction (not bit-identical)")

    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs")
    peak_src = "measured"
    if not hbm_peak:
        hbm_peak, peak_src = 6800.0, "fallback"
    fp64_rate = ctypes.c_double(0.0)
    fp32_rate = ctypes.c_double(0.0)
    chk(lib.gbns_measure_fma_rate(1, ctypes.byref(fp64_rate), st))
    chk(lib.gbns_measure_fma_rate(0, ctypes.byref(fp32_rate), st))

    flux_avg_ms = sum(flux_ms) / len(flux_ms)
    achieved = ALG_BYTES_FUSED * cells / (flux_avg_ms * 1e-3) / 1e9
    traffic = _read_traffic(cells)
    return {
        "ms": ms, "cells": cells, "launches": launches, "flux_avg_ms": flux_avg_ms,
        "flux_share": sum(flux_ms) / ms, "achieved": achieved, "hbm_peak": hbm_peak, "peak_src": peak_src,
        "clocks": clk, "health_bad_cells": health.value, "e2e_ms": e2e_ms, "e2e_serial_ms": e2e_serial_ms,
        "h2d": host_q.numel() * 8, "d2h": host_q.numel() * 8, "fp32": fp32, "fma": fma,
        "fp64_fma_flops": fp64_rate.value, "fp32_fma_flops": fp32_rate.value, "traffic": traffic,
        "tuned": tuned,
    }


def fp64_ops_roof(r):
    """The fused FP64 launch against the FP64 unit's roof: FP64-pipe thread
    operations per cell and stage (ncu, mean of the three stages of the
    committed channel capture) x cells / the launch's CUDA-event time, over
    the measured DFMA lane rate (one operation per lane and DFMA)."""
    per_cell = _profile_value("fp64_ops_per_cell")
    if not per_cell or not r.get("fp64_fma_flops"):
        return {}
    achieved = per_cell * r["cells"] / (r["flux_avg_ms"] * 1e-3)
    peak = r["fp64_fma_flops"] / 2.0
    return {"fp64_ops_per_cell_ncu": per_cell, "achieved_fp64_ops_per_s": achieved, "peak_fp64_ops_per_s": peak,
            "frac_of_fp64_peak": achieved / peak}


def _profile_value(key):
    """A `key: value` line of the committed ncu summary of the fused FP64
    flux kernel (2.1M-cell capture of the channel scheme)."""
    path = os.path.join(ROOT, "profiles", "flux_div_rk_channel_fp64.md")
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":")[1])
    except Exception:
        pass
    return None


def _read_traffic(cells):
    """DRAM bytes per fused flux_div launch (mean over the three SSPRK3
    stages) from the committed ncu summary, scaled to this workload's cell
    count (traffic grows with the cells processed)."""
    v = _profile_value("traffic_bytes_per_cell")
    return None if v is None else v * cells


# ---------------------------------------------------------------------------
# batched form: 96 Taylor-Green instances of uneven size in one batch
# ---------------------------------------------------------------------------
BLOCK_ARRANGEMENTS = {1: (1, 1, 1), 2: (2, 1, 1), 4: (2, 2, 1), 8: (2, 2, 2), 16: (4, 2, 2), 32: (4, 4, 2), 64: (4, 4, 4)}


def batch_instances(n, seed=0):
    """Seeded instance mix: blocks of 16^3 in {1,...,64}, Re log-uniform in
    [100, 3000], Mach uniform in [0.05, 0.4]."""
    import numpy as np
    r = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n):
        nb = int(r.choice(list(BLOCK_ARRANGEMENTS)))
        re = float(math.exp(r.uniform(math.log(100.0), math.log(3000.0))))
        ma = float(r.uniform(0.05, 0.4))
        out.append((BLOCK_ARRANGEMENTS[nb], re, ma))
    return out


def run_small_tgv(args):
    """The reference's CPU-runnable case (Taylor-Green, 2x2x2 blocks of 16^3
    = 32,768 cells, cent_keep<2> + visc_lr, SSPRK3) on the GPU: 20 steps with
    the fused step replayed from a CUDA graph, i.e. the per-step latency of a
    launch-bound problem, next to the same steps on the host cores."""
    import torch
    from spade_gb300 import _abi, workloads
    from spade_gb300.time_integration import ssprk3_stepper
    from spade_gb300 import autotune
    prob = workloads.taylor_green(nblk=(2, 2, 2), ncell=(16, 16, 16), ng=2, rng="torch", seed=0)
    s = prob.scheme_desc(_abi.PREC_FP64)
    r = torch.zeros_like(prob.q.data)
    best, _ = autotune.tune(prob.q.desc(), s, prob.q.ptr(), r.data_ptr(), reps=5, use_cache=False)
    st = ssprk3_stepper(prob.q, s, prob.bc_desc(), prob.dt, use_graph=True)
    st.step(3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    st.step(20)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 20
    out = {"workload": "Taylor-Green 2x2x2 blocks of 16^3 (32,768 cells), cent_keep<2> + visc_lr(constant), "
                       "FP64, fused step replayed from a CUDA graph", "steps": 20, "ms_per_step": ms,
           "tile_variant": best, "cell_steps_per_s": 32768 / (ms * 1e-3)}
    if not args.no_cpu_baseline:
        # the same 20 steps on the host cores (the oracle restatement, bit-identical
        # to the reference's CPU path for this scheme)
        import numpy as np
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
        from oracle import oracle as O
        q = prob.q.data.cpu().numpy().copy()
        work = np.zeros((3,) + q.shape)
        t = time.perf_counter()
        for _ in range(20):
            O.ssprk3_step(prob.q.desc(), s, prob.bc_desc(), q, work, prob.dt)
        el = time.perf_counter() - t
        out["cpu_baseline"] = {"ms_per_step": el / 20 * 1e3, "cell_steps_per_s": 32768 * 20 / el,
                               "cores": O.max_threads(), "kind": "port"}
    return out


def run_batch_form(args):
    import torch
    from spade_gb300 import _abi, _native, workloads
    from spade_gb300.batch import batch_t
    lib = _native.lib()
    st = int(torch.cuda.current_stream().cuda_stream)
    mix = batch_instances(args.batch_instances, seed=1)
    probs = []
    for i, (nb, re, ma) in enumerate(mix):
        probs.append(workloads.taylor_green(nblk=nb, ncell=(16, 16, 16), ng=2, mach=ma, reynolds=re, seed=i, rng="torch",
                                            p_factor=1.0 / 16.0))
    cells = sum(p.grid.get_grid_size() for p in probs)
    out = {"workload": "%d Taylor-Green instances (textbook pressure field), 16^3 blocks, blocks per instance from "
                       "{1,...,64}, Re log-uniform [100,3000], Mach uniform [0.05,0.4]" % len(probs),
           "instances": len(probs), "cells": cells, "steps": args.batch_steps}
    for name, prec in (("fp64", _abi.PREC_FP64), ("fp32_flux", _abi.PREC_FP32_FLUX)):
        budget = sum(batch_t.instance_bytes(p.q.desc()) for p in probs) + (256 << 20)
        b = batch_t(budget, prec, True)
        for p in probs:
            b.add(p.q.desc(), p.scheme_desc(prec), p.bc_desc(), p.dt, p.q.ptr())
        # tile variant per kernel class, timed on the instances' own arrays
        tuned = b.autotune(reps=3)
        b.step(2)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        b.step(args.batch_steps)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.batch_steps
        out[name] = {"cell_steps_per_s": cells / (ms * 1e-3), "ms_per_step": ms,
                     "launches_per_step": 6, "graph": True, "autotuned": tuned}
        b.close()
    # the same instances one grid at a time (one gbns_ssprk3_step per instance)
    works = [torch.zeros(3 * p.q.data.numel(), dtype=torch.float64, device="cuda") for p in probs]
    descs = [(p.q.desc(), p.scheme_desc(_abi.PREC_FP64), p.bc_desc(), p.q.ptr(), w.data_ptr(), ctypes.c_double(p.dt))
             for p, w in zip(probs, works)]
    def one_step():
        for g, sc, bc, qp, wp, dt in descs:
            _native.check(lib.gbns_ssprk3_step(g, sc, bc, qp, wp, dt, st))
    one_step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    n_plain = max(1, min(args.batch_steps, 20))
    for _ in range(n_plain):
        one_step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / n_plain
    out["fp64_one_grid_at_a_time"] = {"cell_steps_per_s": cells / (ms * 1e-3), "ms_per_step": ms, "steps": n_plain,
                                      "launches_per_step": 6 * len(probs)}
    out["fp32_batched_vs_fp64_plain"] = out["fp32_flux"]["cell_steps_per_s"] / out["fp64_one_grid_at_a_time"]["cell_steps_per_s"]
    del probs, works
    torch.cuda.empty_cache()
    return out


def run_serve_form(args):
    """Serving form, FP32-flux beside plain FP64.  Two streams per precision:
    the configured one (Poisson 40 req/s, `--serve-requests` requests; it
    offers far more work than one GPU does, so it is served for
    `--serve-time-limit` seconds and what completed is reported), and a
    sustainable one at 70 % of the capacity that run measured, where the
    latencies are those of continuous batching rather than of a queue."""
    import torch
    from spade_gb300 import _abi, serve
    out = {"workload": ("Poisson arrivals, 70% Taylor-Green / 30% channel, edges {16,32,64,128} (16^3 blocks up to "
                        "32^3, 32^3 beyond), steps U[100,2000], Re log-U[100,3000], Mach U[0.05,0.4], 150 GB HBM budget")}
    for name, prec in (("fp32_flux", _abi.PREC_FP32_FLUX), ("fp64", _abi.PREC_FP64)):
        reqs = serve.poisson_requests(args.serve_requests, rate=40.0, seed=3)
        work = [r.cells * r.steps for r in reqs]
        span = reqs[-1].arrival - reqs[0].arrival
        srv = serve.server_t(prec, hbm_budget=150 << 30, chunk=16, health_every=8)
        full = srv.run(reqs, time_limit=args.serve_time_limit)
        srv.close()
        torch.cuda.empty_cache()
        full["rate_req_per_s"] = 40.0
        full["offered_cell_steps_per_s"] = sum(work) / span
        full["offered_over_capacity"] = full["offered_cell_steps_per_s"] / full["cell_steps_per_s"]
        # a stream the GPU sustains: 70 % of the measured capacity
        mean_work = sum(work) / len(work)
        rate = 0.7 * full["cell_steps_per_s"] / mean_work
        n = 30 if prec == _abi.PREC_FP32_FLUX else 6
        sreqs = serve.poisson_requests(n, rate=rate, seed=5)
        srv = serve.server_t(prec, hbm_budget=150 << 30, chunk=16, health_every=8)
        # served until every request has arrived plus the configured window
        sus = srv.run(sreqs, time_limit=sreqs[-1].arrival + args.serve_time_limit)
        srv.close()
        torch.cuda.empty_cache()
        sus["rate_req_per_s"] = rate
        sus["offered_cell_steps_per_s"] = sum(r.cells * r.steps for r in sreqs) / (sreqs[-1].arrival - sreqs[0].arrival)
        out[name] = {"configured_stream": full, "sustainable_stream": sus}
    out["fp32_flux_vs_fp64_throughput"] = (out["fp32_flux"]["configured_stream"]["cell_steps_per_s"] /
                                           out["fp64"]["configured_stream"]["cell_steps_per_s"])
    return out


# ---------------------------------------------------------------------------
# CPU baseline: the oracle restatement on the host cores, bounded sample
# ---------------------------------------------------------------------------
def run_reference_gpu(args, reps=3):
    """The reference's own GPU flux_div (basic, bfoct, longf), replayed on
    this GPU from launch scripts recorded where its sources are
    (oracle/refgpu.py), beside this library's flux_div on the same grid,
    scheme and state: ms per flux_div (CUDA events on the launching stream,
    median of `reps` after one warm-up) and cell-RHS/s."""
    import torch
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle import refgpu
    from spade_gb300 import _abi, _native, autotune, workloads
    if not refgpu.available():
        return {"unavailable": "reference GPU recordings absent (recorded where the reference sources are)"}
    lib = _native.lib()
    out = {}
    clocks = Clocks(torch.cuda.current_device())
    for case in refgpu.CASE_NAMES:
        if case == "tgv_ck2_visc":
            prob = workloads.taylor_green(nblk=(8, 8, 8), ncell=(32, 32, 32), ng=2, rng="torch", seed=0)
        else:
            prob = workloads.channel(nblk=(8, 8, 8), ncell=(32, 32, 32), ng=2, beta=None, weno="fweno",
                                     law="constant", rng="torch", seed=0)
        cells = 8 * 8 * 8 * 32 ** 3
        st = torch.cuda.current_stream()
        sp = int(st.cuda_stream)

        def timed(fn):
            fn()
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                fn()
                e1.record(st)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1))
            return statistics.median(ts)

        rhs = torch.zeros_like(prob.q.data)
        rep = refgpu.Replay(case, prob.q.data, rhs, sp)
        row = {"cells": cells, "scheme": case, "reference": {}, "gbns": {}}
        try:
            for alg in ("basic", "bfoct", "longf"):
                ms = timed(lambda: rep.run(alg, sp))
                row["reference"][alg] = {"ms": ms, "cell_rhs_per_s": cells / (ms * 1e-3), "launches": rep.launches[alg]}
        finally:
            rep.close()
        for prec, name in ((_abi.PREC_FP64, "fp64"), (_abi.PREC_FP32_FLUX, "fp32_flux")):
            sd = prob.scheme_desc(prec)
            best, times = autotune.tune(prob.q.desc(), sd, prob.q.ptr(), rhs.data_ptr(), use_cache=False)
            ms = timed(lambda: _native.check(lib.gbns_flux_div_variant(prob.q.desc(), sd, prob.q.ptr(),
                                                                        rhs.data_ptr(), 0, best, sp)))
            row["gbns"][name] = {"ms": ms, "cell_rhs_per_s": cells / (ms * 1e-3), "variant": best}
        best_ref = min(v["ms"] for v in row["reference"].values())
        row["speedup_fp64_vs_best_reference"] = best_ref / row["gbns"]["fp64"]["ms"]
        row["speedup_fp32_flux_vs_best_reference"] = best_ref / row["gbns"]["fp32_flux"]["ms"]
        out[case] = row
        del prob, rhs
        torch.cuda.empty_cache()
    out["clocks"] = clocks.stop()
    out["note"] = ("the reference's CUDA flux_div kernels (its own source, nvcc defaults + lambda flags, sm_103a) "
                   "run unchanged on this GPU: one flux_div in increment mode per algorithm; gbns: one flux_div "
                   "in overwrite mode with the autotuned tile")
    return out


def cpu_sample(steps=1, nblk=(2, 2, 2), ncell=(32, 32, 32), threads=0):
    import numpy as np
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle import oracle as O
    from spade_gb300 import _abi
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    beta = 2.0
    bounds = (0.0, 4 * math.pi * nblk[0] / 8, -1.0, 1.0, 0.0, 4 * math.pi / 3 * nblk[2] / 8)
    grid = _abi.grid_desc(nblk, ncell, 3, bounds, _abi.COORDS_TANH_Y, (beta, 0, 0, 0))
    gamma, R, Tw = 1.4, 287.0, 300.0
    c_w = math.sqrt(gamma * R * Tw)
    U_b = 0.5 * c_w
    shape = (nblk[0] * nblk[1] * nblk[2], ncell[2] + 6, ncell[1] + 6, ncell[0] + 6, 5)
    r = np.random.Generator(np.random.PCG64(0))
    q = np.empty(shape)
    q[..., 0] = R * Tw
    q[..., 1] = Tw
    q[..., 2] = U_b * (1.0 + 0.05 * r.standard_normal(shape[:-1]))
    q[..., 3] = 0.05 * U_b * r.standard_normal(shape[:-1])
    q[..., 4] = 0.05 * U_b * r.standard_normal(shape[:-1])
    s = _abi.SchemeDesc()
    s.convective = _abi.CONV_WENO5
    s.order = 2
    s.weno_smooth = 1
    s.dissipation = 1
    s.sensor_alpha = 1.0
    s.eps_p = s.eps_T = 0.01 * c_w
    s.viscous = 1
    s.visc_law = _abi.LAW_SUTHERLAND
    s.mu = U_b / 3000.0
    s.prandtl = 0.72
    s.T_ref = Tw
    s.S = 110.4
    s.gas.gamma = gamma
    s.gas.R = R
    bc = _abi.bc_desc([0, 0, 2, 2, 0, 0], [0, 0, Tw, Tw, 0, 0])
    O.fill_ghosts(grid, bc, q)
    work = np.zeros((3,) + shape)
    cells = math.prod(nblk) * math.prod(ncell)
    dt = 1e-7
    t = time.perf_counter()
    for _ in range(steps):
        O.ssprk3_step(grid, s, bc, q, work, dt, threads)
    el = time.perf_counter() - t
    cores = O.max_threads() if threads == 0 else threads
    return {"value": cells * steps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d SSPRK3 step(s) of the channel scheme on a %dx%dx%d-block sub-box of %d^3 cells (%d cells), "
                      "oracle/gbns_oracle.c (face-twice like flux_div_basic), OpenMP over blocks, %.1f s"
                      % (steps, nblk[0], nblk[1], nblk[2], ncell[0], cells, el)}


def run_precision_report(args):
    """Precision form on the channel workload: STEPS SSPRK3 steps in plain
    FP64 (bit-identical to the reference's arithmetic) and in the FP32-flux
    form from the same initial state.  Reports, per conserved variable, the
    max and L2 error of the FP32-flux state against the FP64 run, the drift of
    total mass and energy in both runs, and the kinetic-energy history error."""
    import torch
    from spade_gb300 import _abi, _native, workloads
    lib = _native.lib()
    st = int(torch.cuda.current_stream().cuda_stream)
    prob = workloads.channel(nblk=tuple(args.nblk), ncell=tuple(args.ncell), ng=3, rng="torch", seed=0)
    g = prob.q.desc()
    bc = prob.bc_desc()
    gas = prob.gas.desc()
    dt = prob.dt
    q0 = prob.q.data.clone()
    n = q0.numel()
    work = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    every = max(1, args.precision_report // 50)

    def reduce(ptr, kind):
        out = (ctypes.c_double * 5)()
        _native.check(lib.gbns_reduce(g, gas, ctypes.c_void_p(ptr), kind, ctypes.byref(out), st))
        return list(out)

    def run(prec):
        from spade_gb300 import autotune
        s = prob.scheme_desc(prec)
        q = prob.q
        q.data.copy_(q0)
        # the tuned tile, as the bench line's runs use (results do not depend on it)
        autotune.tune(g, s, q.ptr(), work.data_ptr(), reps=2, use_cache=False)
        hist = {"step": [], "ke": [], "mass": [], "energy": []}
        t0 = time.perf_counter()
        for k in range(args.precision_report + 1):
            if k % every == 0 or k == args.precision_report:
                c = reduce(q.ptr(), _abi.RED_CONSERVED)
                hist["step"].append(k)
                hist["ke"].append(reduce(q.ptr(), _abi.RED_KINETIC)[0])
                hist["mass"].append(c[0])
                hist["energy"].append(c[1])
            if k < args.precision_report:
                _native.check(lib.gbns_ssprk3_step(g, s, bc, q.ptr(), work.data_ptr(), ctypes.c_double(dt), st))
        torch.cuda.synchronize()
        return q.data.clone(), hist, time.perf_counter() - t0

    q64, h64, t64 = run(_abi.PREC_FP64)
    q32, h32, t32 = run(_abi.PREC_FP32_FLUX)
    ng = prob.ng
    i64 = q64[:, ng:-ng, ng:-ng, ng:-ng, :].reshape(-1, 5)
    i32 = q32[:, ng:-ng, ng:-ng, ng:-ng, :].reshape(-1, 5)
    # conserved variables (rho, rhoE, rhou, rhov, rhow) from the primitives
    def cons(a):
        p, T, u = a[:, 0], a[:, 1], a[:, 2:5]
        rho = p / (prob.gas.R * T)
        e = p / (rho * (prob.gas.gamma - 1.0)) + 0.5 * (u * u).sum(1)
        return torch.stack([rho, rho * e, rho * u[:, 0], rho * u[:, 1], rho * u[:, 2]], 1)
    c64, c32 = cons(i64), cons(i32)
    names = ["rho", "rhoE", "rhou", "rhov", "rhow"]
    err = {}
    for v, nm in enumerate(names):
        d = (c32[:, v] - c64[:, v])
        scale = c64[:, v].abs().max().item()
        err[nm] = {"max_abs": d.abs().max().item(), "max_rel_to_field_max": d.abs().max().item() / scale,
                   "l2_rel": (d.norm() / c64[:, v].norm()).item()}
    ke_rel = max(abs(a - b) / abs(b) for a, b in zip(h32["ke"], h64["ke"]))
    out = {
        "report": "precision_form", "workload": config(args)["workload"], "cells": prob.grid.get_grid_size(),
        "steps": args.precision_report, "dt": dt,
        "per_variable_error_fp32_flux_vs_fp64": err,
        "ke_history_max_rel_error": ke_rel,
        "mass_drift_rel": {"fp64": (h64["mass"][-1] - h64["mass"][0]) / h64["mass"][0],
                           "fp32_flux": (h32["mass"][-1] - h32["mass"][0]) / h32["mass"][0]},
        "energy_drift_rel": {"fp64": (h64["energy"][-1] - h64["energy"][0]) / h64["energy"][0],
                             "fp32_flux": (h32["energy"][-1] - h32["energy"][0]) / h32["energy"][0]},
        "wall_s": {"fp64": t64, "fp32_flux": t32},
        "history": {"step": h64["step"], "ke_fp64": h64["ke"], "ke_fp32_flux": h32["ke"],
                    "energy_fp64": h64["energy"], "energy_fp32_flux": h32["energy"]},
    }
    print(json.dumps(out))


def run_flux_variants(args):
    """One plain flux_div (overwrite mode) per tile variant, CUDA events on
    the launching stream: one warm-up launch and --steps timed launches each
    (median).  Workloads: taylor_green (cent_keep<2> + visc_lr(constant),
    identity, ng 2), channel (the bench's WENO5 + pressure dissipation +
    Sutherland on tanh-y, ng 3), channel_fweno (fweno_t + pressure dissipation
    + constant viscosity, uniform, ng 2: the reference-GPU comparison's)."""
    import torch
    from spade_gb300 import _abi, _native, workloads
    lib = _native.lib()
    nb, nc = tuple(args.nblk), tuple(args.ncell)
    if args.flux_variants == "taylor_green":
        prob = workloads.taylor_green(nblk=nb, ncell=nc, ng=2, rng="torch", seed=0)
    elif args.flux_variants == "channel":
        prob = workloads.channel(nblk=nb, ncell=nc, ng=3, rng="torch", seed=0)
    else:
        prob = workloads.channel(nblk=nb, ncell=nc, ng=2, beta=None, weno="fweno", law="constant", rng="torch", seed=0)
    prec = _abi.PREC_FP32_FLUX if args.precision == "fp32_flux" else _abi.PREC_FP64
    g, s = prob.q.desc(), prob.scheme_desc(prec)
    rhs = torch.zeros_like(prob.q.data)
    st = torch.cuda.current_stream()
    sp = int(st.cuda_stream)
    times = {}
    for v in range(lib.gbns_flux_variant_count(s)):
        launch = lambda: _native.check(lib.gbns_flux_div_variant(g, s, prob.q.ptr(), rhs.data_ptr(), 0, v, sp))
        launch()
        ts = []
        for _ in range(max(1, args.steps)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            launch()
            e1.record(st)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        times[v] = statistics.median(ts)
    cells = int(math.prod(nb) * math.prod(nc))
    print(json.dumps({"flux_variants": args.flux_variants, "precision": args.precision, "cells": cells,
                      "ms_per_variant": times, "best": min(times, key=times.get),
                      "cell_rhs_per_s": {v: cells / (t * 1e-3) for v, t in times.items()}}))


def main():
    args = parse()
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    cfg = config(args)
    if args.precision_report:
        run_precision_report(args)
        return
    if args.flux_variants:
        if rank == 0:
            run_flux_variants(args)
        return
    if args.batch_only:
        if rank == 0:
            print(json.dumps({"batch_form": run_batch_form(args)}))
        return
    if args.reference_gpu_only:
        if rank == 0:
            print(json.dumps({"reference_gpu": run_reference_gpu(args)}))
        return
    if args.impl == "reference":
        if rank != 0:
            return
        warm = 0
        tw = time.perf_counter()
        while warm < args.warmup and time.perf_counter() - tw < 60:
            cpu_sample(steps=1, nblk=(4, 4, 2))
            warm += 1
        vals = []
        cb = None
        t0 = time.perf_counter()
        for _ in range(max(1, args.steps)):
            cb = cpu_sample(steps=1, nblk=(4, 4, 2))
            vals.append(cb["value"])
            if time.perf_counter() - t0 > 120:
                break
        v = statistics.median(vals)
        line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
                "steps": len(vals), "warmup": warm, "ms_per_step": cfg["cells"] / v * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": dict(cfg, reference_sample="each step: 1 SSPRK3 step of a 4x4x2-block sub-box of 32^3 cells "
                                                     "(1,048,576 cells, same scheme, coordinates and walls); value = "
                                                     "sub-box cells / sub-box step time, ms_per_step = the full "
                                                     "grid's cells / value (extrapolated, per-cell cost is "
                                                     "state-independent for these branch-free schemes)"),
                "cpu_baseline": {"value": v, "unit": UNIT, "cores": cb["cores"], "kind": "port",
                                 "sample": "per step: 1 SSPRK3 step on a 4x4x2-block sub-box of 32^3 cells "
                                           "(1048576 cells) of the channel workload; the reference's CPU path cannot "
                                           "be built on the GPU host (its sources are absent there), so the oracle "
                                           "restatement oracle/gbns_oracle.c (bit-exact to the reference on the "
                                           "pinned schemes) runs on all host cores"},
                "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    r = run_gpu(args, rank, world)
    cells_all = r["cells"] * world
    value = cells_all * args.steps / (r["ms"] * 1e-3)
    if rank != 0:
        return
    forms = {}
    if not args.no_forms:
        forms["small_tgv"] = run_small_tgv(args)
        forms["batch_form"] = run_batch_form(args)
        forms["serve_form"] = run_serve_form(args)
        if not args.no_reference_gpu:
            forms["reference_gpu"] = run_reference_gpu(args)
    cpu = None
    cpu1 = None
    if world == 1 and not args.no_cpu_baseline:
        cpu = cpu_sample(steps=1, nblk=(4, 4, 2))
        cpu1 = cpu_sample(steps=1, nblk=(1, 2, 1), threads=1)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["ms"] / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.precision == "fp64" else "f32-flux/f64-state", "data": "synthetic", "config": cfg,
        "roofline": {"bound": "hbm", "kernel": "flux_div_kernel (with the fused RK stage update)",
                     "achieved": r["achieved"], "peak": r["hbm_peak"],
                     "unit": "GB/s", "frac": r["achieved"] / r["hbm_peak"],
                     "traffic": r["traffic"],
                     "traffic_source": "scaled from 2.1M-cell ncu capture (dram__bytes_read.sum + dram__bytes_write.sum "
                                       "per cell, profiles/flux_div_rk_channel_fp64.md) to this workload's cells",
                     "peak_source": r["peak_src"] + " (MEASURED_PEAKS.json hbm_gbs)",
                     "alg_bytes_per_cell": ALG_BYTES_FUSED, "avg_launch_ms": r["flux_avg_ms"],
                     "share_of_step": r["flux_share"]},
        "fp64_roof": {"fma_rate_tflops": r["fp64_fma_flops"] / 1e12, "fp32_fma_rate_tflops": r["fp32_fma_flops"] / 1e12,
                      "note": "measured DFMA/FFMA chains on this GPU; the FP64 kernel is bound by the FP64 unit, with its "
                              "products, quotients and square roots computed exactly on the integer pipes",
                      "fp64_pipe_active_frac_ncu": _profile_value("fp64_pipe_active_frac"),
                      "pipe_source": "profiles/flux_div_rk_channel_fp64.md (sm__pipe_fp64_cycles_active, 2.1M-cell capture)",
                      **fp64_ops_roof(r)},
        "step_bytes": {"alg_bytes_per_cell_step": ALG_BYTES_STEP,
                       "achieved_gbs": ALG_BYTES_STEP * cells_all * args.steps / (r["ms"] * 1e-3) / 1e9},
        "clocks": r["clocks"],
        "e2e": {"value": r["cells"] * world / (r["e2e_ms"] * 1e-3), "unit": UNIT,
                "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": r["d2h"],
                "path": "gbns_ssprk3_step_host (C ABI): the state copied from pinned host memory and back every "
                        "step, in 8 block groups overlapped with stages 1 and 3",
                "serial_ms_per_step": r["e2e_serial_ms"],
                "serial_path": "copy in, gbns_ssprk3_step, copy out on one stream"},
        "gpu_launches": r["launches"],
        "health_bad_cells": r["health_bad_cells"],
        "fp32_flux": r["fp32"],
        "fp64_fma": r["fma"],
        "autotune": r["tuned"],
        # one plain flux_div (overwrite mode, no stage update) with the tuned
        # tile, from the autotuner's CUDA-event timings: cell-RHS/s
        "flux_div_cell_rhs_per_s": {k: r["cells"] / (min(v["ms_per_variant"].values()) * 1e-3)
                                    for k, v in r["tuned"].items()},
    }
    line.update(forms)
    if cpu is not None:
        line["cpu_baseline"] = cpu
        line["cpu_baseline_1core"] = cpu1
    print(json.dumps(line))


if __name__ == "__main__":
    main()
