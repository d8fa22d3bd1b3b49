"""Autotuner for the flux_div tile shape.

Every tile variant of a scheme (gbns_flux_variant_count) computes the same
results (bit for bit in FP64; in FP32-flux to single-precision rounding,
since each instantiation's FP32 arithmetic is FMA-contracted on its own);
they differ in tile size, threads per CTA and, for FP32-flux, in how the halo
is staged (a TMA copy from the FP32 copy of the state, or of the FP64 box).  tune() times each variant on the caller's own
arrays with CUDA events and caches the winner per (scheme, block shape,
block count, ghosts, precision, GPU) in spade_gb300/_build/autotune.json.
"""
import json
import os

import torch

from . import _native

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build", "autotune.json")


def _key(grid, scheme):
    """Everything that selects a different kernel or changes its cost: the
    GPU, every scheme field that picks code (convective kind and order, WENO
    smoothness switch, dissipation and its sensor, hybrid blend, viscous term
    and law, precision), the block shape, ghosts, coordinates and the block
    count (small grids favour small tiles)."""
    dev = torch.cuda.get_device_name()
    return "|".join(str(x) for x in (
        dev, scheme.convective, scheme.order, scheme.weno_smooth, scheme.dissipation, scheme.sensor,
        scheme.hybrid_flux, scheme.hybrid_sensor, scheme.hybrid_param,
        scheme.viscous, scheme.visc_law, scheme.precision, tuple(grid.ncell), grid.ng, grid.coords,
        tuple(grid.nblk)))


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except Exception:
        return {}


def _store(cache):
    os.makedirs(os.path.dirname(CACHE), exist_ok=True)
    tmp = CACHE + ".tmp"
    with open(tmp, "w") as f:
        json.dump(cache, f, indent=1, sort_keys=True)
    os.replace(tmp, CACHE)


def tune(grid, scheme, prims_ptr, rhs_ptr, reps=3, use_cache=True, stream=None):
    """Returns (best_variant, {variant: ms}) and sets scheme.tile_variant."""
    lib = _native.lib()
    key = _key(grid, scheme)
    cache = _load() if use_cache else {}
    if use_cache and key in cache:
        scheme.tile_variant = int(cache[key]["variant"])
        return scheme.tile_variant, {int(k): v for k, v in cache[key]["ms"].items()}
    st = int((stream or torch.cuda.current_stream()).cuda_stream)
    n = lib.gbns_flux_variant_count(scheme)
    times = {}
    s = torch.cuda.current_stream() if stream is None else stream
    for v in range(n):
        _native.check(lib.gbns_flux_div_variant(grid, scheme, prims_ptr, rhs_ptr, 0, v, st))   # warm-up
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            _native.check(lib.gbns_flux_div_variant(grid, scheme, prims_ptr, rhs_ptr, 0, v, st))
        e1.record(s)
        e1.synchronize()
        times[v] = e0.elapsed_time(e1) / reps
    best = min(times, key=times.get)
    scheme.tile_variant = best
    if use_cache:
        cache[key] = {"variant": best, "ms": times}
        _store(cache)
    return best, times
