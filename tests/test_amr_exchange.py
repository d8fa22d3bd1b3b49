"""AMR coarse/fine exchange from the reference's own exchange plan.

The reference builds its exchange transactions for a refined block layout in
make_exchange (grid/make_exchange.h:98-421, grid/get_transaction.h:10-263):
same-level injections and coarse/fine interpolations (8 donors summed, then
x 1/8).  tests/golden/amr_ref.npz holds, for three layouts refined in place
through cartesian_grid_t::refine_blocks (one level periodic, two levels with
y walls, non-cubic blocks), the reference's plan and the array after its
exchange (tests/golden/gen_golden.py).  Here, on the CPU:

* the oracle's plan execution reproduces the reference's exchange bit for bit;
* where the reference harness is built, fresh layouts too;
* the C++ drop-in lowers the reference's own handle into exactly that plan
  (host only, where the reference sources are);
* gbns_exchange_plan_create rejects malformed plans before touching the GPU.

The GPU execution is tests/test_gpu_amr_exchange.py."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

from spade_gb300 import _abi, _native
from oracle import oracle as O
from __graft_entry__ import ref_src

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLD = os.path.join(ROOT, "tests", "golden", "amr_ref.npz")
CASES = ("one_level_periodic", "two_levels_walls_y", "anisotropic_blocks")


def amr_fill(boxes, ncell, ng):
    """The harness's interior field at cell centres (exact for power-of-two
    boxes), ghosts 0: p = 3 + x, T = 1 + y^2, u = z, v = x y, w = 2."""
    nb = boxes.shape[0]
    q = np.zeros((nb, ncell[2] + 2 * ng, ncell[1] + 2 * ng, ncell[0] + 2 * ng, 5))
    for lb in range(nb):
        c = [boxes[lb, 2 * d] + (np.arange(ncell[d]) + 0.5) * ((boxes[lb, 2 * d + 1] - boxes[lb, 2 * d]) / ncell[d])
             for d in range(3)]
        z, y, x = np.meshgrid(c[2], c[1], c[0], indexing="ij")
        inner = q[lb, ng:-ng, ng:-ng, ng:-ng]
        inner[..., 0] = 3.0 + x
        inner[..., 1] = 1.0 + y * y
        inner[..., 2] = z
        inner[..., 3] = x * y
        inner[..., 4] = 2.0
    return q


def golden(case):
    g = np.load(GOLD)
    return {k: g[case + "_" + k] for k in ("plan", "ninject", "boxes", "levels", "after", "ncell", "ng")}


@pytest.mark.parametrize("case", CASES)
def test_oracle_plan_execution_equals_reference_exchange(case):
    g = golden(case)
    ng = int(g["ng"])
    q = amr_fill(g["boxes"], g["ncell"], ng)
    O.exchange_patches(g["ncell"], ng, q.shape[0], g["plan"], q)
    assert np.array_equal(q, g["after"])
    assert len(set(g["levels"].tolist())) >= 2                     # coarse/fine interfaces present
    assert np.any(g["plan"][:, 0] == 1) and np.any(g["plan"][:, 0] == 0)


@pytest.mark.skipif(not O.ref_available(), reason="reference harness not built")
@pytest.mark.parametrize("layout", [((2, 2, 2), (4, 4, 4), 1, (0, 0, 0), [[5]]),
                                    ((3, 2, 2), (4, 4, 8), 2, (1, 1, 0), [[0, 4], [1]]),
                                    ((2, 2, 2), (8, 8, 8), 3, (1, 1, 1), [[7]])])
def test_oracle_plan_execution_equals_reference_fresh_layouts(layout):
    r = O.ref_amr_exchange(*layout)
    q = r["before"].copy()
    O.exchange_patches(layout[1], layout[2], q.shape[0], r["plan"], q)
    assert np.array_equal(q, r["after"])


@pytest.mark.skipif(not ref_src(), reason="reference sources not present")
def test_cpp_dropin_lowers_the_reference_handle_into_its_plan():
    src = ref_src()
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "dropin_amr")
        cmd = ["g++", "-std=c++20", "-O0", "-I" + src, "-I" + os.path.join(ROOT, "include"),
               "-I" + os.path.join(ROOT, "oracle", "mpi_stub"), "-I/usr/local/cuda/include",
               os.path.join(ROOT, "tests", "cpp", "dropin_amr_plan.cc"), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        out = subprocess.run([exe], capture_output=True, text=True, timeout=120).stdout.splitlines()
    plan = np.array([[int(x) for x in l.split()] for l in out[1:]], dtype=np.int32)
    want = golden("two_levels_walls_y")["plan"]
    assert np.array_equal(plan, want)


def _create(plan, ncell=(4, 4, 4), ng=2, nblocks=15):
    h = ctypes.c_void_p()
    plan = np.ascontiguousarray(plan, dtype=np.int32)
    return _native.lib().gbns_exchange_plan_create(ctypes.byref(h), ncell[0], ncell[1], ncell[2], ng, nblocks,
                                                   ctypes.c_void_p(plan.ctypes.data), int(plan.shape[0]), None)


def test_plan_validation_rejects_malformed_plans():
    g = golden("one_level_periodic")
    plan = g["plan"]
    twice = np.concatenate([plan, plan[:1]])                        # one ghost cell written twice
    assert _create(twice) == _abi.ERR_INVALID
    bad = plan.copy()
    bad[0, 6:9] = [0, 0, 0]                                         # destination inside the interior
    bad[0, 9:12] = [1, 1, 1]
    assert _create(bad) == _abi.ERR_INVALID
    bad = plan.copy()
    bad[0, 3] = 5                                                   # donor box past the padded array
    assert _create(bad) == _abi.ERR_INVALID
    # an injection whose donors are its own destination ghost cells
    selfread = np.zeros((1, 18), dtype=np.int32)
    selfread[0, :12] = [0, 0, 0, -2, 0, 0, -2, 0, 0, 0, 1, 1]
    assert _create(selfread) == _abi.ERR_UNSUPPORTED
    bad = plan.copy()
    bad[-1, 12] = 2                                                 # interpolation coefficient out of range
    assert _create(bad) == _abi.ERR_INVALID
    bad = plan.copy()
    bad[0, 1] = 99                                                  # block index out of range
    assert _create(bad) == _abi.ERR_INVALID
    assert _create(plan, ng=0) == _abi.ERR_INVALID


def _waves(g):
    plan = np.ascontiguousarray(g["plan"], dtype=np.int32)
    waves = np.zeros(plan.shape[0], dtype=np.int32)
    nc, ng = g["ncell"], int(g["ng"])
    rc = _native.lib().gbns_exchange_plan_waves(int(nc[0]), int(nc[1]), int(nc[2]), ng, int(g["boxes"].shape[0]),
                                                ctypes.c_void_p(plan.ctypes.data), int(plan.shape[0]),
                                                ctypes.c_void_p(waves.ctypes.data))
    assert rc == _abi.OK
    return plan, waves


def _run_in_waves(g, plan, waves, q):
    """Executes the plan wave by wave, every transaction of a wave reading
    before any of them writes (what one launch per wave guarantees)."""
    ng = int(g["ng"])
    for kind in (0, 1):
        for w in sorted(set(int(x) for x, r in zip(waves, plan) if r[0] == kind)):
            pending = []
            for r, wr in zip(plan, waves):
                if r[0] != kind or wr != w:
                    continue
                sb, db, slo, dlo, dhi, c, inc = r[1], r[2], r[3:6], r[6:9], r[9:12], r[12:15], r[15:18]
                for dk in range(dhi[2] - dlo[2]):
                    for dj in range(dhi[1] - dlo[1]):
                        for di in range(dhi[0] - dlo[0]):
                            if kind == 0:
                                v = q[sb, slo[2] + dk + ng, slo[1] + dj + ng, slo[0] + di + ng].copy()
                            else:
                                b = [(d << (cc + 1)) >> 1 for d, cc in zip((di, dj, dk), c)]
                                acc = np.zeros(5)
                                for iv in range(8):
                                    ii = slo[0] + b[0] + (iv & 1) * inc[0]
                                    jj = slo[1] + b[1] + ((iv >> 1) & 1) * inc[1]
                                    kk = slo[2] + b[2] + ((iv >> 2) & 1) * inc[2]
                                    acc = acc + q[sb, kk + ng, jj + ng, ii + ng]
                                v = acc * 0.125
                            pending.append(((db, dlo[2] + dk + ng, dlo[1] + dj + ng, dlo[0] + di + ng), v))
            for idx, v in pending:
                q[idx] = v


def test_plan_waves_reproduce_the_reference_order():
    """gbns_exchange_plan_waves (the launches gbns_exchange_plan_create would
    issue, host only): executing each wave as one gather (all reads before
    any write) reproduces the reference's transaction-by-transaction exchange
    bit for bit.  With y walls some interpolation donors are ghost cells
    other interpolations write: one injection wave and three interpolation
    waves; without such donors one of each."""
    for case in CASES:
        g = golden(case)
        plan, waves = _waves(g)
        q = amr_fill(g["boxes"], g["ncell"], int(g["ng"]))
        _run_in_waves(g, plan, waves, q)
        assert np.array_equal(q, g["after"]), case
        nw = {k: len(set(int(w) for w, r in zip(waves, plan) if r[0] == k)) for k in (0, 1)}
        if case == "two_levels_walls_y":
            assert nw == {0: 1, 1: 3}
        else:
            assert nw[0] <= 1 and nw[1] <= 1
