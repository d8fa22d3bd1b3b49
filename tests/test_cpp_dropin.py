"""The C++ drop-in header (include/spade_gb300.h) compiled against the
reference's own headers: the gb300 trait selects the GB300 overload of
spade::pde_algs::flux_div and the functor / grid lowering produces the
expected C-ABI descriptors; the ghost fill and the fused SSPRK3 integrator
lower the periodic flags and wall kernels, and the wall kernels also work as
the kernel of the reference's own CPU boundary_fill.  Host only (the GPU call goes to a hook); runs
only where the reference sources exist."""
import os
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

from __graft_entry__ import ref_src

REF_SRC = ref_src() or ""
CUDA_INC = "/usr/local/cuda/include"


@pytest.mark.skipif(not REF_SRC, reason="reference sources not present")
def test_dropin_overload_and_lowering():
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "dropin")
        cmd = ["g++", "-std=c++20", "-O0", "-I" + REF_SRC, "-I" + os.path.join(ROOT, "include"),
               "-I" + os.path.join(ROOT, "oracle", "mpi_stub"), "-I" + CUDA_INC,
               os.path.join(ROOT, "tests", "cpp", "dropin_lowering.cc"), "-o", exe]
        r = subprocess.run(cmd, capture_output=True, text=True)
        assert r.returncode == 0, r.stderr[-3000:]
        out = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = out.stdout.strip().splitlines()
    grids = [l.split() for l in lines if l.startswith("grid")]
    schemes = [l.split() for l in lines if l.startswith("scheme")]
    coords = [l.split() for l in lines if l.startswith("coords")]
    assert len(grids) == 7 and len(schemes) == 7 and len(coords) == 7
    assert all(c[1] == "0" for c in coords[:5])
    # weno5_t + pressure_diss + visc_lr(sutherland_t) on the tanh-stretched grid
    s, c = schemes[5], coords[5]
    assert s[1] == "4" and s[4] == "1" and s[5] == "1" and s[6] == "2"
    assert c[1] == "1" and float(c[2]) == 2.0
    assert float(c[c.index("S") + 1]) == 110.4 and float(c[c.index("Tref") + 1]) == 300.0
    assert float(c[c.index("pr") + 1]) == 0.72 and float(s[11]) == 1.8e-5
    # ... and on the integrated-tanh grid: its (y0, y1, inflation, rate) recovered
    c = coords[6]
    assert c[1] == "2" and float(c[2]) == -1.0 and float(c[3]) == 1.0
    assert abs(float(c[4]) - 0.3) < 1e-14 and abs(float(c[5]) - 2.5) < 1e-14
    assert grids[0][1:8] == ["2", "3", "1", "8", "6", "4", "3"]
    assert [float(x) for x in grids[0][8:14]] == [0.0, 2.0, -1.0, 1.0, 0.0, 0.5]
    # cent_keep<2> + visc_lr(constant), FP64, increment
    s = schemes[0]
    assert s[1:8] == ["1", "2", "1", "0", "1", "0", "0"] and s[s.index("incr") + 1] == "1"
    assert float(s[11]) == 1.5e-5 and float(s[12]) == 1.0 / 0.72
    # fweno + pressure_diss(const 0.25, 0.1, 0.2) + visc, FP32 flux, overwrite
    s = schemes[1]
    assert s[1:8] == ["3", "2", "1", "1", "1", "0", "1"] and s[s.index("incr") + 1] == "0"
    assert [float(x) for x in s[8:11]] == [0.1, 0.2, 0.25]
    assert s[s.index("sensor") + 1] == "0"
    # totani alone
    s = schemes[2]
    assert s[1:8] == ["2", "2", "1", "0", "0", "0", "0"]
    # fweno + pressure_diss(ducros_t(0.5), 0.1, 0.2) + visc: the sensor kind
    # is ducros and sensor_alpha carries epsilon
    s = schemes[3]
    assert s[1:8] == ["3", "2", "1", "1", "1", "0", "0"] and s[s.index("sensor") + 1] == "1"
    assert [float(x) for x in s[8:11]] == [0.1, 0.2, 0.5]
    # hybrid_scheme_t(cent_keep<4>, fweno_t, ducros_t(0.125), diss_flux) + visc
    s = schemes[4]
    assert s[1:3] == ["5", "4"] and s[5] == "1"
    h = s.index("hyb")
    assert s[h + 1:h + 3] == ["1", "1"] and float(s[h + 3]) == 0.125
    # source_term overload: body force, then body acceleration with the gas R
    srcs = [l.split() for l in lines if l.startswith("source")]
    assert len(srcs) == 2
    assert srcs[0][1] == "1" and [float(x) for x in srcs[0][4:7]] == [2.5, 0.0, -1.0]
    assert srcs[1][1] == "2" and [float(x) for x in srcs[1][4:7]] == [0.0, -9.81, 0.0] and float(srcs[1][8]) == 287.0
    # boundary_flux overload: y-min and y-max flags, cent_keep<4> + visc_lr lowered
    bf = [l.split() for l in lines if l.startswith("bflux")]
    assert len(bf) == 1
    assert bf[0][1:7] == ["0", "0", "1", "1", "0", "0"]
    assert bf[0][bf[0].index("conv") + 1] == "1" and bf[0][bf[0].index("order") + 1] == "4"
    assert bf[0][bf[0].index("visc") + 1] == "1" and bf[0][bf[0].index("ng") + 1] == "3"
    # ghost fill and fused SSPRK3 integrator: periodic x/z, isothermal walls
    # (300 K) in y; then a slip wall on z-min only, x and y periodic
    bcs = [l.split() for l in lines if l.startswith("bc")]
    assert len(bcs) == 4
    assert bcs[0][1:7] == ["0", "0", "2", "2", "0", "0"] and [float(x) for x in bcs[0][8:10]] == [300.0, 300.0]
    assert bcs[0][bcs[0].index("step") + 1] == "0"
    for b in bcs[1:3]:
        assert b[1:7] == bcs[0][1:7] and b[b.index("step") + 1] == "1" and b[b.index("conv") + 1] == "4"
        assert float(b[b.index("dt") + 1]) == 2.5e-4
    assert bcs[3][1:7] == ["0", "0", "0", "0", "3", "1"]
    t = [l.split() for l in lines if l.startswith("integrator")][0]
    assert float(t[2]) == 5e-4
    # the wall kernel through the reference's own CPU boundary_fill: the
    # ghost below y-min of a uniform (1e5, 310, 2, -1, 0.5) state
    w = [l.split() for l in lines if l.startswith("cpu_wall")][0]
    assert [float(x) for x in w[1:6]] == [1.0e5, 290.0, -2.0, 1.0, -0.5]


@pytest.mark.skipif(not REF_SRC, reason="reference sources not present")
def test_dropin_host_array_path_compiles():
    """Without the test hooks, the gb300 flux_div overload compiles for
    device::cpu grid_arrays (the host path through gbns_flux_div_host)."""
    cmd = ["g++", "-std=c++20", "-fsyntax-only", "-I" + REF_SRC, "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "oracle", "mpi_stub"), "-I" + CUDA_INC,
           os.path.join(ROOT, "tests", "cpp", "dropin_host_arrays.cc")]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]


@pytest.mark.skipif(not REF_SRC, reason="reference sources not present")
def test_dropin_gpu_array_path_compiles():
    """Without the test hooks, the gb300 flux_div overload, the ghost fill
    and the fused SSPRK3 integrator instantiate for device::gpu grid_arrays
    under nvcc with the reference's CUDA build options (compile only)."""
    with tempfile.TemporaryDirectory() as d:
        cmd = ["nvcc", "-x", "cu", "-std=c++20", "--extended-lambda", "--expt-relaxed-constexpr", "-w",
               "-gencode", "arch=compute_103a,code=sm_103a", "-I" + REF_SRC, "-I" + os.path.join(ROOT, "include"),
               "-I" + os.path.join(ROOT, "oracle", "mpi_stub"), "-c",
               os.path.join(ROOT, "tests", "cpp", "dropin_gpu_arrays.cu"), "-o", os.path.join(d, "dropin_gpu.o")]
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=1200)
        assert r.returncode == 0, r.stderr[-3000:]


def test_recorded_dropin_calls_reproduce_the_reference_on_the_oracle():
    """The C-ABI calls the drop-in made at a SPADE call site
    (tests/golden/dropin_ref.npz, recorded by tests/cpp/dropin_record.cc):
    run by the oracle, the two schemes the reference has give its own CPU
    result bit for bit, so the recorded descriptors carry the reference's
    scheme and grid exactly (the GPU replay is tests/test_gpu_dropin_replay.py)."""
    import numpy as np
    from spade_gb300 import _abi
    from oracle import oracle as O
    g = np.load(os.path.join(ROOT, "tests", "golden", "dropin_ref.npz"))
    for k in range(2):
        grid = _abi.GridDesc.from_buffer_copy(g["grid%d" % k].tobytes())
        s = _abi.SchemeDesc.from_buffer_copy(g["scheme%d" % k].tobytes())
        shape = (grid.nblk[0] * grid.nblk[1] * grid.nblk[2], grid.ncell[2] + 2 * grid.ng,
                 grid.ncell[1] + 2 * grid.ng, grid.ncell[0] + 2 * grid.ng, 5)
        q = g["q"].reshape(shape).copy()
        r = g["rhs_in%d" % k].reshape(shape).copy()
        O.flux_div(grid, s, q, r, increment=bool(g["incr%d" % k]))
        assert np.array_equal(r.ravel(), g["ref"][k]), k


def refined_dropin_call(k):
    """Call k of tests/golden/dropin_amr_ref.npz (the drop-in on a refined
    grid, recorded by tests/cpp/dropin_amr_record.cc): its descriptors, block
    boxes, the rebuilt state (seeded noise, then the reference's exchange plan
    of the same layout), the rhs the call started from, its increment flag,
    ghost depth and the reference's interior result."""
    import numpy as np
    from spade_gb300 import _abi
    from oracle import oracle as O
    from golden.gen_golden import AMR_CASES, dropin_noise_state
    g = np.load(os.path.join(ROOT, "tests", "golden", "dropin_amr_ref.npz"))
    amr = np.load(os.path.join(ROOT, "tests", "golden", "amr_ref.npz"))
    grid = _abi.GridDesc.from_buffer_copy(g["grid%d" % k].tobytes())
    s = _abi.SchemeDesc.from_buffer_copy(g["scheme%d" % k].tobytes())
    nb, nc, ng, per, passes = AMR_CASES["one_level_periodic"]
    assert tuple(grid.ncell) == tuple(nc) and grid.ng == ng and tuple(grid.nblk)[1:] == (1, 1)
    shape = (grid.nblk[0], nc[2] + 2 * ng, nc[1] + 2 * ng, nc[0] + 2 * ng, 5)
    q = dropin_noise_state(int(np.prod(shape))).reshape(shape)
    O.exchange_patches(nc, ng, shape[0], amr["one_level_periodic_plan"], q)
    r = np.full(shape, float(g["rhs_fill%d" % k]))
    return grid, s, amr["one_level_periodic_boxes"], q, r, int(g["incr%d" % k]), ng, g["ref%d" % k]


def test_refined_dropin_calls_reproduce_the_reference_on_the_oracle():
    """The drop-in at a SPADE call site on a refined (amr_blocks_t) grid lowers
    to gbns_flux_div_blocks_host with nblk = (15, 1, 1) and the grid's own
    block boxes; run by the oracle, both recorded calls (overwrite and
    increment) give the reference's CPU flux_div bit for bit."""
    import numpy as np
    from oracle import oracle as O
    for k in range(2):
        grid, s, boxes, q, r, incr, ng, want = refined_dropin_call(k)
        assert grid.nblk[0] == 15
        O.flux_div_blocks(grid, s, boxes, q, r, increment=bool(incr))
        assert np.array_equal(r[:, ng:-ng, ng:-ng, ng:-ng], want), k


@pytest.mark.skipif(not REF_SRC, reason="reference sources not present")
def test_refined_dropin_records_match_the_golden():
    """tests/cpp/dropin_amr_record.cc built here against the reference's
    headers and the recording stand-in makes exactly the recorded calls:
    the same descriptors, block boxes and arrays, and the reference's result."""
    import numpy as np
    from golden.gen_golden import read_dropin_blocks_records
    g = np.load(os.path.join(ROOT, "tests", "golden", "dropin_amr_ref.npz"))
    with tempfile.TemporaryDirectory() as d:
        stub, exe = os.path.join(d, "stub.o"), os.path.join(d, "rec")
        subprocess.run(["gcc", "-O1", "-c", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "gbns_record_stub.c"), "-o", stub], check=True)
        subprocess.run(["g++", "-std=c++20", "-O1", "-I" + REF_SRC, "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "oracle", "mpi_stub"), "-I" + CUDA_INC,
                        os.path.join(ROOT, "tests", "cpp", "dropin_amr_record.cc"), stub, "-o", exe], check=True)
        rec, res = os.path.join(d, "calls.bin"), os.path.join(d, "ref.bin")
        subprocess.run([exe, res], check=True, env=dict(os.environ, GBNS_RECORD_BLOCKS=rec))
        calls = read_dropin_blocks_records(rec)
        refs = np.fromfile(res)
    assert len(calls) == 2
    for k, (gb, sb, incr, boxes, q, r) in enumerate(calls):
        grid, s, boxes_g, q_g, r_g, incr_g, ng, want = refined_dropin_call(k)
        assert gb == g["grid%d" % k].tobytes() and sb == g["scheme%d" % k].tobytes() and incr == incr_g
        assert np.array_equal(boxes, boxes_g) and np.array_equal(q, q_g.ravel()) and np.array_equal(r, r_g.ravel())
        ref = refs.reshape(2, *q_g.shape)[k]
        assert np.array_equal(ref[:, ng:-ng, ng:-ng, ng:-ng], want)
