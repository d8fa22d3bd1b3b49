"""Generates the golden fixtures in tests/golden/ from the REFERENCE's own CPU
path (oracle/_ref/libspade_ref.so, built by `make -C oracle ref` where the
reference sources exist).  Run from the repository root:

    python tests/golden/gen_golden.py

Fixtures hold inputs (or the 1-D tables and seeds that rebuild them
bit-exactly, tests/problems.py) and the reference's outputs.
"""
import hashlib
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

from spade_gb300 import _abi  # noqa: E402
from oracle import oracle as O  # noqa: E402
import problems as P  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))

# (reference harness scheme id, scheme kwargs for tests/problems.scheme)
FLUX_CASES = {
    "ck2_visc": (O.REF_CK2_VISC, dict(conv=_abi.CONV_CENT_KEEP, order=2, visc=1)),
    "totani_visc": (O.REF_TOTANI_VISC, dict(conv=_abi.CONV_TOTANI, visc=1)),
    "ck4_visc": (O.REF_CK4_VISC, dict(conv=_abi.CONV_CENT_KEEP, order=4, visc=1)),
    "ck2": (O.REF_CK2, dict(conv=_abi.CONV_CENT_KEEP, order=2)),
    "visc": (O.REF_VISC, dict(conv=_abi.CONV_NONE, visc=1)),
    "fweno_diss_visc": (O.REF_FWENO_DISS_VISC, dict(conv=_abi.CONV_FWENO, diss=1, visc=1)),
    "fweno": (O.REF_FWENO, dict(conv=_abi.CONV_FWENO)),
    "diss": (O.REF_DISS, dict(conv=_abi.CONV_NONE, diss=1)),
    "totani": (O.REF_TOTANI, dict(conv=_abi.CONV_TOTANI)),
    "ck6": (O.REF_CK6, dict(conv=_abi.CONV_CENT_KEEP, order=6)),
    "ck8": (O.REF_CK8, dict(conv=_abi.CONV_CENT_KEEP, order=8)),
    "fweno_nosmooth": (O.REF_FWENO_NOSMOOTH, dict(conv=_abi.CONV_FWENO, smooth=0)),
    "ck2_diss_visc": (O.REF_CK2_DISS_VISC, dict(conv=_abi.CONV_CENT_KEEP, order=2, diss=1, visc=1)),
    "ducros_diss": (O.REF_DUCROS_DISS, dict(conv=_abi.CONV_NONE, diss=1, sensor=_abi.SENSOR_DUCROS, alpha=0.7)),
    "fweno_ducros_visc": (O.REF_FWENO_DUCROS_VISC, dict(conv=_abi.CONV_FWENO, diss=1, visc=1,
                                                         sensor=_abi.SENSOR_DUCROS, alpha=0.7)),
    "hyb_ck2_full": (O.REF_HYB_CK2_FULL, dict(conv=_abi.CONV_HYBRID, order=2, hybrid_flux=_abi.HYBRID_FULL_FLUX,
                                               hybrid_sensor=_abi.SENSOR_DUCROS, hybrid_param=0.5)),
    "hyb_ck4_diss_visc": (O.REF_HYB_CK4_DISS_VISC, dict(conv=_abi.CONV_HYBRID, order=4, visc=1,
                                                         hybrid_flux=_abi.HYBRID_DISS_FLUX,
                                                         hybrid_sensor=_abi.SENSOR_DUCROS, hybrid_param=0.5)),
    "hyb_ck2_const_ducros_diss_visc": (O.REF_HYB_CK2_CONST_DISS_VISC,
                                       dict(conv=_abi.CONV_HYBRID, order=2, diss=1, visc=1, sensor=_abi.SENSOR_DUCROS,
                                            alpha=0.7, hybrid_flux=_abi.HYBRID_FULL_FLUX,
                                            hybrid_sensor=_abi.SENSOR_CONST, hybrid_param=0.3)),
}

FLUX_GRID = dict(nblk=(2, 1, 1), ncell=(6, 5, 4), ng=4, bounds=(0.0, 1.3, 0.0, 0.9, 0.0, 0.7))
GHOST_GRID = dict(nblk=(2, 3, 2), ncell=(4, 3, 5), ng=2, bounds=(0.0, 1.0, -1.0, 1.0, 0.0, 2.0))


def interior(a, ng):
    return a[:, ng:-ng, ng:-ng, ng:-ng, :]


def gen_flux():
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    q = P.random_state(fg["nblk"], fg["ncell"], fg["ng"], seed=11)
    out = {"q": q}
    for name, (rid, kw) in FLUX_CASES.items():
        s = P.scheme(**kw)
        r = np.zeros_like(q)
        O.ref_flux_div(rid, grid, s, q, r, increment=False)
        out["rhs_" + name] = interior(r, fg["ng"]).copy()
    # increment mode on a nonzero residual
    r0 = P.random_state(fg["nblk"], fg["ncell"], fg["ng"], seed=12, p0=1.0, T0=1.0, u0=1.0)
    r = r0.copy()
    O.ref_flux_div(O.REF_CK2_VISC, grid, P.scheme(conv=_abi.CONV_CENT_KEEP, order=2, visc=1), q, r, increment=True)
    out["rhs0_increment"] = r0
    out["rhs_increment_ck2_visc"] = interior(r, fg["ng"]).copy()
    np.savez_compressed(os.path.join(OUT, "flux_div_ref.npz"), **out)


SOURCE_C = (0.25, -1.5, 3.0, -0.75, 1.25)


def source_desc(kind):
    src = _abi.SourceDesc()
    src.kind = kind
    for v, x in enumerate(SOURCE_C):
        src.c[v] = x
    src.gas.gamma = P.GAMMA
    src.gas.R = P.RGAS
    return src


def gen_source():
    # pde_algs::source_term with the three lowered point-source forms
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    q = P.random_state(fg["nblk"], fg["ncell"], fg["ng"], seed=11)
    r0 = P.random_state(fg["nblk"], fg["ncell"], fg["ng"], seed=13, p0=1.0, T0=1.0, u0=1.0)
    out = {"rhs0": r0}
    for kind in (_abi.SOURCE_CONST, _abi.SOURCE_BODY_FORCE, _abi.SOURCE_BODY_ACCEL):
        r = r0.copy()
        O.ref_source_term(grid, P.scheme(), source_desc(kind), q, r)
        out["rhs_%d" % kind] = r
    np.savez_compressed(os.path.join(OUT, "source_ref.npz"), **out)


def gen_ghosts():
    gg = GHOST_GRID
    grid = _abi.grid_desc(gg["nblk"], gg["ncell"], gg["ng"], gg["bounds"])
    q = P.random_state(gg["nblk"], gg["ncell"], gg["ng"], seed=21)
    s = P.scheme()
    a = q.copy()
    O.ref_fill_ghosts(grid, s, P.periodic_bc(), a)
    b = q.copy()
    O.ref_fill_ghosts(grid, s, P.channel_bc(290.0), b)
    np.savez_compressed(os.path.join(OUT, "ghosts_ref.npz"), q=q, periodic=a, walls=b)


def gen_tgv():
    # C1: 2x2x2 blocks of 16^3, ng = 2, cent_keep<2> + visc_lr(constant), 20 SSPRK3 steps
    nblk, ncell, ng = (2, 2, 2), (16, 16, 16), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    tables = P.tgv_tables(nblk, ncell, ng)
    q = P.tgv_state(nblk, ncell, ng, tables, seed=0)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    dt = P.tgv_dt(q, grid, ng)
    s = P.tgv_scheme()
    r = np.zeros_like(q)
    O.ref_flux_div(O.REF_CK2_VISC, grid, s, q, r, increment=False)
    rin = interior(r, ng)
    qf = q.copy()
    ke = O.ref_ssprk3(O.REF_CK2_VISC, grid, s, P.periodic_bc(), qf, dt, 20)
    qi = interior(qf, ng)
    np.savez_compressed(os.path.join(OUT, "tgv_ref.npz"), dt=dt, ke=ke,
                        rhs_sum=rin.reshape(-1, 5).sum(axis=0), rhs_abs=np.abs(rin).reshape(-1, 5).sum(axis=0),
                        rhs_probe=rin[:, ::5, ::5, ::5, :].copy(),
                        q_sum=qi.reshape(-1, 5).sum(axis=0), q_probe=qi[:, ::3, ::3, ::3, :].copy(),
                        **{"tab_" + k: v for k, v in tables.items()})
    # a smaller TGV whose whole final state is stored
    nblk, ncell, ng = (2, 2, 2), (8, 8, 8), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    tables = P.tgv_tables(nblk, ncell, ng)
    q = P.tgv_state(nblk, ncell, ng, tables, seed=3)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    dt = P.tgv_dt(q, grid, ng)
    qf = q.copy()
    ke = O.ref_ssprk3(O.REF_CK2_VISC, grid, s, P.periodic_bc(), qf, dt, 10)
    np.savez_compressed(os.path.join(OUT, "tgv_small_ref.npz"), dt=dt, ke=ke, q_final=interior(qf, ng).copy(),
                        **{"tab_" + k: v for k, v in tables.items()})


def gen_channel():
    # uniform-grid channel subset the reference can run: fweno_t +
    # pressure_diss_lr(const_sensor) + visc_lr(constant), isothermal walls
    nblk, ncell, ng = (2, 2, 2), (8, 8, 8), 3
    bounds = (0.0, 4 * math.pi, -1.0, 1.0, 0.0, 4 * math.pi / 3)
    grid = _abi.grid_desc(nblk, ncell, ng, bounds)
    c_w = math.sqrt(P.GAMMA * P.RGAS * 300.0)
    U_b = 0.5 * c_w
    y = P.cell_centres(nblk, ncell, ng, bounds, 1)[:, None, :, None]
    q = np.empty(P.padded_shape(nblk, ncell, ng))
    q[..., 0] = P.RGAS * 300.0
    q[..., 1] = 300.0
    q[..., 2] = 1.5 * U_b * (1.0 - y * y)
    q[..., 3] = 0.0
    q[..., 4] = 0.0
    r = np.random.Generator(np.random.PCG64(5))
    inner = q[:, ng:-ng, ng:-ng, ng:-ng, 2:5]
    inner += r.standard_normal(inner.shape) * (0.05 * U_b)
    bc = P.channel_bc(300.0)
    O.fill_ghosts(grid, bc, q)
    s = P.scheme(conv=_abi.CONV_FWENO, diss=1, visc=1, mu=U_b / 3000.0, eps_p=0.01 * c_w, eps_T=0.01 * c_w, alpha=1.0)
    a = q[:, ng:-ng, ng:-ng, ng:-ng, :]
    amax = float((np.sqrt(P.GAMMA * P.RGAS * a[..., 1]) + np.sqrt((a[..., 2:] ** 2).sum(-1))).max())
    dt = 0.5 * min(4 * math.pi / 16, 2.0 / 16, (4 * math.pi / 3) / 16) / amax
    qf = q.copy()
    ke = O.ref_ssprk3(O.REF_FWENO_DISS_VISC, grid, s, bc, qf, dt, 5)
    assert np.all(np.isfinite(qf)) and np.all(np.isfinite(ke))
    np.savez_compressed(os.path.join(OUT, "channel_ref.npz"), q0=q, dt=dt, ke=ke, q_final=interior(qf, ng).copy(),
                        mu=U_b / 3000.0, eps=0.01 * c_w)


# AMR layouts refined in place (cartesian_grid_t::refine_blocks), one refinement
# pass per inner list of global block indices: (base blocks, cells per block,
# ghosts, periodic flags, passes)
AMR_CASES = {
    "one_level_periodic": ((2, 2, 2), (4, 4, 4), 2, (1, 1, 1), [[0]]),
    "two_levels_walls_y": ((2, 2, 2), (4, 4, 4), 3, (1, 0, 1), [[0], [0]]),
    "anisotropic_blocks": ((2, 2, 1), (8, 4, 4), 2, (1, 1, 1), [[0, 3]]),
}


def amr_fill(boxes, ncell, ng):
    """The harness's interior field at cell centres (exact in binary floating
    point for these power-of-two boxes), ghosts 0."""
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


def gen_amr():
    out = {}
    for name, (nb, nc, ng, per, passes) in AMR_CASES.items():
        r = O.ref_amr_exchange(nb, nc, ng, per, passes)
        before = amr_fill(r["boxes"], nc, ng)
        assert np.array_equal(before, r["before"]), name        # the fill is rebuilt exactly
        out[name + "_plan"] = r["plan"]
        out[name + "_ninject"] = np.int32(r["ninject"])
        out[name + "_boxes"] = r["boxes"]
        out[name + "_levels"] = r["levels"]
        out[name + "_after"] = r["after"]
        out[name + "_ncell"] = np.array(nc, dtype=np.int32)
        out[name + "_ng"] = np.int32(ng)
    np.savez_compressed(os.path.join(OUT, "amr_ref.npz"), **out)


# flux_div on the refined layouts of AMR_CASES, the reference's own
# (pde_algs::flux_div, overwrite mode, each block's 1/dx from its own box) on
# the exchanged array, with ghost cells the exchange leaves at 0 (walls, not
# filled by it) set to a valid state first: (reference scheme id, scheme fields)
AMR_FLUX_SCHEMES = {
    "ck2_visc": (O.REF_CK2_VISC, dict(conv=_abi.CONV_CENT_KEEP, visc=1)),
    "fweno_diss_visc": (O.REF_FWENO_DISS_VISC, dict(conv=_abi.CONV_FWENO, diss=1, visc=1)),
}


AMR_SSPRK3_DT, AMR_SSPRK3_STEPS = 1e-4, 3
AMR_T_WALL = 1.25


def amr_flux_input(after):
    q = after.copy()
    hole = q[..., 1] == 0.0
    q[hole] = (3.0, 1.0, 0.0, 0.0, 0.0)
    return q


def gen_amr_flux():
    g = np.load(os.path.join(OUT, "amr_ref.npz"))
    out = {}
    for name, (nb, nc, ng, per, passes) in AMR_CASES.items():
        q = amr_flux_input(g[name + "_after"])
        for sname, (sid, kw) in AMR_FLUX_SCHEMES.items():
            rhs = O.ref_amr_flux_div(sid, nb, nc, ng, per, passes, P.scheme(**kw), q)
            inner = rhs[:, ng:-ng, ng:-ng, ng:-ng]
            assert np.all(np.isfinite(inner)), (name, sname)
            out[name + "_" + sname] = inner.copy()
            # AMR_SSPRK3_STEPS of the reference's SSPRK3 with the exchange as
            # boundary condition: the SHA-256 of the final interior's bytes
            a = q.copy()
            O.ref_amr_ssprk3(sid, nb, nc, ng, per, passes, P.scheme(**kw), a, AMR_SSPRK3_DT, AMR_SSPRK3_STEPS)
            inner = np.ascontiguousarray(a[:, ng:-ng, ng:-ng, ng:-ng])
            assert np.all(np.isfinite(inner)), (name, sname)
            out[name + "_ssprk3_" + sname] = np.frombuffer(hashlib.sha256(inner.tobytes()).digest(), dtype=np.uint8)
            if not all(per):
                # the same with the non-periodic y faces as isothermal walls at
                # AMR_T_WALL, filled after each exchange (boundary_fill)
                a = q.copy()
                O.ref_amr_ssprk3(sid, nb, nc, ng, per, passes, P.scheme(**kw), a, AMR_SSPRK3_DT, AMR_SSPRK3_STEPS,
                                 t_wall=AMR_T_WALL)
                inner = np.ascontiguousarray(a[:, ng:-ng, ng:-ng, ng:-ng])
                assert np.all(np.isfinite(inner)), (name, sname)
                out[name + "_ssprk3_walls_" + sname] = np.frombuffer(hashlib.sha256(inner.tobytes()).digest(),
                                                                     dtype=np.uint8)
    np.savez_compressed(os.path.join(OUT, "amr_flux_ref.npz"), **out)


def read_dropin_records(path):
    """Parses the calls tests/cpp/gbns_record_stub.c recorded."""
    import struct
    d = open(path, "rb").read()
    i, out = 0, []
    while i < len(d):
        gs = struct.unpack_from("<Q", d, i)[0]; i += 8
        gb = d[i:i + gs]; i += gs
        ss = struct.unpack_from("<Q", d, i)[0]; i += 8
        sb = d[i:i + ss]; i += ss
        incr = struct.unpack_from("<i", d, i)[0]; i += 4
        n = struct.unpack_from("<Q", d, i)[0]; i += 8
        q = np.frombuffer(d, dtype=np.float64, count=n, offset=i).copy(); i += 8 * n
        r = np.frombuffer(d, dtype=np.float64, count=n, offset=i).copy(); i += 8 * n
        out.append((gb, sb, incr, q, r))
    return out


def gen_dropin():
    """Runs the C++ drop-in at a SPADE call site with no test hook
    (tests/cpp/dropin_record.cc), linked with the recording stand-in for
    libgbns.so, and stores the C-ABI calls it made with the reference's own
    CPU results for the two schemes the reference runs."""
    import subprocess
    import tempfile
    from __graft_entry__ import ref_src
    src = ref_src()
    with tempfile.TemporaryDirectory() as d:
        stub = os.path.join(d, "stub.o")
        exe = os.path.join(d, "dropin_record")
        subprocess.run(["gcc", "-O1", "-c", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "gbns_record_stub.c"), "-o", stub], check=True)
        subprocess.run(["g++", "-std=c++20", "-O1", "-I" + src, "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "oracle", "mpi_stub"), "-I/usr/local/cuda/include",
                        os.path.join(ROOT, "tests", "cpp", "dropin_record.cc"), stub, "-o", exe], check=True)
        rec, res = os.path.join(d, "calls.bin"), os.path.join(d, "ref.bin")
        subprocess.run([exe, res], check=True, env=dict(os.environ, GBNS_RECORD=rec))
        calls = read_dropin_records(rec)
        refs = np.fromfile(res)
    assert len(calls) == 3
    n = calls[0][3].size
    out = {"q": calls[0][3], "ref": refs.reshape(2, n)}
    for k, (gb, sb, incr, q, r) in enumerate(calls):
        assert np.array_equal(q, calls[0][3])              # one state for all three calls
        out["grid%d" % k] = np.frombuffer(gb, dtype=np.uint8)
        out["scheme%d" % k] = np.frombuffer(sb, dtype=np.uint8)
        out["incr%d" % k] = np.int32(incr)
        out["rhs_in%d" % k] = r
    np.savez_compressed(os.path.join(OUT, "dropin_ref.npz"), **out)


def dropin_noise_state(n):
    """The seeded state of tests/cpp/dropin_amr_record.cc over n doubles
    (splitmix64 noise per index; the same operations in the same order)."""
    i = np.arange(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        k = i + np.uint64(0x9E3779B97F4A7C15)
        k = (k ^ (k >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        k = (k ^ (k >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        k = k ^ (k >> np.uint64(31))
    nz = (k >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0) - 0.5
    q = np.empty(n)
    q[0::5] = 1.0e5 * (1.0 + 0.02 * nz[0::5])
    q[1::5] = 300.0 * (1.0 + 0.02 * nz[1::5])
    q[2::5] = 30.0 * nz[2::5]
    q[3::5] = 30.0 * nz[3::5]
    q[4::5] = 30.0 * nz[4::5]
    return q


def read_dropin_blocks_records(path):
    """Parses the gbns_flux_div_blocks_host calls the stand-in recorded."""
    import struct
    d = open(path, "rb").read()
    pos, out = 0, []
    while pos < len(d):
        gs = struct.unpack_from("<Q", d, pos)[0]; pos += 8
        gb = d[pos:pos + gs]; pos += gs
        ss = struct.unpack_from("<Q", d, pos)[0]; pos += 8
        sb = d[pos:pos + ss]; pos += ss
        incr = struct.unpack_from("<i", d, pos)[0]; pos += 4
        nb = struct.unpack_from("<Q", d, pos)[0]; pos += 8
        boxes = np.frombuffer(d, dtype=np.float64, count=6 * nb, offset=pos).reshape(nb, 6).copy(); pos += 48 * nb
        n = struct.unpack_from("<Q", d, pos)[0]; pos += 8
        q = np.frombuffer(d, dtype=np.float64, count=n, offset=pos).copy(); pos += 8 * n
        r = np.frombuffer(d, dtype=np.float64, count=n, offset=pos).copy(); pos += 8 * n
        out.append((gb, sb, incr, boxes, q, r))
    return out


def gen_dropin_amr():
    """The C++ drop-in on a refined grid (tests/cpp/dropin_amr_record.cc),
    linked with the recording stand-in: the lowered gbns_flux_div_blocks_host
    calls (descriptors, boxes) and the reference's own flux_div interiors.
    The state is rebuilt by the tests from the seeded noise and the
    reference's exchange plan of the same layout (AMR_CASES
    one_level_periodic); checked here against the recorded arrays."""
    import subprocess
    import tempfile
    from __graft_entry__ import ref_src
    src = ref_src()
    with tempfile.TemporaryDirectory() as d:
        stub = os.path.join(d, "stub.o")
        exe = os.path.join(d, "dropin_amr_record")
        subprocess.run(["gcc", "-O1", "-c", "-I" + os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "gbns_record_stub.c"), "-o", stub], check=True)
        subprocess.run(["g++", "-std=c++20", "-O1", "-I" + src, "-I" + os.path.join(ROOT, "include"),
                        "-I" + os.path.join(ROOT, "oracle", "mpi_stub"), "-I/usr/local/cuda/include",
                        os.path.join(ROOT, "tests", "cpp", "dropin_amr_record.cc"), stub, "-o", exe], check=True)
        rec, res = os.path.join(d, "calls.bin"), os.path.join(d, "ref.bin")
        subprocess.run([exe, res], check=True, env=dict(os.environ, GBNS_RECORD_BLOCKS=rec))
        calls = read_dropin_blocks_records(rec)
        refs = np.fromfile(res)
    assert len(calls) == 2
    amr = np.load(os.path.join(OUT, "amr_ref.npz"))
    nb, nc, ng, per, passes = AMR_CASES["one_level_periodic"]
    q = dropin_noise_state(calls[0][4].size).reshape(-1, nc[2] + 2 * ng, nc[1] + 2 * ng, nc[0] + 2 * ng, 5)
    O.exchange_patches(nc, ng, q.shape[0], amr["one_level_periodic_plan"], q)
    refs = refs.reshape(2, *q.shape)
    out = {}
    for k, (gb, sb, incr, boxes, qr, r) in enumerate(calls):
        assert np.array_equal(qr, q.ravel())                   # the state is rebuilt exactly
        assert np.array_equal(boxes, amr["one_level_periodic_boxes"])
        assert np.all(r == (0.0 if k == 0 else 0.25))
        out["grid%d" % k] = np.frombuffer(gb, dtype=np.uint8)
        out["scheme%d" % k] = np.frombuffer(sb, dtype=np.uint8)
        out["incr%d" % k] = np.int32(incr)
        out["rhs_fill%d" % k] = np.float64(0.0 if k == 0 else 0.25)
        out["ref%d" % k] = refs[k][:, ng:-ng, ng:-ng, ng:-ng].copy()
    np.savez_compressed(os.path.join(OUT, "dropin_amr_ref.npz"), **out)


if __name__ == "__main__":
    if not O.ref_available():
        sys.exit("reference harness not built: make -C oracle ref")
    gen_flux()
    gen_source()
    gen_ghosts()
    gen_tgv()
    gen_channel()
    gen_amr()
    gen_amr_flux()
    gen_dropin()
    gen_dropin_amr()
    for f in sorted(os.listdir(OUT)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(OUT, f)))
