"""The CPU oracle (oracle/gbns_oracle.c) against the reference's own outputs
(tests/golden/, made by tests/golden/gen_golden.py from the reference's CPU
path) — the oracle must reproduce them bit for bit."""
import math
import os

import numpy as np
import pytest

from spade_gb300 import _abi
from oracle import oracle as O
import problems as P

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
from golden.gen_golden import FLUX_CASES, FLUX_GRID, GHOST_GRID  # noqa: E402


def load(name):
    return np.load(os.path.join(GOLD, name))


def interior(a, ng):
    return a[:, ng:-ng, ng:-ng, ng:-ng, :]


@pytest.mark.parametrize("name", sorted(FLUX_CASES))
def test_flux_div_matches_reference_bitwise(name):
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    q = g["q"]
    r = np.zeros_like(q)
    O.flux_div(grid, P.scheme(**FLUX_CASES[name][1]), q, r, increment=False)
    assert np.array_equal(interior(r, fg["ng"]), g["rhs_" + name])


def test_flux_div_increment_mode_bitwise():
    g = load("flux_div_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    r = g["rhs0_increment"].copy()
    O.flux_div(grid, P.scheme(conv=_abi.CONV_CENT_KEEP, order=2, visc=1), g["q"], r, increment=True)
    assert np.array_equal(interior(r, fg["ng"]), g["rhs_increment_ck2_visc"])


def test_ghost_fill_matches_reference_bitwise():
    g = load("ghosts_ref.npz")
    gg = GHOST_GRID
    grid = _abi.grid_desc(gg["nblk"], gg["ncell"], gg["ng"], gg["bounds"])
    a = g["q"].copy()
    O.fill_ghosts(grid, P.periodic_bc(), a)
    assert np.array_equal(a, g["periodic"])
    b = g["q"].copy()
    O.fill_ghosts(grid, P.channel_bc(290.0), b)
    assert np.array_equal(b, g["walls"])


def test_tgv_small_20_steps_bitwise():
    g = load("tgv_small_ref.npz")
    nblk, ncell, ng = (2, 2, 2), (8, 8, 8), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    tables = {k[4:]: g[k] for k in g.files if k.startswith("tab_")}
    q = P.tgv_state(nblk, ncell, ng, tables, seed=3)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    dt = float(g["dt"])
    assert dt == P.tgv_dt(q, grid, ng)
    work = np.zeros((3,) + q.shape)
    ke = [O.reduce(grid, P.gas_desc(), q, _abi.RED_KINETIC)]
    for _ in range(10):
        O.ssprk3_step(grid, P.tgv_scheme(), P.periodic_bc(), q, work, dt)
        ke.append(O.reduce(grid, P.gas_desc(), q, _abi.RED_KINETIC))
    assert np.array_equal(interior(q, ng), g["q_final"])
    np.testing.assert_allclose(ke, g["ke"], rtol=1e-13)


def test_channel_walls_fweno_5_steps_bitwise():
    g = load("channel_ref.npz")
    nblk, ncell, ng = (2, 2, 2), (8, 8, 8), 3
    bounds = (0.0, 4 * math.pi, -1.0, 1.0, 0.0, 4 * math.pi / 3)
    grid = _abi.grid_desc(nblk, ncell, ng, bounds)
    c_w = math.sqrt(P.GAMMA * P.RGAS * 300.0)
    s = P.scheme(conv=_abi.CONV_FWENO, diss=1, visc=1, mu=float(g["mu"]), eps_p=float(g["eps"]), eps_T=float(g["eps"]), alpha=1.0)
    q = g["q0"].copy()
    work = np.zeros((3,) + q.shape)
    for _ in range(5):
        O.ssprk3_step(grid, s, P.channel_bc(300.0), q, work, float(g["dt"]))
    assert np.array_equal(interior(q, ng), g["q_final"])


def test_tgv_c1_flux_and_ke_history():
    """C1 (2x2x2 x 16^3, ng=2): one flux_div and 20 SSPRK3 steps."""
    g = load("tgv_ref.npz")
    nblk, ncell, ng = (2, 2, 2), (16, 16, 16), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    tables = {k[4:]: g[k] for k in g.files if k.startswith("tab_")}
    q = P.tgv_state(nblk, ncell, ng, tables, seed=0)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    r = np.zeros_like(q)
    O.flux_div(grid, P.tgv_scheme(), q, r, increment=False, nthreads=0)
    ri = interior(r, ng)
    assert np.array_equal(ri[:, ::5, ::5, ::5, :], g["rhs_probe"])
    np.testing.assert_allclose(ri.reshape(-1, 5).sum(axis=0), g["rhs_sum"], rtol=0, atol=1e-9 * np.abs(g["rhs_abs"]).max())


@pytest.mark.skipif(not O.ref_available(), reason="reference harness not built here")
def test_oracle_against_live_reference_random_states():
    """Fresh seeds, live reference (only where the reference sources exist)."""
    nblk, ncell, ng = (3, 2, 1), (5, 4, 6), 3
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 2.0, 0.0, 1.0, 0.0, 3.0))
    for seed in (101, 102):
        q = P.random_state(nblk, ncell, ng, seed=seed)
        for name, (rid, kw) in FLUX_CASES.items():
            if kw.get("order", 2) > 6:
                continue
            s = P.scheme(**kw)
            a = np.zeros_like(q)
            b = np.zeros_like(q)
            O.ref_flux_div(rid, grid, s, q, a, increment=False)
            O.flux_div(grid, s, q, b, increment=False)
            assert np.array_equal(a, b), name


@pytest.mark.parametrize("kind", [_abi.SOURCE_CONST, _abi.SOURCE_BODY_FORCE, _abi.SOURCE_BODY_ACCEL])
def test_source_term_matches_reference_bitwise(kind):
    from golden.gen_golden import source_desc
    g = load("source_ref.npz")
    fg = FLUX_GRID
    grid = _abi.grid_desc(fg["nblk"], fg["ncell"], fg["ng"], fg["bounds"])
    q = P.random_state(fg["nblk"], fg["ncell"], fg["ng"], seed=11)
    r = g["rhs0"].copy()
    O.source_term(grid, source_desc(kind), q, r)
    assert np.array_equal(r, g["rhs_%d" % kind])
