"""The oracle against the reference itself on fresh seeds and ragged grids:
ghost exchange and wall fill (grid/make_exchange.h:98-421,
grid/boundary_fill.h:31-133) over several block layouts and ghost depths, and
short SSPRK3 runs (time-integration/advance.h:234-280) of seven scheme
compositions, periodic and with isothermal walls, all bit for bit.  Runs only
where the reference harness (oracle/_ref) has been built from the reference
sources; the committed golden fixtures cover the same paths elsewhere."""
import numpy as np
import pytest

from spade_gb300 import _abi
from oracle import oracle as O
import problems as P
from golden.gen_golden import FLUX_CASES

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference harness not built here")


def interior(a, ng):
    return a[:, ng:-ng, ng:-ng, ng:-ng, :]

LAYOUTS = [
    ((1, 1, 1), (4, 4, 4), 1),
    ((3, 2, 1), (5, 3, 4), 2),
    ((1, 4, 2), (6, 4, 3), 3),
    ((2, 2, 3), (4, 5, 4), 4),
    ((2, 3, 2), (7, 4, 5), 2),
]


@pytest.mark.parametrize("layout", range(len(LAYOUTS)))
@pytest.mark.parametrize("walls", [False, True])
def test_ghost_fill_live(layout, walls):
    nblk, ncell, ng = LAYOUTS[layout]
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.1, -1.0, 1.0, 0.0, 0.8))
    bc = P.channel_bc(287.5) if walls else P.periodic_bc()
    q = P.random_state(nblk, ncell, ng, seed=300 + layout)
    a = q.copy()
    b = q.copy()
    O.ref_fill_ghosts(grid, P.scheme(), bc, a)
    O.fill_ghosts(grid, bc, b)
    assert np.array_equal(a, b)


SSP_CASES = ["ck2_visc", "totani_visc", "ck4_visc", "fweno_diss_visc", "fweno_ducros_visc",
             "hyb_ck4_diss_visc", "hyb_ck2_const_ducros_diss_visc"]


@pytest.mark.parametrize("name", SSP_CASES)
@pytest.mark.parametrize("walls", [False, True])
def test_ssprk3_live(name, walls):
    rid, kw = FLUX_CASES[name]
    nblk, ncell, ng = (2, 1, 2), (8, 4, 4), 3   # the reference's transform_inplace wants multiples of 4
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.3, -1.0, 1.0, 0.0, 0.7))
    bc = P.channel_bc(300.0) if walls else P.periodic_bc()
    s = P.scheme(**kw)
    q = P.random_state(nblk, ncell, ng, seed=400 + SSP_CASES.index(name))
    O.fill_ghosts(grid, bc, q)
    dt = 2e-7
    a = q.copy()
    ke = O.ref_ssprk3(rid, grid, s, bc, a, dt, 3)
    b = q.copy()
    work = np.zeros((3,) + q.shape)
    ke_o = [O.reduce(grid, P.gas_desc(), b, _abi.RED_KINETIC)]
    for _ in range(3):
        O.ssprk3_step(grid, s, bc, b, work, dt)
        ke_o.append(O.reduce(grid, P.gas_desc(), b, _abi.RED_KINETIC))
    assert np.all(np.isfinite(a))
    assert np.array_equal(interior(a, ng), interior(b, ng))
    assert not np.array_equal(interior(a, ng), interior(q, ng))
    np.testing.assert_allclose(ke_o, ke, rtol=1e-13)
