"""Axis-permutation and mirror symmetry on the oracle (CPU): on a cubic
periodic grid, permuting the coordinate axes cyclically (x <- y <- z <- x, with the velocity
and momentum components permuted alike) permutes the residual the same way.
Only the order in which the three directions are accumulated changes, so the
results agree to round-off.  This checks that every functor treats the three
directions alike (stencils, face normals, transverse gradient terms), which
the bitwise comparisons with the reference on fixed inputs do not by
themselves.  Reflecting one axis checks that the upwind-biased left and right
states mirror each other."""
import numpy as np
import pytest

from spade_gb300 import _abi
from oracle import oracle as O
import problems as P

CASES = {
    "ck4_visc": dict(conv=_abi.CONV_CENT_KEEP, order=4, visc=1),
    "totani_diss": dict(conv=_abi.CONV_TOTANI, diss=1),
    "fweno_ducros_visc": dict(conv=_abi.CONV_FWENO, diss=1, visc=1, sensor=_abi.SENSOR_DUCROS, alpha=0.7),
    "weno5_diss_suth": dict(conv=_abi.CONV_WENO5, diss=1, visc=1, law=_abi.LAW_SUTHERLAND),
    "hyb_ck4_ducros_visc": dict(conv=_abi.CONV_HYBRID, order=4, visc=1, hybrid_sensor=_abi.SENSOR_DUCROS,
                                hybrid_param=1e-3),
}


def _rot(a):
    """New x = old y, new y = old z, new z = old x (array axes are z, y, x),
    and the vector components (slots 2, 3, 4) follow."""
    b = np.ascontiguousarray(np.transpose(a, (0, 3, 1, 2, 4)))
    return np.ascontiguousarray(b[..., [0, 1, 3, 4, 2]])


@pytest.mark.parametrize("name", sorted(CASES))
def test_cyclic_axis_permutation(name):
    n, ng = 6, 3
    grid = _abi.grid_desc((1, 1, 1), (n, n, n), ng, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    q = P.random_state((1, 1, 1), (n, n, n), ng, seed=67)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    s = P.scheme(**CASES[name])
    r = np.zeros_like(q)
    O.flux_div(grid, s, q, r, increment=False)
    qr = _rot(q)
    rr = np.zeros_like(qr)
    O.flux_div(grid, s, qr, rr, increment=False)
    a = rr[:, ng:-ng, ng:-ng, ng:-ng, :].reshape(-1, 5)
    b = _rot(r)[:, ng:-ng, ng:-ng, ng:-ng, :].reshape(-1, 5)
    scale = np.abs(b).max(axis=0)
    assert np.all(np.abs(a - b).max(axis=0) <= 1e-12 * scale), np.abs(a - b).max(axis=0) / scale
    # three rotations are the identity
    assert np.array_equal(_rot(_rot(_rot(q))), q)


def _mirror(a, axis, comp):
    """Reflect array axis `axis` (3 = x, 2 = y, 1 = z) and negate the velocity
    or momentum component `comp` (2, 3, 4) normal to the mirror."""
    b = np.ascontiguousarray(np.flip(a, axis=axis))
    b[..., comp] = -b[..., comp]
    return b


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("axis", [1, 2, 3])
def test_mirror_reflection(name, axis):
    """Reflecting one axis (x -> -x with u -> -u) reflects the residual and
    negates its normal momentum component: the upwind-biased stencils of
    fweno_t / WENO5 and their left/right states must mirror each other."""
    comp = {3: 2, 2: 3, 1: 4}[axis]
    n, ng = 6, 3
    grid = _abi.grid_desc((1, 1, 1), (n, n, n), ng, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    q = P.random_state((1, 1, 1), (n, n, n), ng, seed=71 + axis)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    s = P.scheme(**CASES[name])
    r = np.zeros_like(q)
    O.flux_div(grid, s, q, r, increment=False)
    qm = _mirror(q, axis, comp)
    rm = np.zeros_like(qm)
    O.flux_div(grid, s, qm, rm, increment=False)
    a = rm[:, ng:-ng, ng:-ng, ng:-ng, :].reshape(-1, 5)
    b = _mirror(r, axis, comp)[:, ng:-ng, ng:-ng, ng:-ng, :].reshape(-1, 5)
    scale = np.abs(b).max(axis=0)
    assert np.all(np.abs(a - b).max(axis=0) <= 1e-12 * scale), np.abs(a - b).max(axis=0) / scale


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("walls", [False, True])
def test_mirror_y_on_stretched_channel(name, walls):
    """The tanh-stretched y map is symmetric about the channel centre, so the
    y-reflection holds there too, with isothermal no-slip walls at both ends:
    checks the metric terms and the wall ghost fill, which have no reference
    counterpart to compare with bit for bit."""
    n, ng = 6, 3
    grid = _abi.grid_desc((1, 2, 1), (n, n, n), ng, (0.0, 1.0, -1.0, 1.0, 0.0, 1.0),
                          coords=_abi.COORDS_TANH_Y, coord_param=(2.0, 0.0, 0.0, 0.0))
    bc = P.channel_bc(290.0) if walls else P.periodic_bc()
    q = P.random_state((1, 2, 1), (n, n, n), ng, seed=81)
    O.fill_ghosts(grid, bc, q)
    s = P.scheme(**CASES[name])
    r = np.zeros_like(q)
    O.flux_div(grid, s, q, r, increment=False)

    def mirror_y(a):
        # two blocks stacked in y: swap them and reflect each
        b = _mirror(a, 2, 3)
        return np.ascontiguousarray(b[::-1])

    qm = mirror_y(q)
    refill = qm.copy()
    O.fill_ghosts(grid, bc, refill)
    assert np.array_equal(refill, qm)   # the ghost fill commutes with the reflection
    rm = np.zeros_like(qm)
    O.flux_div(grid, s, qm, rm, increment=False)
    a = rm[:, ng:-ng, ng:-ng, ng:-ng, :].reshape(-1, 5)
    b = mirror_y(r)[:, ng:-ng, ng:-ng, ng:-ng, :].reshape(-1, 5)
    scale = np.abs(b).max(axis=0)
    assert np.all(np.abs(a - b).max(axis=0) <= 1e-12 * scale), np.abs(a - b).max(axis=0) / scale
