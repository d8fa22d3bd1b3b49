"""pde_algs::boundary_flux (pde-algs/boundary_flux.h:16-105).

The reference's boundary_flux does not compile against its current grid
headers, so its semantics are pinned here by construction on the oracle's
restatement (CPU): on a uniform state every face carries the analytic Euler
flux, and the operator must add exactly -F/dx to the cell inside each selected
boundary face and +F/dx to the ghost cell beyond it, over the boundary plane's
transverse index range [-1, n), only on blocks that lie on that boundary.
The GPU kernel is compared with the restatement bit for bit
(tests/test_gpu_parity.py)."""
import numpy as np
import pytest

from spade_gb300 import _abi, pde_algs
from oracle import oracle as O
import problems as P

NG = 3


def _uniform(nblk, ncell, p=9.0e4, T=310.0, u=(31.0, -12.0, 7.5)):
    q = np.zeros(P.padded_shape(nblk, ncell, NG))
    q[..., 0], q[..., 1] = p, T
    q[..., 2], q[..., 3], q[..., 4] = u
    return q


def _euler_flux(d, p=9.0e4, T=310.0, u=(31.0, -12.0, 7.5)):
    rho = p / (P.RGAS * T)
    ke = 0.5 * (u[0] ** 2 + u[1] ** 2 + u[2] ** 2)
    E = p / (rho * (P.GAMMA - 1.0)) + ke
    un = u[d]
    mom = [rho * un * u[k] + (p if k == d else 0.0) for k in range(3)]
    return np.array([rho * un, un * (rho * E + p)] + mom)


@pytest.mark.parametrize("d,side", [(0, 0), (0, 1), (1, 0), (1, 1), (2, 0), (2, 1)])
def test_uniform_state_adds_the_euler_flux_on_the_selected_plane(d, side):
    nblk, ncell = (2, 2, 2), (5, 4, 3)
    bounds = (0.0, 2.0, 0.0, 1.0, 0.0, 1.5)
    grid = _abi.grid_desc(nblk, ncell, NG, bounds)
    q = _uniform(nblk, ncell)
    rhs = np.zeros_like(q)
    apply = [0] * 6
    apply[2 * d + side] = 1
    O.boundary_flux(grid, P.scheme(conv=_abi.CONV_CENT_KEEP, order=2), q, rhs, apply)
    F = _euler_flux(d)
    dx = (bounds[2 * d + 1] - bounds[2 * d]) / nblk[d] / ncell[d]
    want = np.zeros_like(q)
    for lb in range(8):
        b = (lb % 2, (lb // 2) % 2, lb // 4)
        if b[d] != (0 if side == 0 else nblk[d] - 1):
            continue
        il = -1 if side == 0 else ncell[d] - 1
        sl_l = [slice(NG - 1, NG + ncell[k]) for k in range(3)]   # transverse [-1, n)
        sl_r = list(sl_l)
        sl_l[d] = slice(NG + il, NG + il + 1)
        sl_r[d] = slice(NG + il + 1, NG + il + 2)
        want[(lb, sl_l[2], sl_l[1], sl_l[0])] -= F / dx
        want[(lb, sl_r[2], sl_r[1], sl_r[0])] += F / dx
    scale = np.abs(F).max() / dx
    assert np.abs(rhs - want).max() <= 1e-13 * scale
    assert np.array_equal(rhs != 0.0, want != 0.0)


def test_apply_flags_follow_bound_box_order():
    bb = pde_algs.bound_box_t(False)
    bb.max(0, True)
    bb.min(2, True)
    assert bb.flags() == [False, True, False, False, True, False]
    assert (~bb).flags() == [True, False, True, True, False, True]


def test_restatement_rejects_stretched_grids_and_thin_halos():
    nblk, ncell = (1, 1, 1), (4, 4, 4)
    q = _uniform(nblk, ncell)
    grid = _abi.grid_desc(nblk, ncell, NG, (0.0, 1.0, -1.0, 1.0, 0.0, 1.0), _abi.COORDS_TANH_Y, (2.0, 0, 0, 0))
    with pytest.raises(Exception):
        O.boundary_flux(grid, P.scheme(), q, np.zeros_like(q), [1] * 6)
    thin = _abi.grid_desc(nblk, ncell, 1, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    q1 = np.zeros(P.padded_shape(nblk, ncell, 1))
    with pytest.raises(Exception):
        O.boundary_flux(thin, P.scheme(visc=1), q1, np.zeros_like(q1), [1] * 6)
