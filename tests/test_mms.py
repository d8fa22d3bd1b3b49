"""Order of accuracy by manufactured solutions, for the features without a
reference implementation (WENO5, Sutherland's law, tanh-stretched y metrics):
a smooth primitive field is sampled at cell centres (ghosts included), the
oracle's flux divergence is compared with the exact -dF/dx of the continuous
flux (complex-step derivatives of closed forms), and the error must fall at
the scheme's order as the grid is refined.  The method follows the
reference's MMS driver (development/mms/main.cc:60-111) with hand-written
derivatives in place of its symbolic library.  CPU only (oracle)."""
import math

import numpy as np
import pytest

from spade_gb300 import _abi
from oracle import oracle as O
import problems as P

G, R, PR = P.GAMMA, P.RGAS, P.PRANDTL
NG = 3


def _field_x(x):
    """p, T, u as functions of x (v = w = 0)."""
    p = 1.0e5 * (1.0 + 0.1 * np.sin(2 * np.pi * x))
    T = 300.0 * (1.0 + 0.05 * np.cos(2 * np.pi * x))
    u = 50.0 * (1.0 + 0.2 * np.sin(2 * np.pi * x + 0.3))
    return p, T, u


def _flux_x(x):
    """Inviscid x-flux in flux_t order (continuity, energy, x-, y-, z-momentum)."""
    p, T, u = _field_x(x)
    rho = p / (R * T)
    E = p / (rho * (G - 1.0)) + 0.5 * u * u
    return [rho * u, u * (rho * E + p), rho * u * u + p]


def _dx(f, x, h=1e-30):
    return [np.imag(c) / h for c in f(x + 1j * h)]


def _errors_x(conv, order, n):
    grid = _abi.grid_desc((1, 1, 1), (n, 2, 2), NG, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    q = np.zeros(P.padded_shape((1, 1, 1), (n, 2, 2), NG))
    x = (np.arange(-NG, n + NG) + 0.5) / n
    p, T, u = _field_x(x)
    q[..., 0] = p[None, None, None, :]
    q[..., 1] = T[None, None, None, :]
    q[..., 2] = u[None, None, None, :]
    r = np.zeros_like(q)
    O.flux_div(grid, P.scheme(conv=conv, order=order), q, r, increment=False)
    xi = x[NG:-NG]
    exact = [-d for d in _dx(_flux_x, xi)]
    num = r[0, NG, NG, NG:-NG, :]
    return max(np.abs(num[:, k] - exact[j]).max() / np.abs(exact[j]).max() for j, k in enumerate((0, 1, 2)))


@pytest.mark.parametrize("conv,order,want", [(_abi.CONV_CENT_KEEP, 2, 1.9), (_abi.CONV_CENT_KEEP, 4, 3.8),
                                             (_abi.CONV_WENO5, 2, 3.5)])
def test_convective_order_identity(conv, order, want):
    e = [_errors_x(conv, order, n) for n in (32, 64, 128)]
    rates = [math.log2(e[i] / e[i + 1]) for i in range(2)]
    assert e[2] < e[1] < e[0]
    assert rates[-1] >= want, (e, rates)


def _field_y(y):
    p = 1.0e5 * (1.0 + 0.05 * np.sin(np.pi * y))
    T = 300.0 * (1.0 + 0.1 * np.cos(np.pi * y))
    u = 80.0 * (1.0 - 0.5 * y * y)
    return p, T, u


def _sutherland(T, mu_ref, T_ref=300.0, S=110.4):
    x = T / T_ref
    return mu_ref * x * np.sqrt(x) * ((T_ref + S) / (T + S))


def _errors_y(n, beta=1.5, mu_ref=2.0):
    grid = _abi.grid_desc((1, 1, 1), (2, n, 2), NG, (0.0, 1.0, -1.0, 1.0, 0.0, 1.0), coords=_abi.COORDS_TANH_Y,
                          coord_param=(beta, 0.0, 0.0, 0.0))
    q = np.zeros(P.padded_shape((1, 1, 1), (2, n, 2), NG))
    eta = -1.0 + (np.arange(-NG, n + NG) + 0.5) * (2.0 / n)
    y = np.tanh(beta * eta) / math.tanh(beta)
    p, T, u = _field_y(y)
    q[..., 0] = p[None, None, :, None]
    q[..., 1] = T[None, None, :, None]
    q[..., 2] = u[None, None, :, None]
    s = P.scheme(conv=_abi.CONV_CENT_KEEP, order=2, visc=1, law=_abi.LAW_SUTHERLAND, mu=mu_ref, T_ref=300.0, S=110.4)
    r = np.zeros_like(q)
    O.flux_div(grid, s, q, r, increment=False)
    cp = G * R / (G - 1.0)

    def flux(yy):
        pp, TT, uu = _field_y(yy)
        # first derivatives of the closed forms (exact for real yy)
        uy = -80.0 * yy
        Ty = -300.0 * 0.1 * np.pi * np.sin(np.pi * yy)
        mu = _sutherland(TT, mu_ref)
        tau_xy = mu * uy
        heat = cp * (mu / PR) * Ty
        return [-(uu * tau_xy + heat), -tau_xy, pp]

    yi = y[NG:-NG]
    d = _dx(flux, yi)
    exact = {1: -d[0], 2: -d[1], 3: -d[2]}
    num = r[0, NG, NG:-NG, NG, :]
    return max(np.abs(num[:, k] - exact[k]).max() / np.abs(exact[k]).max() for k in (1, 2, 3))


def test_viscous_sutherland_stretched_y_second_order():
    e = [_errors_y(n) for n in (16, 32, 64)]
    rates = [math.log2(e[i] / e[i + 1]) for i in range(2)]
    assert e[2] < e[1] < e[0]
    assert rates[-1] >= 1.8, (e, rates)
