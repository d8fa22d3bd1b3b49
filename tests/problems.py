"""Seeded numpy inputs shared by the golden-fixture generator and the tests.

Every input here is bit-reproducible across machines: random numbers come
from numpy's PCG64, and the Taylor–Green field is assembled only with IEEE
+,-,* from 1-D sin/cos tables that the fixtures carry.
"""
import math

import numpy as np

from spade_gb300 import _abi

GAMMA, RGAS, PRANDTL = 1.4, 287.0, 0.72


def padded_shape(nblk, ncell, ng):
    return (nblk[0] * nblk[1] * nblk[2], ncell[2] + 2 * ng, ncell[1] + 2 * ng, ncell[0] + 2 * ng, 5)


def random_state(nblk, ncell, ng, seed, p0=86100.0, T0=300.0, u0=34.7, rel=0.02):
    """A smooth-free random primitive state (every cell independent)."""
    r = np.random.Generator(np.random.PCG64(seed))
    shape = padded_shape(nblk, ncell, ng)
    q = np.empty(shape)
    q[..., 0] = p0 * (1.0 + rel * r.standard_normal(shape[:-1]))
    q[..., 1] = T0 * (1.0 + rel * r.standard_normal(shape[:-1]))
    q[..., 2:] = u0 * r.standard_normal(shape[:-1] + (3,))
    return q


def scheme(conv=_abi.CONV_CENT_KEEP, order=2, diss=0, visc=0, smooth=1, law=_abi.LAW_CONSTANT,
           mu=2.17e-2, eps_p=0.3, eps_T=0.2, alpha=0.7, T_ref=300.0, power=0.76, S=110.4,
           precision=_abi.PREC_FP64, gamma=GAMMA, R=RGAS, sensor=_abi.SENSOR_CONST,
           hybrid_flux=_abi.HYBRID_FULL_FLUX, hybrid_sensor=_abi.SENSOR_DUCROS, hybrid_param=0.5):
    """alpha is const_sensor_t's alpha, or ducros_t's epsilon when sensor is
    SENSOR_DUCROS.  hybrid_* describe the blender of a CONV_HYBRID scheme."""
    s = _abi.SchemeDesc()
    s.convective = conv
    s.order = order
    s.weno_smooth = smooth
    s.dissipation = diss
    s.viscous = visc
    s.visc_law = law
    s.precision = precision
    s.mu = mu
    s.prandtl = PRANDTL
    s.eps_p = eps_p
    s.eps_T = eps_T
    s.sensor = sensor
    s.sensor_alpha = alpha
    s.hybrid_flux = hybrid_flux
    s.hybrid_sensor = hybrid_sensor
    s.hybrid_param = hybrid_param
    s.T_ref = T_ref
    s.power = power
    s.S = S
    s.gas.gamma = gamma
    s.gas.R = R
    return s


def gas_desc(gamma=GAMMA, R=RGAS):
    g = _abi.GasDesc()
    g.gamma = gamma
    g.R = R
    return g


# ---- Taylor–Green (development/cuda-tgv/main.cc:107-116) --------------

TGV_T0, TGV_RHO0, TGV_MACH, TGV_RE = 300.0, 1.0, 0.1, 1600.0


def tgv_constants():
    p0 = TGV_RHO0 * RGAS * TGV_T0
    u0 = TGV_MACH * math.sqrt(GAMMA * RGAS * TGV_T0)
    mu = TGV_RHO0 * u0 * 1.0 / TGV_RE
    return p0, u0, mu


def cell_centres(nblk, ncell, ng, bounds, d):
    """Computational cell centres along d per block (ghosts included), with
    the reference's block arithmetic (cartesian_blocks.h:49,69-70)."""
    nb = nblk
    nlb = nb[0] * nb[1] * nb[2]
    idx = np.arange(-ng, ncell[d] + ng, dtype=np.float64)
    out = np.empty((nlb, ncell[d] + 2 * ng))
    for lb in range(nlb):
        b = [lb % nb[0], (lb // nb[0]) % nb[1], lb // (nb[0] * nb[1])][d]
        lo, hi = bounds[2 * d], bounds[2 * d + 1]
        bsize = (hi - lo) / nb[d]
        mn = lo + b * bsize
        dx = ((mn + bsize) - mn) / ncell[d]
        out[lb] = mn + (idx + 0.5) * dx
    return out


def tgv_tables(nblk, ncell, ng):
    """1-D sin/cos tables per block and direction (the only transcendental
    evaluations of the TGV field)."""
    b = (0.0, 2 * math.pi) * 3
    t = {}
    for d, name in enumerate("xyz"):
        x = cell_centres(nblk, ncell, ng, b, d)
        t["sin_" + name] = np.sin(x)
        t["cos_" + name] = np.cos(x)
        t["cos2_" + name] = np.cos(2.0 * x)
    return t


def tgv_state(nblk, ncell, ng, tables, seed=0, noise=1e-3):
    """TGV primitive field (reference driver form, no 1/16 pressure factor)
    plus uniform U(-noise, noise)*u0 velocity noise on interior cells."""
    p0, u0, _ = tgv_constants()
    shape = padded_shape(nblk, ncell, ng)
    q = np.empty(shape)
    sx, cx, c2x = (tables[k][:, None, None, :] for k in ("sin_x", "cos_x", "cos2_x"))
    sy, cy, c2y = (tables[k][:, None, :, None] for k in ("sin_y", "cos_y", "cos2_y"))
    sz, cz, c2z = (tables[k][:, :, None, None] for k in ("sin_z", "cos_z", "cos2_z"))
    q[..., 0] = p0 + TGV_RHO0 * u0 * u0 * (c2x + c2y) * (c2z + 2.0)
    q[..., 1] = TGV_T0
    q[..., 2] = u0 * sx * cy * cz
    q[..., 3] = -u0 * cx * sy * cz
    q[..., 4] = 0.0
    if noise:
        r = np.random.Generator(np.random.PCG64(seed))
        g = ng
        inner = q[:, g:-g, g:-g, g:-g, 2:5]
        inner += r.uniform(-1.0, 1.0, size=inner.shape) * (noise * u0)
    return q


def tgv_scheme(conv=_abi.CONV_CENT_KEEP, precision=_abi.PREC_FP64):
    _, _, mu = tgv_constants()
    return scheme(conv=conv, order=2, visc=1, mu=mu, precision=precision)


def tgv_grid(nblk=(2, 2, 2), ncell=(16, 16, 16), ng=2):
    return _abi.grid_desc(nblk, ncell, ng, (0.0, 2 * math.pi) * 3)


def periodic_bc():
    return _abi.bc_desc([_abi.BC_PERIODIC] * 6)


def channel_bc(t_wall=300.0):
    k = [_abi.BC_PERIODIC, _abi.BC_PERIODIC, _abi.BC_ISOTHERMAL_NOSLIP, _abi.BC_ISOTHERMAL_NOSLIP,
         _abi.BC_PERIODIC, _abi.BC_PERIODIC]
    return _abi.bc_desc(k, [0.0, 0.0, t_wall, t_wall, 0.0, 0.0])


def tgv_dt(q, grid, ng, cfl=0.5):
    """dt = CFL*dx/max(sqrt(gamma R T) + |u|) over the initial interior
    (development/cuda-tgv/main.cc:170-172)."""
    g = ng
    inner = q[:, g:-g, g:-g, g:-g, :]
    a = np.sqrt(GAMMA * RGAS * inner[..., 1]) + np.sqrt(inner[..., 2] ** 2 + inner[..., 3] ** 2 + inner[..., 4] ** 2)
    dx = ((0.0 + 2 * math.pi / grid.nblk[0]) - 0.0) / grid.ncell[0]
    return cfl * dx / float(a.max())


def rel_err(a, b, floor_frac=1e-6):
    """Per-cell, per-variable relative error |a-b| / max(|b|, floor) where the
    floor is floor_frac times the variable's largest magnitude (guards cells
    whose exact value is ~0 by symmetry)."""
    b = np.asarray(b)
    scale = np.abs(b).reshape(-1, b.shape[-1]).max(axis=0)
    denom = np.maximum(np.abs(b), floor_frac * scale)
    return (np.abs(np.asarray(a) - b) / np.where(denom > 0, denom, 1.0)).max()
