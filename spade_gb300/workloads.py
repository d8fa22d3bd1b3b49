"""Synthetic workloads with the shapes of the benchmark configurations:
the Taylor–Green vortex cube and the stretched wall-bounded channel.

Initial fields follow the reference drivers where one exists
(development/cuda-tgv/main.cc:107-116 for the TGV, which omits the usual
1/16 pressure factor; that form is used here).  Random perturbations come
from numpy's PCG64 (platform-independent) or, for very large grids, from a
seeded torch generator on the device.
"""
import math

import numpy as np
import torch

from . import _abi, algs, boundary, convective, coords, fluid_state, grid as _grid
from . import omni, pde_algs, state_sensor, viscous, viscous_laws


def stable_dt(cfl, dmin, umax, nu_max):
    """Explicit SSPRK3 time step: the convective CFL limit cfl*dx/max(|u|+a)
    and the 3-D diffusive limit 0.2*dx^2/nu (SSPRK3 reaches about 2.5 along
    the negative real axis; the viscous operator's largest eigenvalue is
    about 12 nu/dx^2), whichever is smaller."""
    return min(cfl * dmin / umax, 0.2 * dmin * dmin / nu_max)


class problem:
    """A grid, its primitive state, the flux functor, BCs and the time step."""

    def __init__(self, **kw):
        self.__dict__.update(kw)

    def scheme_desc(self, precision=_abi.PREC_FP64):
        return pde_algs.lower(self.flux, precision)

    def bc_desc(self):
        return self.exchange.bc_desc(self.walls)


def _cell_centres(g, lb_count, ng, d):
    """Computational cell-centre coordinates along d for every block,
    ghosts included: array (nblocks, n_d + 2 ng)."""
    nb = g.blocks.num_blocks
    out = np.empty((lb_count, g.cells[d] + 2 * ng))
    idx = np.arange(-ng, g.cells[d] + ng, dtype=np.float64)
    for lb in range(lb_count):
        b = [lb % nb[0], (lb // nb[0]) % nb[1], lb // (nb[0] * nb[1])][d]
        lo, hi = g.blocks.bounds[2 * d], g.blocks.bounds[2 * d + 1]
        bsize = (hi - lo) / nb[d]
        mn = lo + b * bsize
        dx = ((mn + bsize) - mn) / g.cells[d]
        out[lb] = mn + (idx + 0.5) * dx
    return out


def _noise(shape, kind, scale, seed, rng, device):
    if rng == "numpy":
        r = np.random.Generator(np.random.PCG64(seed))
        a = r.uniform(-1.0, 1.0, size=shape) if kind == "uniform" else r.standard_normal(size=shape)
        return torch.from_numpy(a * scale).to(device)
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    if kind == "uniform":
        return (torch.rand(shape, generator=g, device=device, dtype=torch.float64) * 2.0 - 1.0) * scale
    return torch.randn(shape, generator=g, device=device, dtype=torch.float64) * scale


def taylor_green(nblk=(2, 2, 2), ncell=(16, 16, 16), ng=2, mach=0.1, reynolds=1600.0, prandtl=0.72,
                 gamma=1.4, R=287.0, T0=300.0, rho0=1.0, noise=1e-3, seed=0, cfl=0.5,
                 rng="numpy", device="cuda", convective_scheme="cent_keep2", p_factor=1.0):
    """Taylor–Green vortex on [0, 2 pi]^3 (identity coordinates, periodic).

    p = p0 + p_factor rho0 u0^2 (cos 2x + cos 2y)(cos 2z + 2).  p_factor = 1
    is the reference driver's form (development/cuda-tgv/main.cc:107-116),
    which omits the textbook 1/16 and so turns the pressure negative above
    Mach ~0.27 (gamma M^2 * 6 > 1); p_factor = 1/16 is the textbook field,
    positive up to Mach ~1."""
    L = 1.0
    p0 = rho0 * R * T0
    u0, mu = tgv_params(mach, reynolds, gamma, R, T0, rho0)
    air = fluid_state.ideal_gas_t(gamma, R)
    blocks = _grid.cartesian_blocks_t(nblk, (0.0, 2 * math.pi, 0.0, 2 * math.pi, 0.0, 2 * math.pi))
    g = _grid.cartesian_grid_t(ncell, blocks, coords.identity())
    q = _grid.grid_array(g, 0.0, ng, device=device)
    nb = g.get_num_global_blocks()
    x = torch.from_numpy(_cell_centres(g, nb, ng, 0)).to(device)[:, None, None, :]
    y = torch.from_numpy(_cell_centres(g, nb, ng, 1)).to(device)[:, None, :, None]
    z = torch.from_numpy(_cell_centres(g, nb, ng, 2)).to(device)[:, :, None, None]
    d = q.data
    d[..., 0] = p0 + p_factor * rho0 * u0 * u0 * (torch.cos(2 * x / L) + torch.cos(2 * y / L)) * (torch.cos(2 * z / L) + 2.0)
    d[..., 1] = T0
    d[..., 2] = u0 * torch.sin(x / L) * torch.cos(y / L) * torch.cos(z / L)
    d[..., 3] = -u0 * torch.cos(x / L) * torch.sin(y / L) * torch.cos(z / L)
    d[..., 4] = 0.0
    if noise:
        inner = q.interior()
        inner[..., 2:5] += _noise(inner[..., 2:5].shape, "uniform", noise * u0, seed, rng, device)
    h = _grid.make_exchange(q, (True, True, True))
    h.exchange(q)
    if convective_scheme == "cent_keep2":
        conv = convective.cent_keep(2, air)
    elif convective_scheme == "totani":
        conv = convective.totani_lr(air)
    else:
        raise ValueError(convective_scheme)
    flux = omni.compose(conv, viscous.visc_lr(viscous_laws.constant_viscosity_t(mu, prandtl), air))
    dx = min(g.get_dx(0), g.get_dx(1), g.get_dx(2))
    umax = algs.transform_reduce(q, air, algs.reduce_ops.max_wavespeed)
    rho_min = float((q.interior()[..., 0] / (R * q.interior()[..., 1])).min())
    dt = stable_dt(cfl, dx, umax, mu / rho_min)
    return problem(name="taylor_green", grid=g, q=q, gas=air, flux=flux, exchange=h, walls={},
                   dt=dt, mu=mu, u0=u0, ng=ng)


def channel_flux(air, mu_ref, c_w, prandtl=0.72, T_wall=300.0, sutherland_S=110.4, eps_diss=0.01,
                 weno="weno5", law="sutherland"):
    """The channel's flux functor: compose(WENO, pressure_diss_lr(const
    sensor 1, eps = eps_diss * c_w), visc_lr(law))."""
    if weno == "weno5":
        conv = convective.weno5_t(air)
    elif weno == "fweno":
        conv = convective.fweno_t(air)
    else:
        raise ValueError(weno)
    if law == "sutherland":
        vlaw = viscous_laws.sutherland_t(mu_ref, T_wall, sutherland_S, prandtl)
    elif law == "power":
        vlaw = viscous_laws.power_law_t(mu_ref, T_wall, 0.76, prandtl)
    else:
        vlaw = viscous_laws.constant_viscosity_t(mu_ref, prandtl)
    diss = convective.pressure_diss_lr(air, state_sensor.const_sensor_t(1.0), eps_diss * c_w, eps_diss * c_w)
    return omni.compose(conv, diss, viscous.visc_lr(vlaw, air))


def channel_params(mach_b=0.5, re_b=3000.0, gamma=1.4, R=287.0, T_wall=300.0, rho_b=1.0):
    """(c_w, U_b, mu_ref) of the channel: wall sound speed, bulk velocity,
    viscosity rho_b U_b h / Re_b with half-height h = 1."""
    c_w = math.sqrt(gamma * R * T_wall)
    U_b = mach_b * c_w
    return c_w, U_b, rho_b * U_b * 1.0 / re_b


def tgv_params(mach=0.1, reynolds=1600.0, gamma=1.4, R=287.0, T0=300.0, rho0=1.0):
    """(u0, mu) of the Taylor-Green vortex with L = 1."""
    u0 = mach * math.sqrt(gamma * R * T0)
    return u0, rho0 * u0 * 1.0 / reynolds


def channel(nblk=(8, 8, 8), ncell=(32, 32, 32), ng=3, beta=2.0, mach_b=0.5, re_b=3000.0, prandtl=0.72,
            gamma=1.4, R=287.0, T_wall=300.0, rho_b=1.0, sutherland_S=110.4, pert=0.05, seed=0, cfl=0.5,
            eps_diss=0.01, rng="numpy", device="cuda", weno="weno5", law="sutherland"):
    """Wall-bounded channel 4 pi x 2 x 4 pi/3, tanh-stretched in y (beta;
    beta=None: uniform identity coordinates), periodic in x and z,
    isothermal no-slip walls at y = +-1; laminar Poiseuille profile plus
    Gaussian velocity perturbations."""
    air = fluid_state.ideal_gas_t(gamma, R)
    c_w, U_b, mu_ref = channel_params(mach_b, re_b, gamma, R, T_wall, rho_b)
    p0 = rho_b * R * T_wall
    blocks = _grid.cartesian_blocks_t(nblk, (0.0, 4 * math.pi, -1.0, 1.0, 0.0, 4 * math.pi / 3))
    if beta:
        csys = coords.diagonal_coords(coords.identity_1D(), coords.tanh_stretch_1D(beta), coords.identity_1D())
    else:
        csys = coords.identity()
    g = _grid.cartesian_grid_t(ncell, blocks, csys)
    q = _grid.grid_array(g, 0.0, ng, device=device)
    nb = g.get_num_global_blocks()
    eta = _cell_centres(g, nb, ng, 1)
    yphys = np.tanh(beta * eta) / math.tanh(beta) if beta else eta
    y = torch.from_numpy(yphys).to(device)[:, None, :, None]
    d = q.data
    d[..., 0] = p0
    d[..., 1] = T_wall
    d[..., 2] = 1.5 * U_b * (1.0 - y * y)
    d[..., 3] = 0.0
    d[..., 4] = 0.0
    if pert:
        inner = q.interior()
        inner[..., 2:5] += _noise(inner[..., 2:5].shape, "normal", pert * U_b, seed, rng, device)
    h = _grid.make_exchange(q, (True, False, True))
    wall = boundary.isothermal_wall_t(T_wall)
    walls = {2: wall, 3: wall}
    algs.boundary_fill(q, boundary.combine(boundary.ymin, boundary.ymax), wall)
    flux = channel_flux(air, mu_ref, c_w, prandtl, T_wall, sutherland_S, eps_diss, weno, law)
    # physical spacing: dy = deta * dy/deta, smallest at the walls
    deta = g.get_dx(1)
    s_wall = 1.0
    dydeta_min = beta * (1.0 - math.tanh(beta * s_wall) ** 2) / math.tanh(beta) if beta else 1.0
    dmin = min(g.get_dx(0), g.get_dx(2), deta * dydeta_min)
    umax = algs.transform_reduce(q, air, algs.reduce_ops.max_wavespeed)
    dt = stable_dt(cfl, dmin, umax, mu_ref / rho_b)
    return problem(name="channel", grid=g, q=q, gas=air, flux=flux, exchange=h, walls=walls,
                   dt=dt, mu=mu_ref, u0=U_b, ng=ng)
