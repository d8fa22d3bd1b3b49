"""Boundary identifiers and wall kernels (grid/boundary_fill.h:7-27)."""
from . import _abi

xmin, xmax, ymin, ymax, zmin, zmax = (0,), (1,), (2,), (3,), (4,), (5,)


def combine(*ids):
    out = ()
    for i in ids:
        out = out + tuple(i)
    return out


class isothermal_wall_t:
    """Isothermal no-slip wall ghost kernel: p_g = p, T_g = 2 T_w - T,
    u_g = -u (the wall lambda of a reference channel driver)."""
    kind = _abi.BC_ISOTHERMAL_NOSLIP

    def __init__(self, t_wall):
        self.t_wall = float(t_wall)


class slip_wall_t:
    """Adiabatic slip wall: p_g = p, T_g = T, normal velocity reflected."""
    kind = _abi.BC_SLIP_ADIABATIC
    t_wall = 0.0
