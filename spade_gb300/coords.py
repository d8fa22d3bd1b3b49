"""Coordinate systems (core/coord_system.h).  The GB300 path supports the
identity map and diagonal maps whose only non-identity direction is y."""
from . import _abi


class identity:
    """coords::identity (coord_system.h:51-56)."""
    kind = _abi.COORDS_IDENTITY
    params = (0.0, 0.0, 0.0, 0.0)


class identity_1D:
    """coords::identity_1D (coord_system.h:58-63)."""


class tanh_stretch_1D:
    """y = ymid + half*tanh(beta*s)/tanh(beta), s = (2*eta - (y0 + y1))/(y1 - y0):
    the usual channel wall clustering with stretching parameter beta.  No
    reference counterpart (the reference's integrated_tanh_1D is
    parametrised differently)."""

    def __init__(self, beta):
        self.beta = float(beta)


class integrated_tanh_1D:
    """coords::integrated_tanh_1D(y0, y1, inflation, rate)
    (coord_system.h:103-140)."""

    def __init__(self, y0, y1, inflation, rate):
        self.args = (float(y0), float(y1), float(inflation), float(rate))


class diagonal_coords:
    """coords::diagonal_coords(x, y, z) (coord_system.h:65-90); only y may be
    non-identity on this path."""

    def __init__(self, xcoord, ycoord, zcoord):
        if not isinstance(xcoord, identity_1D) or not isinstance(zcoord, identity_1D):
            raise ValueError("diagonal_coords: only the y direction may be stretched")
        if isinstance(ycoord, tanh_stretch_1D):
            self.kind = _abi.COORDS_TANH_Y
            self.params = (ycoord.beta, 0.0, 0.0, 0.0)
        elif isinstance(ycoord, integrated_tanh_1D):
            self.kind = _abi.COORDS_INTEGRATED_TANH_Y
            self.params = ycoord.args
        elif isinstance(ycoord, identity_1D):
            self.kind = _abi.COORDS_IDENTITY
            self.params = (0.0, 0.0, 0.0, 0.0)
        else:
            raise ValueError("unsupported y coordinate map")
