"""Coordinate systems (core/coord_system.h).  The GB300 path supports the
identity map and diagonal maps whose only non-identity direction is y."""
import math

import numpy as np

from . import _abi


class identity:
    """coords::identity (coord_system.h:51-56)."""
    kind = _abi.COORDS_IDENTITY
    params = (0.0, 0.0, 0.0, 0.0)

    def map_y(self, eta, y0, y1):
        return np.asarray(eta, dtype=np.float64)


class identity_1D:
    """coords::identity_1D (coord_system.h:58-63)."""

    def map(self, eta, y0, y1):
        return np.asarray(eta, dtype=np.float64)


class tanh_stretch_1D:
    """y = ymid + half*tanh(beta*s)/tanh(beta), s = (2*eta - (y0 + y1))/(y1 - y0):
    the usual channel wall clustering with stretching parameter beta.  No
    reference counterpart (the reference's integrated_tanh_1D is
    parametrised differently)."""

    def __init__(self, beta):
        self.beta = float(beta)

    def map(self, eta, y0, y1):
        """Physical y of computational eta on the domain [y0, y1]."""
        s = (2.0 * np.asarray(eta, dtype=np.float64) - (y0 + y1)) / (y1 - y0)
        return 0.5 * (y0 + y1) + 0.5 * (y1 - y0) * np.tanh(self.beta * s) / math.tanh(self.beta)


class integrated_tanh_1D:
    """coords::integrated_tanh_1D(y0, y1, inflation, rate)
    (coord_system.h:103-140)."""

    def __init__(self, y0, y1, inflation, rate):
        self.args = (float(y0), float(y1), float(inflation), float(rate))

    def map(self, eta, y0=None, y1=None):
        """integrated_tanh_1D::map (coord_system.h:125-133)."""
        eta1, eta0, strch, k = self.args
        deta = eta1 - eta0
        a0, a1 = k / deta, -k / deta
        b0, b1 = a0 * (strch * deta - eta0), a0 * (eta1 + strch * deta)

        def f(e):
            return np.log(np.abs(np.cosh(a0 * e + b0))) / a0 + np.log(np.abs(np.cosh(a1 * e + b1))) / a1 - e

        f0 = f(eta0)
        return eta0 + deta * (f(np.asarray(eta, dtype=np.float64)) - f0) * (1.0 / (f(eta1) - f0))


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
        self.ycoord = ycoord

    def map_y(self, eta, y0, y1):
        return self.ycoord.map(eta, y0, y1)
