"""Convective flux functors (navier-stokes/convective.h)."""
from . import _abi


class cent_keep_scheme_t:
    """convective::cent_keep_scheme_t<gas, order> (convective.h:96-192)."""

    def __init__(self, gas, order):
        if order not in (2, 4, 6, 8):
            raise ValueError("cent_keep order must be 2, 4, 6 or 8")
        self.gas = gas
        self.order = int(order)
        self.kind = _abi.CONV_CENT_KEEP


def cent_keep(order, gas):
    """convective::cent_keep<order>(gas) (convective.h:187-192)."""
    if order % 2:
        raise ValueError("nominal order for centered scheme must be even")
    return cent_keep_scheme_t(gas, order)


class totani_lr:
    """convective::totani_lr(gas) (convective.h:54-94): 2-point KEEP."""

    def __init__(self, gas):
        self.gas = gas
        self.order = 2
        self.kind = _abi.CONV_TOTANI


enable_smooth = 1
disable_smooth = 0


class fweno_t:
    """convective::fweno_t<gas, smooth> (convective.h:335-497): 4-point,
    3rd-order WENO on a per-point Rusanov split."""

    def __init__(self, gas, smooth=enable_smooth):
        self.gas = gas
        self.order = 2
        self.smooth = int(smooth)
        self.kind = _abi.CONV_FWENO


class weno5_t:
    """5th-order WENO-JS on fweno_t's Rusanov split (6-point stencil, three
    ghost layers).  No reference counterpart."""

    def __init__(self, gas, smooth=enable_smooth):
        self.gas = gas
        self.order = 2
        self.smooth = int(smooth)
        self.kind = _abi.CONV_WENO5


class pressure_diss_lr:
    """convective::pressure_diss_lr(gas, sensor, eps_p[, eps_T])
    (convective.h:194-246)."""

    def __init__(self, gas, sensor, eps_p, eps_T=None):
        self.gas = gas
        self.sensor = sensor
        self.eps_p = float(eps_p)
        self.eps_T = float(eps_p if eps_T is None else eps_T)
