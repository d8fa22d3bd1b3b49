"""Viscous flux functor (navier-stokes/viscous.h)."""


class visc_lr:
    """viscous::visc_lr(law, gas) (viscous.h:13-113): face average state,
    10-cell face gradient, Newtonian stress and Fourier heat flux."""

    def __init__(self, vlaw, gas):
        self.vlaw = vlaw
        self.gas = gas
