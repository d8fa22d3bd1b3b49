"""Viscosity laws (navier-stokes/viscous_laws.h)."""
from . import _abi


class constant_viscosity_t:
    """viscous_laws::constant_viscosity_t(mu, Pr) (viscous_laws.h:62-100):
    mu, beta = -2 mu/3, alpha = mu/Pr."""
    law = _abi.LAW_CONSTANT

    def __init__(self, visc, prandtl):
        self.mu = float(visc)
        self.prandtl = float(prandtl)
        self.T_ref = 1.0
        self.power = 0.0
        self.S = 0.0


class power_law_t:
    """viscous_laws::power_law_t(mu_ref, T_ref, power, Pr)
    (viscous_laws.h:102-135): mu = mu_ref (T/T_ref)^power at the face
    state, beta = -0.66666666667 mu, alpha = mu/Pr."""
    law = _abi.LAW_POWER

    def __init__(self, mu_ref, T_ref, power, prandtl):
        self.mu = float(mu_ref)
        self.T_ref = float(T_ref)
        self.power = float(power)
        self.prandtl = float(prandtl)
        self.S = 0.0


class sutherland_t:
    """Sutherland's law mu = mu_ref (T/T_ref)^1.5 (T_ref + S)/(T + S) at the
    face state, beta = -2 mu/3, alpha = mu/Pr.  No reference counterpart;
    follows the constant law's conventions."""
    law = _abi.LAW_SUTHERLAND

    def __init__(self, mu_ref, T_ref, S, prandtl):
        self.mu = float(mu_ref)
        self.T_ref = float(T_ref)
        self.S = float(S)
        self.prandtl = float(prandtl)
        self.power = 1.5
