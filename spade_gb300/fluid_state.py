"""Gas model and state vocabularies (navier-stokes/gas.h:35-49,
navier-stokes/fluid_state.h:60-126)."""
from . import _abi

PRIM_NAMES = ("P", "T", "U", "V", "W")                       # prim_t
CONS_NAMES = ("rho", "rhoH", "rhoU", "rhoV", "rhoW")          # cons_t
FLUX_NAMES = ("continuity", "energy", "x_momentum", "y_momentum", "z_momentum")  # flux_t


class ideal_gas_t:
    """fluid_state::ideal_gas_t(gamma, R)."""

    def __init__(self, gamma, R):
        self.gamma = float(gamma)
        self.R = float(R)

    def desc(self):
        g = _abi.GasDesc()
        g.gamma = self.gamma
        g.R = self.R
        return g


class prim_t:
    """Tag for the primitive state (p, T, u, v, w)."""
    names = PRIM_NAMES


class cons_t:
    """Tag for the conservative state (rho, rho E, rho u, rho v, rho w)."""
    names = CONS_NAMES


class flux_t:
    """Tag for residual/flux arrays (continuity, energy, x-, y-, z-momentum)."""
    names = FLUX_NAMES


class state_transform_t:
    """fluid_state::state_transform_t(cons_t(), gas): the RK update is done in
    conservative variables while the state is stored primitive
    (navier-stokes/state_transformation.h:38-66)."""

    def __init__(self, forward, gas):
        self.forward = forward
        self.gas = gas
