"""Shock sensors (navier-stokes/state_sensor.h)."""
from . import _abi


class const_sensor_t:
    """state_sensor::const_sensor_t(alpha) (state_sensor.h:46-60)."""
    kind = _abi.SENSOR_CONST

    def __init__(self, alpha):
        self.alpha = float(alpha)
