"""Shock sensors (navier-stokes/state_sensor.h)."""
from . import _abi


class const_sensor_t:
    """state_sensor::const_sensor_t(alpha) (state_sensor.h:46-60)."""
    kind = _abi.SENSOR_CONST

    def __init__(self, alpha):
        self.alpha = float(alpha)


class ducros_t:
    """state_sensor::ducros_t(epsilon) (state_sensor.h:21-43): the face value
    theta^2 / (theta^2 + |omega|^2 + epsilon), theta the velocity divergence
    and omega the vorticity of the face gradient (info::gradient)."""
    kind = _abi.SENSOR_DUCROS

    def __init__(self, epsilon):
        self.epsilon = float(epsilon)

    @property
    def alpha(self):
        # the scheme descriptor carries epsilon in sensor_alpha for this kind
        return self.epsilon
