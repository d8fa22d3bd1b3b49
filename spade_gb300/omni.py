"""omni::compose (omni/compose.h:7-45): sum of flux functors over the union
stencil, evaluated as k0 + (k1 + k2)."""


class composite_kernel_t:
    def __init__(self, kernels):
        self.kernels = tuple(kernels)


def compose(*kernels):
    if not kernels:
        raise ValueError("compose needs at least one kernel")
    return composite_kernel_t(kernels)
