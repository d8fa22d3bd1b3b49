"""Generic array algorithms (algs/): traits, boundary_fill, reductions."""
import ctypes

import numpy as np

from . import _abi, _native
from .grid import _stream


def make_traits(*tags):
    """algs::make_traits(tag...) (algs/alg_traits.h:77-81)."""
    return tuple(tags)


def get_trait(traits, label, default=None):
    for t in traits or ():
        if getattr(t, "trait_label", None) == label:
            return t
    return default


def boundary_fill(q, boundaries, kern, stream=None):
    """algs::boundary_fill(q, boundary::ymin, wall) (grid/boundary_fill.h:31-133):
    fills the ghost layers across the given domain faces from the mirrored
    interior with the wall kernel `kern` (boundary.isothermal_wall_t /
    slip_wall_t).  Other ghosts are refilled from their donors as well
    (idempotent with the last exchange)."""
    periodic = q.periodic if q.periodic is not None else (False, False, False)
    from .grid import arr_exchange_t
    h = arr_exchange_t(periodic)
    for f in boundaries:
        if periodic[f // 2]:
            raise ValueError("boundary_fill on a periodic direction")
    walls = {f: kern for f in boundaries}
    bc = h.bc_desc(walls)
    _native.check(_native.lib().gbns_fill_ghosts(q.desc(), bc, q.ptr(), _stream(stream)))


class reduce_ops:
    max_wavespeed = _abi.RED_MAX_WAVESPEED
    kinetic_energy = _abi.RED_KINETIC
    conserved = _abi.RED_CONSERVED
    health = _abi.RED_HEALTH


def transform_reduce(q, gas, kind, stream=None):
    """Interior reduction (algs/transform_reduce.h:53-191) for the reductions
    the reference drivers use: max(|u| + a) for the CFL, volume-averaged
    kinetic energy, Jacobian-weighted conserved sums, or the count of
    non-physical cells.  Synchronises the stream."""
    out = np.zeros(5)
    _native.check(_native.lib().gbns_reduce(q.desc(), gas.desc(), q.ptr(), int(kind),
                                            out.ctypes.data_as(ctypes.c_void_p), _stream(stream)))
    return out if kind == _abi.RED_CONSERVED else float(out[0])


include_exchanges = "include_exchanges"
exclude_exchanges = "exclude_exchanges"


def fill_array(q, func, exchange_policy=include_exchanges):
    """algs::fill_array(array, kernel, exchange_policy)
    (algs/transform_inplace.h:97-101): q = func(x, y, z) at every cell centre
    (ghosts too with include_exchanges).  func receives the physical
    coordinates as torch tensors on q's device (broadcastable shapes) and
    returns the five primitives (p, T, u, v, w), each a tensor or a number.
    Host-side initialisation: not a hot path."""
    import torch
    ng = q.ng
    x, y, z = (torch.from_numpy(np.ascontiguousarray(a)).to(q.data.device) for a in q.grid.get_coords(ng))
    vals = func(x, y, z)
    if len(vals) != 5:
        raise ValueError("fill_array: func must return (p, T, u, v, w)")
    full = q.data.shape[:-1]
    target = q.data if exchange_policy == include_exchanges else q.interior()
    for v, val in enumerate(vals):
        t = torch.as_tensor(val, dtype=torch.float64, device=q.data.device).expand(full)
        if exchange_policy == include_exchanges:
            target[..., v] = t
        else:
            target[..., v] = t[:, ng:-ng, ng:-ng, ng:-ng]
    return q
