"""Batched form: many independent grids of uneven size advanced together by
flux launches over device work-lists of tiles, one CUDA graph per step
(gbns_batch_* in include/gbns.h).  Instance state stays resident in an arena
sized by an HBM budget; every instance's result is bit-identical to
advancing it alone."""
import ctypes

import torch

from . import _abi, _native
from .grid import _stream


class _DevView:
    """A raw device pointer exposed through __cuda_array_interface__ so torch
    can view it without a copy."""

    def __init__(self, ptr, shape):
        self.__cuda_array_interface__ = {"shape": tuple(shape), "typestr": "<f8", "data": (int(ptr), False),
                                         "version": 3, "strides": None}


class batch_t:
    def __init__(self, hbm_budget_bytes, precision=_abi.PREC_FP64, use_graph=True, stream=None):
        self.lib = _native.lib()
        self.stream = stream or torch.cuda.current_stream()
        h = ctypes.c_void_p()
        _native.check(self.lib.gbns_batch_create(ctypes.byref(h), int(hbm_budget_bytes), int(precision),
                                                 int(bool(use_graph)), _stream(self.stream)))
        self.handle = h
        self.precision = precision
        self.meta = {}

    def add(self, grid_desc, scheme_desc, bc_desc, dt, prims_ptr, shape=None):
        """Adds an instance; prims_ptr is a device (or pinned host) pointer to
        its AoS5 initial state.  Returns the slot.  Raises SpadeError with
        code ERR_CAPACITY when the HBM budget cannot hold it."""
        slot = ctypes.c_int(-1)
        _native.check(self.lib.gbns_batch_add(self.handle, grid_desc, scheme_desc, bc_desc, ctypes.c_double(dt),
                                              ctypes.c_void_p(int(prims_ptr)), ctypes.byref(slot)))
        self.meta[slot.value] = (grid_desc, scheme_desc, bc_desc, dt, shape)
        return slot.value

    def remove(self, slot):
        _native.check(self.lib.gbns_batch_remove(self.handle, int(slot)))
        self.meta.pop(slot, None)

    def step(self, nsteps=1):
        _native.check(self.lib.gbns_batch_step(self.handle, int(nsteps)))

    CLASS_NAMES = ("cent_keep2/identity", "totani_lr/identity", "fweno/identity", "weno5/stretched-y",
                   "weno5/identity", "hybrid(cent_keep2,fweno)/identity")

    def autotune(self, reps=3):
        """Times every tile variant of each kernel class present among the
        active instances on their own arrays (gbns_batch_autotune) and keeps
        the fastest.  Returns {class name: {"variant": v, "tile": (x, y, z)}}."""
        n = int(self.lib.gbns_batch_class_count())
        out = (ctypes.c_int * n)()
        _native.check(self.lib.gbns_batch_autotune(self.handle, int(reps), out))
        res = {}
        for c in range(n):
            if out[c] < 0:
                continue
            t = (ctypes.c_int * 3)()
            _native.check(self.lib.gbns_batch_class_variant_info(c, int(self.precision), int(out[c]), t))
            res[self.CLASS_NAMES[c]] = {"variant": int(out[c]), "tile": (t[0], t[1], t[2])}
        return res

    def set_steps(self, slot, nsteps):
        """The instance does at most `nsteps` more steps (counted on the
        device), then idles until removed; nsteps < 0 lifts the limit."""
        _native.check(self.lib.gbns_batch_set_steps(self.handle, int(slot), int(nsteps)))

    def steps_left(self, slot):
        n = ctypes.c_longlong()
        _native.check(self.lib.gbns_batch_steps_left(self.handle, int(slot), ctypes.byref(n)))
        return n.value

    def set_variant(self, kernel_class, variant):
        _native.check(self.lib.gbns_batch_set_variant(self.handle, int(kernel_class), int(variant)))

    def state_ptr(self, slot):
        p = ctypes.c_void_p()
        n = ctypes.c_longlong()
        _native.check(self.lib.gbns_batch_state(self.handle, int(slot), ctypes.byref(p), ctypes.byref(n)))
        return p.value, n.value

    def state(self, slot):
        """A torch view (no copy) of the instance's AoS5 state."""
        g = self.meta[slot][0]
        ptr, _ = self.state_ptr(slot)
        shape = (g.nblk[0] * g.nblk[1] * g.nblk[2], g.ncell[2] + 2 * g.ng, g.ncell[1] + 2 * g.ng, g.ncell[0] + 2 * g.ng, 5)
        return torch.as_tensor(_DevView(ptr, shape), device="cuda")

    def steps_done(self, slot):
        return self.state_ptr(slot)[1]

    def usage(self):
        used, budget = ctypes.c_size_t(), ctypes.c_size_t()
        active, cells = ctypes.c_int(), ctypes.c_longlong()
        _native.check(self.lib.gbns_batch_usage(self.handle, ctypes.byref(used), ctypes.byref(budget),
                                                ctypes.byref(active), ctypes.byref(cells)))
        return {"bytes_used": used.value, "bytes_budget": budget.value, "active": active.value, "cells": cells.value}

    @staticmethod
    def instance_bytes(grid_desc):
        return int(_native.lib().gbns_batch_instance_bytes(grid_desc))

    def close(self):
        if self.handle:
            self.lib.gbns_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
