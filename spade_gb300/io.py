"""Native checkpoint format of the reference (io/io_native.h:15-55,
core/parallel.h:200-260): the raw memory of every block of a grid_array —
all variables, ghost layers included, the AoS5 linear map — written at byte
offset lb_glob * block_bytes, with no header.  The reference's own writer no
longer compiles against its current grid_array (it calls var_map() /
block_map(), which grid_array.h no longer has); this module writes and reads
that layout for the current array.

Works on torch tensors (any device) or numpy arrays of shape
(local blocks, nz+2ng, ny+2ng, nx+2ng, 5); `first_block` is the global index
of the first local block (block_partition_t.starts[rank] on a partitioned
grid), so ranks can write their blocks of one file independently.
"""
import os

import numpy as np


def _host(a):
    try:
        import torch
        if isinstance(a, torch.Tensor):
            return a.detach().cpu().contiguous().numpy()
    except ImportError:
        pass
    return np.ascontiguousarray(a)


def _payload(q):
    """The array behind a grid_array, or q itself (numpy / torch)."""
    return q.data if hasattr(q, "desc") else q


def block_bytes(shape):
    return int(np.prod(shape[1:])) * 8


def binary_write(filename, q, first_block=0):
    """Writes the local blocks of q into `filename` at their global offsets
    (the file is created if needed and is not truncated, so several ranks can
    fill one file)."""
    h = _host(_payload(q))
    if h.dtype != np.float64 or h.ndim != 5 or h.shape[-1] != 5:
        raise ValueError("expected a float64 AoS5 array (blocks, nk, nj, ni, 5)")
    bb = block_bytes(h.shape)
    fd = os.open(filename, os.O_RDWR | os.O_CREAT, 0o644)
    try:
        for lb in range(h.shape[0]):
            os.pwrite(fd, h[lb].tobytes(), (first_block + lb) * bb)
    finally:
        os.close(fd)


def binary_read(filename, q, first_block=0):
    """Reads the local blocks of q from `filename` (the inverse of
    binary_write); q is updated in place and returned."""
    data = _payload(q)
    shape = tuple(data.shape)
    bb = block_bytes(shape)
    out = np.empty(shape, dtype=np.float64)
    fd = os.open(filename, os.O_RDONLY)
    try:
        for lb in range(shape[0]):
            buf = os.pread(fd, bb, (first_block + lb) * bb)
            if len(buf) != bb:
                raise IOError("checkpoint %s is too short for block %d" % (filename, first_block + lb))
            out[lb] = np.frombuffer(buf, dtype=np.float64).reshape(shape[1:])
    finally:
        os.close(fd)
    try:
        import torch
        if isinstance(data, torch.Tensor):
            data.copy_(torch.from_numpy(out))
            return q
    except ImportError:
        pass
    data[...] = out
    return q
