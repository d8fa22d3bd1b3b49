"""Block-structured grid and the AoS5 grid_array (grid/cartesian_blocks.h,
grid/cartesian_grid.h, grid/grid_array.h, core/mem_map.h:465-497).

A grid_array owns one torch float64 tensor on the GPU of shape
(nblocks, nz+2ng, ny+2ng, nx+2ng, 5), which is byte-for-byte SPADE's
linear_t<5> map: variables fastest, then i, j, k, block.  torch is used only
for device memory and streams.
"""
import ctypes

import numpy as np
import torch

from . import _abi, _native
from . import coords as _coords


class cartesian_blocks_t:
    """grid::cartesian_blocks_t(num_blocks, bounds) (cartesian_blocks.h:23-117).
    `bounds` = (xmin, xmax, ymin, ymax, zmin, zmax)."""

    def __init__(self, num_blocks, bounds):
        self.num_blocks = tuple(int(n) for n in num_blocks)
        if len(self.num_blocks) != 3:
            raise ValueError("num_blocks must have 3 entries")
        self.bounds = tuple(float(b) for b in bounds)
        if len(self.bounds) != 6:
            raise ValueError("bounds must be (xmin, xmax, ymin, ymax, zmin, zmax)")

    def total_num_blocks(self):
        n = self.num_blocks
        return n[0] * n[1] * n[2]


class cartesian_grid_t:
    """grid::cartesian_grid_t(cells_in_block, blocks, coords) (cartesian_grid.h:48-384)."""

    def __init__(self, cells_in_block, blocks, coord_sys=None):
        self.cells = tuple(int(n) for n in cells_in_block)
        self.blocks = blocks
        self.coord_sys = coord_sys if coord_sys is not None else _coords.identity()

    def get_num_cells(self, i=None):
        return self.cells if i is None else self.cells[i]

    def get_num_global_blocks(self):
        return self.blocks.total_num_blocks()

    get_num_local_blocks = get_num_global_blocks

    def get_grid_size(self):
        c = self.cells
        return c[0] * c[1] * c[2] * self.get_num_global_blocks()

    def desc(self, ng):
        return _abi.grid_desc(self.blocks.num_blocks, self.cells, ng, self.blocks.bounds,
                              self.coord_sys.kind, self.coord_sys.params)

    def get_coords(self, ng):
        """Physical cell-centre coordinates of every cell, ghosts included
        (cartesian_grid_t::get_coords, cartesian_grid.h:290-310): numpy arrays
        x (nb, 1, 1, ni), y (nb, 1, nj, 1), z (nb, nk, 1, 1) that broadcast to
        the grid_array shape without the variable axis.  Block boxes and
        spacing use the reference's arithmetic; y goes through the
        coordinate map when the system stretches it."""
        nb = self.blocks.num_blocks
        nlb = self.get_num_global_blocks()
        out = []
        for d in range(3):
            idx = np.arange(-ng, self.cells[d] + ng, dtype=np.float64)
            c = np.empty((nlb, self.cells[d] + 2 * ng))
            for lb in range(nlb):
                b = [lb % nb[0], (lb // nb[0]) % nb[1], lb // (nb[0] * nb[1])][d]
                lo, hi = self.blocks.bounds[2 * d], self.blocks.bounds[2 * d + 1]
                bsize = (hi - lo) / nb[d]
                mn = lo + b * bsize
                c[lb] = mn + (idx + 0.5) * (((mn + bsize) - mn) / self.cells[d])
            if d == 1 and getattr(self.coord_sys, "kind", _abi.COORDS_IDENTITY) != _abi.COORDS_IDENTITY:
                c = self.coord_sys.map_y(c, self.blocks.bounds[2], self.blocks.bounds[3])
            out.append(c)
        return out[0][:, None, None, :], out[1][:, None, :, None], out[2][:, :, None, None]

    def get_dx(self, i, lb=0):
        """Block spacing exactly as the reference computes it."""
        nb = self.blocks.num_blocks[i]
        b = [lb % self.blocks.num_blocks[0], (lb // self.blocks.num_blocks[0]) % self.blocks.num_blocks[1],
             lb // (self.blocks.num_blocks[0] * self.blocks.num_blocks[1])][i]
        lo, hi = self.blocks.bounds[2 * i], self.blocks.bounds[2 * i + 1]
        bsize = (hi - lo) / nb
        mn = lo + b * bsize
        return ((mn + bsize) - mn) / self.cells[i]


class grid_array:
    """grid::grid_array(grid, fill, num_exch, device) (grid_array.h:175-422)."""

    def __init__(self, grid, fill=0.0, num_exch=2, device="cuda", data=None):
        self.grid = grid
        ng = num_exch if np.isscalar(num_exch) else num_exch[0]
        if not np.isscalar(num_exch) and len(set(num_exch)) != 1:
            raise ValueError("the GB300 path uses the same ghost depth in every direction")
        self.ng = int(ng)
        c = grid.cells
        self.shape = (grid.get_num_global_blocks(), c[2] + 2 * self.ng, c[1] + 2 * self.ng, c[0] + 2 * self.ng, 5)
        if data is not None:
            if tuple(data.shape) != self.shape or data.dtype != torch.float64:
                raise ValueError("data must be float64 with shape %s" % (self.shape,))
            self.data = data
        else:
            self.data = torch.empty(self.shape, dtype=torch.float64, device=device)
            self.fill_(fill)
        self._desc = grid.desc(self.ng)
        self.periodic = None

    def fill_(self, fill):
        if np.isscalar(fill):
            self.data.fill_(float(fill))
        else:
            self.data.copy_(torch.as_tensor(np.asarray(fill, dtype=np.float64), device=self.data.device).expand(self.shape))
        return self

    def desc(self):
        return self._desc

    def ptr(self):
        return self.data.data_ptr()

    def interior(self):
        g = self.ng
        return self.data[:, g:-g, g:-g, g:-g, :]

    def numpy(self):
        return self.data.detach().cpu().numpy()

    def copy_from_numpy(self, arr):
        self.data.copy_(torch.from_numpy(np.ascontiguousarray(arr, dtype=np.float64)))
        return self

    def device(self):
        return self.data.device

    def __iadd__(self, other):
        self.data += other.data if isinstance(other, grid_array) else other
        return self

    def assign(self, value):
        """rhs = value (grid_array::operator=, grid_array.h:383-392)."""
        if isinstance(value, grid_array):
            self.data.copy_(value.data)
        else:
            self.data.fill_(float(value))
        return self


def _stream(stream):
    if stream is None:
        return ctypes_stream(torch.cuda.current_stream())
    if isinstance(stream, int):
        return stream
    return ctypes_stream(stream)


def ctypes_stream(s):
    return int(s.cuda_stream)


class arr_exchange_t:
    """Handle returned by make_exchange (make_exchange.h:98-421).
    exchange(q) fills every ghost that has a donor block (periodic wrap where
    periodic[d]); ghosts across non-periodic faces are left for boundary_fill."""

    def __init__(self, periodic):
        self.periodic = tuple(bool(p) for p in periodic)

    def bc_desc(self, walls=None):
        kinds = []
        t_wall = []
        for d in range(3):
            for s in range(2):
                face = 2 * d + s
                if walls and face in walls:
                    kinds.append(walls[face].kind)
                    t_wall.append(walls[face].t_wall)
                else:
                    kinds.append(_abi.BC_PERIODIC if self.periodic[d] else _abi.BC_NONE)
                    t_wall.append(0.0)
        return _abi.bc_desc(kinds, t_wall)

    def exchange(self, q, group=None, stream=None):
        bc = self.bc_desc()
        _native.check(_native.lib().gbns_fill_ghosts(q.desc(), bc, q.ptr(), _stream(stream)))


class exchange_plan_t:
    """The ghost fill of a block layout with refinement levels (AMR), run from
    an exchange plan: the reference's own transaction list for that layout
    (its make_exchange on an amr_blocks_t grid, grid/make_exchange.h:98-421),
    as an (n, 18) int32 array of gbns_patch records (kind, source block,
    destination block, source box origin, destination box [lo, hi),
    i_coeff, i_incr).  The C++ drop-in lowers a reference exchange handle into
    such a plan (spade::gb300::lower_exchange).  exchange(q) runs it on a
    grid_array-shaped float64 tensor (nblocks, nz+2ng, ny+2ng, nx+2ng, 5) on
    the GPU: injections, then interpolations, bit-identical to the
    reference's exchange."""

    def __init__(self, ncell, ng, nblocks, plan, stream=None):
        self.plan = np.ascontiguousarray(plan, dtype=np.int32)
        assert self.plan.ndim == 2 and self.plan.shape[1] == 18
        self.ncell, self.ng, self.nblocks = tuple(int(n) for n in ncell), int(ng), int(nblocks)
        h = ctypes.c_void_p()
        _native.check(_native.lib().gbns_exchange_plan_create(ctypes.byref(h), self.ncell[0], self.ncell[1], self.ncell[2],
                                                              self.ng, self.nblocks,
                                                              ctypes.c_void_p(self.plan.ctypes.data),
                                                              int(self.plan.shape[0]), _stream(stream)))
        self.handle = h

    def exchange(self, q, stream=None):
        data = q.data if hasattr(q, "data") and not isinstance(q, torch.Tensor) else q
        want = (self.nblocks, self.ncell[2] + 2 * self.ng, self.ncell[1] + 2 * self.ng, self.ncell[0] + 2 * self.ng, 5)
        if tuple(data.shape) != want or data.dtype != torch.float64 or not data.is_cuda:
            raise ValueError("exchange_plan_t.exchange: expected a CUDA float64 array of shape %s" % (want,))
        _native.check(_native.lib().gbns_exchange_plan_run(self.handle, ctypes.c_void_p(data.data_ptr()), _stream(stream)))

    def close(self):
        if getattr(self, "handle", None):
            _native.lib().gbns_exchange_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class refined_layout_t:
    """A refined (AMR) block layout as the GB300 kernels take it: nblocks
    blocks of the same ncell cells and ng ghost layers, in the caller's
    global block order, each with its bounding box (boxes: (nblocks, 6),
    min and max along x, y, z), identity coordinates.  The block tree stays
    the caller's (the reference's amr_blocks_t refined with
    cartesian_grid_t::refine_blocks); every block takes 1/dx from its own box
    as the reference's flux_div does (flux_div_basic.h:55,
    grid/grid_geometry.h:85-89).  Arrays on it are float64 tensors of shape
    (nblocks, nz+2ng, ny+2ng, nx+2ng, 5)."""

    def __init__(self, ncell, ng, boxes):
        self.ncell = tuple(int(n) for n in ncell)
        self.ng = int(ng)
        self.boxes = np.ascontiguousarray(boxes, dtype=np.float64)
        if self.boxes.ndim != 2 or self.boxes.shape[1] != 6:
            raise ValueError("boxes must be (nblocks, 6)")
        self.nblocks = int(self.boxes.shape[0])
        self._desc = _abi.grid_desc((self.nblocks, 1, 1), self.ncell, self.ng, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))

    def desc(self):
        return self._desc

    def shape(self):
        ng = self.ng
        return (self.nblocks, self.ncell[2] + 2 * ng, self.ncell[1] + 2 * ng, self.ncell[0] + 2 * ng, 5)

    def check(self, t):
        if tuple(t.shape) != self.shape() or t.dtype != torch.float64 or not t.is_contiguous():
            raise ValueError("expected a contiguous float64 array of shape %s" % (self.shape(),))

    def boxes_ptr(self):
        return ctypes.c_void_p(self.boxes.ctypes.data)

    def fill_walls(self, q, bc, bounds=(0.0, 1.0, 0.0, 1.0, 0.0, 1.0), stream=None):
        """The wall faces of bc (a gbns_bc_desc) on the CUDA tensor q, after its
        exchange: the blocks whose box touches a wall face of the domain
        `bounds` mirror their ghost slab through the wall kernel
        (algs::boundary_fill, gbns_wall_fill_blocks)."""
        self.check(q)
        if not q.is_cuda:
            raise ValueError("the wall fill runs on CUDA tensors")
        g = _abi.grid_desc((self.nblocks, 1, 1), self.ncell, self.ng, bounds)
        _native.check(_native.lib().gbns_wall_fill_blocks(g, self.boxes_ptr(), bc, ctypes.c_void_p(q.data_ptr()),
                                                          _stream(stream)))


def make_exchange(q, periodic):
    h = arr_exchange_t(periodic)
    q.periodic = h.periodic
    return h
