"""Multi-rank block decomposition: the block partition of the reference
(grid/partition.h:27-84, contiguous block ranges, the first ranks take one
extra block) and a host-staged halo exchange between ranks over
torch.distributed (gloo on CPU tensors, NCCL on GPU tensors).

On one GPU per box this path is exercised with CPU ranks; the single-device
ghost fill (gbns_fill_ghosts) is the special case world = 1.  The exchange
resolves every ghost cell to an interior donor exactly like the single-device
kernel: mirror across wall faces first (grid/boundary_fill.h:113-114), then
the periodic / inter-block exchange (grid/get_transaction.h:55-87), then the
wall transforms in face order.
"""
import numpy as np
import torch
import torch.distributed as dist

from . import _abi


class block_partition_t:
    """partition::block_partition_t (grid/partition.h:27-84)."""

    def __init__(self, num_global_blocks, world, rank):
        self.num_global_blocks = int(num_global_blocks)
        self.world = int(world)
        self.rank = int(rank)
        per = self.num_global_blocks // self.world
        extra = self.num_global_blocks - per * self.world
        counts = [per + (1 if r < extra else 0) for r in range(self.world)]
        starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(int)
        self.counts = counts
        self.starts = [int(x) for x in starts]
        self.global_to_rank = np.repeat(np.arange(self.world), counts)
        self.num_local_blocks = counts[self.rank]

    def local_blocks(self):
        s = self.starts[self.rank]
        return list(range(s, s + self.num_local_blocks))

    def owner(self, lb_glob):
        return int(self.global_to_rank[lb_glob])

    def to_local(self, lb_glob):
        return int(lb_glob - self.starts[self.owner(lb_glob)])


def _plan(grid, bc):
    """For every ghost cell of every block: (dst block, dst padded flat index,
    src block, src padded flat index, wall faces bitmask in order).  Ghosts
    that stay untouched (GBNS_BC_NONE) are omitted."""
    nb = np.array(grid.nblk)
    n = np.array(grid.ncell)
    ng = grid.ng
    ni, nj, nk = n + 2 * ng
    nblk = int(np.prod(nb))
    ii, jj, kk = np.meshgrid(np.arange(ni), np.arange(nj), np.arange(nk), indexing="ij")
    ii, jj, kk = ii.ravel(), jj.ravel(), kk.ravel()
    c0 = np.stack([ii - ng, jj - ng, kk - ng], axis=1)
    ghost = np.any((c0 < 0) | (c0 >= n), axis=1)
    c0 = c0[ghost]
    flat0 = (kk[ghost] * nj + jj[ghost]) * ni + ii[ghost]
    kinds = np.array(bc.kind)
    out = []
    for lb in range(nblk):
        b0 = np.array([lb % nb[0], (lb // nb[0]) % nb[1], lb // (nb[0] * nb[1])])
        c = c0.copy()
        b = np.tile(b0, (len(c), 1))
        walls = np.zeros((len(c), 3), dtype=np.int64) - 1
        for d in range(3):
            lo = (c[:, d] < 0) & (b0[d] == 0)
            hi = (c[:, d] >= n[d]) & (b0[d] == nb[d] - 1)
            for mask, face in ((lo, 2 * d), (hi, 2 * d + 1)):
                if kinds[face] in (_abi.BC_ISOTHERMAL_NOSLIP, _abi.BC_SLIP_ADIABATIC):
                    sel = mask
                    c[sel, d] = (-1 - c[sel, d]) if face % 2 == 0 else (2 * n[d] - (c[sel, d] + 1))
                    walls[sel, d] = face
        ok = np.ones(len(c), bool)
        for d in range(3):
            o = np.where(c[:, d] < 0, -1, np.where(c[:, d] >= n[d], 1, 0))
            at_min = b[:, d] == 0
            at_max = b[:, d] == nb[d] - 1
            bad = ((o < 0) & at_min & (kinds[2 * d] != _abi.BC_PERIODIC)) | ((o > 0) & at_max & (kinds[2 * d + 1] != _abi.BC_PERIODIC))
            ok &= ~bad
            b[:, d] = (b[:, d] + o) % nb[d]
            c[:, d] -= o * n[d]
        src_lb = b[:, 0] + nb[0] * (b[:, 1] + nb[1] * b[:, 2])
        src_flat = ((c[:, 2] + ng) * nj + (c[:, 1] + ng)) * ni + (c[:, 0] + ng)
        out.append((np.full(ok.sum(), lb), flat0[ok], src_lb[ok], src_flat[ok], walls[ok]))
    cat = [np.concatenate([o[i] for o in out]) for i in range(5)]
    return cat


class halo_exchange_t:
    """Ghost fill of a block-partitioned grid_array across ranks.  q_local has
    shape (local blocks, nz+2ng, ny+2ng, nx+2ng, 5)."""

    def __init__(self, grid, bc, partition, group=None):
        self.grid = grid
        self.bc = bc
        self.part = partition
        self.group = group
        dst_lb, dst_flat, src_lb, src_flat, walls = _plan(grid, bc)
        me = partition.rank
        own = partition.global_to_rank
        self.walls_all = walls
        # cells this rank fills
        mine = own[dst_lb] == me
        self.dst_local = np.array([partition.to_local(x) for x in dst_lb[mine]], dtype=np.int64)
        self.dst_flat = dst_flat[mine]
        self.walls = walls[mine]
        src_rank = own[src_lb[mine]]
        self.recv = {}
        for r in range(partition.world):
            sel = np.nonzero(src_rank == r)[0]
            if len(sel):
                self.recv[r] = sel            # positions (in this rank's fill list) served by rank r
        self.local_src = (np.array([partition.to_local(x) for x in src_lb[mine][src_rank == me]], dtype=np.int64),
                          src_flat[mine][src_rank == me])
        # what this rank sends to each peer: donors it owns for cells others fill
        self.send = {}
        for r in range(partition.world):
            if r == me:
                continue
            theirs = (own[dst_lb] == r) & (own[src_lb] == me)
            if theirs.any():
                self.send[r] = (np.array([partition.to_local(x) for x in src_lb[theirs]], dtype=np.int64), src_flat[theirs])
        self.t_wall = np.array(bc.t_wall)
        self.kinds = np.array(bc.kind)

    def _gather(self, q, lbs, flats):
        flat = q.reshape(q.shape[0], -1, 5)
        return flat[torch.as_tensor(lbs, device=q.device), torch.as_tensor(flats, device=q.device)]

    def exchange(self, q):
        me = self.part.rank
        vals = torch.empty((len(self.dst_flat), 5), dtype=q.dtype, device=q.device)
        reqs = []
        bufs = {}
        for r, (lbs, flats) in sorted(self.send.items()):
            buf = self._gather(q, lbs, flats).contiguous()
            bufs[("s", r)] = buf
            reqs.append(dist.isend(buf, dst=r, group=self.group))
        for r, sel in sorted(self.recv.items()):
            if r == me:
                continue
            buf = torch.empty((len(sel), 5), dtype=q.dtype, device=q.device)
            bufs[("r", r)] = buf
            reqs.append(dist.irecv(buf, src=r, group=self.group))
        if me in self.recv:
            vals[torch.as_tensor(self.recv[me], device=q.device)] = self._gather(q, *self.local_src)
        for rq in reqs:
            rq.wait()
        for r, sel in self.recv.items():
            if r != me:
                vals[torch.as_tensor(sel, device=q.device)] = bufs[("r", r)]
        # wall transforms in face order
        for d in range(3):
            faces = self.walls[:, d]
            for face in np.unique(faces[faces >= 0]):
                sel = torch.as_tensor(np.nonzero(faces == face)[0], device=q.device)
                if self.kinds[face] == _abi.BC_ISOTHERMAL_NOSLIP:
                    vals[sel, 1] = 2.0 * float(self.t_wall[face]) - vals[sel, 1]
                    vals[sel, 2:5] = -vals[sel, 2:5]
                else:
                    vals[sel, 2 + face // 2] = -vals[sel, 2 + face // 2]
        flat = q.view(q.shape[0], -1, 5)
        flat[torch.as_tensor(self.dst_local, device=q.device), torch.as_tensor(self.dst_flat, device=q.device)] = vals
        return q
