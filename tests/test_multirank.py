"""Multi-rank block decomposition on CPU ranks (gloo): the reference's block
partition (grid/partition.h:27-84) and the host-staged halo exchange must
reproduce the single-device ghost fill bit for bit, for periodic boxes and
for isothermal walls, at world sizes 2 and 3."""
import os
import socket
import tempfile

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from spade_gb300 import _abi
from spade_gb300.parallel import block_partition_t, halo_exchange_t
import problems as P


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, case, outdir):
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__))))
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    nblk, ncell, ng, bc = case
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, -1.0, 1.0, 0.0, 2.0))
    full = P.random_state(nblk, ncell, ng, seed=77)
    part = block_partition_t(int(np.prod(nblk)), world, rank)
    local = torch.from_numpy(full[part.starts[rank]:part.starts[rank] + part.num_local_blocks].copy())
    ex = halo_exchange_t(grid, bc, part)
    ex.exchange(local)
    np.save(os.path.join(outdir, "r%d.npy" % rank), local.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_partition_matches_reference_rule():
    p = block_partition_t(10, 3, 0)
    assert p.counts == [4, 3, 3] and p.starts == [0, 4, 7]
    assert [block_partition_t(10, 3, r).owner(b) for r in range(1) for b in range(10)] == [0, 0, 0, 0, 1, 1, 1, 2, 2, 2]
    assert block_partition_t(7, 2, 1).local_blocks() == [4, 5, 6]


@pytest.mark.parametrize("world", [2, 3])
@pytest.mark.parametrize("walls", [False, True])
def test_multirank_exchange_equals_single_device_fill(world, walls):
    from oracle import oracle as O
    nblk, ncell, ng = (3, 2, 2), (4, 3, 5), 2
    bc = P.channel_bc(290.0) if walls else P.periodic_bc()
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, -1.0, 1.0, 0.0, 2.0))
    want = P.random_state(nblk, ncell, ng, seed=77)
    O.fill_ghosts(grid, bc, want)
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_worker, args=(world, _free_port(), (nblk, ncell, ng, bc), d), nprocs=world, join=True)
        got = np.concatenate([np.load(os.path.join(d, "r%d.npy" % r)) for r in range(world)])
    assert np.array_equal(got, want)


def _leaver(rank, world, port, outdir):
    """Rank 1 leaves between steps (after the first exchange, with nothing in
    flight); rank 0's next exchange must end with an error, not hang."""
    import datetime
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__))))
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world,
                            timeout=datetime.timedelta(seconds=20))
    nblk, ncell, ng = (2, 1, 1), (4, 4, 4), 2
    grid = _abi.grid_desc(nblk, ncell, ng, (0.0, 1.0, 0.0, 1.0, 0.0, 1.0))
    full = P.random_state(nblk, ncell, ng, seed=78)
    part = block_partition_t(2, world, rank)
    local = torch.from_numpy(full[part.starts[rank]:part.starts[rank] + part.num_local_blocks].copy())
    ex = halo_exchange_t(grid, P.periodic_bc(), part)
    ex.exchange(local)
    if rank == 1:
        return                      # leaves without joining the next exchange
    try:
        ex.exchange(local)
        outcome = "completed"
    except Exception as e:          # the peer's socket closed: gloo raises
        outcome = "error: " + type(e).__name__
    with open(os.path.join(outdir, "outcome.txt"), "w") as f:
        f.write(outcome)


@pytest.mark.timeout(120)
def test_rank_that_leaves_between_steps_is_detected():
    with tempfile.TemporaryDirectory() as d:
        mp.spawn(_leaver, args=(2, _free_port(), d), nprocs=2, join=True)
        outcome = open(os.path.join(d, "outcome.txt")).read()
    assert outcome.startswith("error"), outcome
