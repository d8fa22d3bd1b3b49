"""Checkpoint format: raw per-block AoS5 memory (ghosts included) at
lb_glob * block_bytes (io/io_native.h:15-55)."""
import os
import tempfile

import numpy as np

from spade_gb300 import io
from spade_gb300.parallel import block_partition_t
import problems as P


def test_round_trip_and_layout():
    q = P.random_state((2, 3, 1), (4, 5, 3), 2, seed=5)
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "check.bin")
        io.binary_write(f, q)
        raw = np.fromfile(f, dtype=np.float64)
        assert raw.size == q.size and np.array_equal(raw, q.ravel())   # block lb at lb*block_bytes
        r = np.zeros_like(q)
        io.binary_read(f, r)
        assert np.array_equal(r, q)


def test_partitioned_ranks_write_one_file():
    nblk = (5, 1, 1)
    q = P.random_state(nblk, (4, 4, 4), 2, seed=6)
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "check.bin")
        for rank in (1, 0):                                  # any order
            part = block_partition_t(5, 2, rank)
            local = q[part.starts[rank]:part.starts[rank] + part.num_local_blocks]
            io.binary_write(f, local, first_block=part.starts[rank])
        whole = np.zeros_like(q)
        io.binary_read(f, whole)
        assert np.array_equal(whole, q)
        part = block_partition_t(5, 2, 1)
        mine = np.zeros((part.num_local_blocks,) + q.shape[1:])
        io.binary_read(f, mine, first_block=part.starts[1])
        assert np.array_equal(mine, q[part.starts[1]:])


def _tgv_small():
    from oracle import oracle as O
    nblk, ncell, ng = (2, 1, 1), (8, 8, 8), 2
    grid = P.tgv_grid(nblk, ncell, ng)
    tables = P.tgv_tables(nblk, ncell, ng)
    q = P.tgv_state(nblk, ncell, ng, tables, seed=4)
    O.fill_ghosts(grid, P.periodic_bc(), q)
    return grid, q, P.tgv_dt(q, grid, ng)


def test_resume_from_checkpoint_is_bitwise_identical_oracle():
    """Checkpoint after 3 SSPRK3 steps, restart from the file, run 4 more:
    the state equals 7 uninterrupted steps bit for bit (the checkpoint holds
    the ghosts too, so nothing is recomputed on restart)."""
    from oracle import oracle as O
    grid, q, dt = _tgv_small()
    s = P.tgv_scheme()
    work = np.zeros((3,) + q.shape)
    full = q.copy()
    for _ in range(7):
        O.ssprk3_step(grid, s, P.periodic_bc(), full, work, dt)
    for _ in range(3):
        O.ssprk3_step(grid, s, P.periodic_bc(), q, work, dt)
    with tempfile.TemporaryDirectory() as d:
        f = os.path.join(d, "restart.bin")
        io.binary_write(f, q)
        r = np.full_like(q, np.nan)
        io.binary_read(f, r)
    for _ in range(4):
        O.ssprk3_step(grid, s, P.periodic_bc(), r, work, dt)
    assert np.array_equal(r, full)
