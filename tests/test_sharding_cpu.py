"""The multi-rank path on CPU: cell ids sharded over two gloo ranks, bands summed exactly.

Each rank runs its share of a chromosome's cells (here with the oracle as the cell engine, since
this machine has no GPU) and the all-reduced band must equal one process running every cell;
the timing reduction takes the max of the ranks' times and sums their counters."""

import ctypes as C
import os
import socket
import tempfile

import numpy as np
import pytest

from modlefork_gb300 import sharding


@pytest.mark.parametrize("n", [0, 1, 7, 64, 513])
@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_cell_ranges_partition_the_cells(n, world):
    ranges = [sharding.cell_range(n, world, r) for r in range(world)]
    ids = [i for lo, hi in ranges for i in range(lo, hi)]
    assert ids == list(range(n))
    sizes = [hi - lo for lo, hi in ranges]
    assert max(sizes) - min(sizes) <= 1


def _chrom_task():
    from modlefork_gb300 import engine, genome

    cfg, gen = genome.parity_10mbp(seed=9)
    chrom, bars = gen[0]
    n = 6
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, n)
    seeds = np.array([engine.cell_seed(chrom.name, chrom.size, cfg.seed, i) for i in range(n)], dtype=np.uint64)
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    return cfg, chrom, bars, nl, te, dict(seeds=seeds, targets=targets, nrows=nrows, ncols=ncols)


def _oracle_runner(cfg, chrom, bars, nl, te):
    from _harness import load_oracle, make_chrom
    from modlefork_gb300 import _abi as abi

    lib = load_oracle()
    bs = abi.make_barriers(bars)
    ch = make_chrom(0, chrom.end, chrom.size, chrom.name.encode())

    def run(seeds, targets, band):
        seeds = np.ascontiguousarray(seeds, dtype=np.uint64)
        targets = np.ascontiguousarray(targets, dtype=np.uint64)
        missed = C.c_uint64(0)
        rc = lib.orc_simulate_cells_mt(C.byref(cfg), C.byref(ch), bs, len(bars),
                                       seeds.ctypes.data_as(C.POINTER(C.c_uint64)),
                                       targets.ctypes.data_as(C.POINTER(C.c_uint64)), te, nl, len(seeds), 2,
                                       band.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(missed), None)
        assert rc == 0
        return missed.value

    return run


def _rank_main(rank, world, port, outdir):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cfg, chrom, bars, nl, te, task = _chrom_task()
        band, missed = sharding.simulate_chromosome_sharded(_oracle_runner(cfg, chrom, bars, nl, te), task,
                                                            world, rank)
        ms, counters = sharding.reduce_timing(10.0 + rank, {"cells": 3, "lef_epochs": 100 * (rank + 1)})
        np.save(os.path.join(outdir, f"band{rank}.npy"), band)
        np.save(os.path.join(outdir, f"meta{rank}.npy"),
                np.array([missed, ms, counters["cells"], counters["lef_epochs"]], dtype=np.float64))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_equal_one_process():
    import torch.multiprocessing as mp

    world = 2
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank_main, args=(world, _free_port(), d), nprocs=world, start_method="spawn", join=True)
        bands = [np.load(os.path.join(d, f"band{r}.npy")) for r in range(world)]
        metas = [np.load(os.path.join(d, f"meta{r}.npy")) for r in range(world)]
    cfg, chrom, bars, nl, te, task = _chrom_task()
    want = np.zeros(task["nrows"] * task["ncols"], dtype=np.uint32)
    missed = _oracle_runner(cfg, chrom, bars, nl, te)(task["seeds"], task["targets"], want)
    for b, m in zip(bands, metas):
        assert np.array_equal(b, want)
        assert m[0] == missed
        assert m[1] == 11.0 and m[2] == 6 and m[3] == 300
