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


# ---------------------------------------------------------------------------------------------
# perturbate: the window queue sharded over ranks, records gathered in task-id order

def _window_case():
    from modlefork_gb300 import engine, genome, perturbate

    cfg = genome.parity_config(diagonal_width=500_000)
    rng = np.random.default_rng(12)
    gen, feats1, feats2 = [], {}, {}
    for k, L in enumerate((2_400_000, 1_800_000)):
        ch = engine.Chromosome(f"chrQ{k}", L)
        gen.append((ch, engine.barriers_from_bed(ch, genome.bed_records(rng, L, 30), 0.7, 0.7)))
        for feats, tag in ((feats1, "a"), (feats2, "b")):
            pos = np.sort(rng.integers(0, L - 1000, 25))
            feats[ch.name] = [(ch.name, int(p), int(p) + 500, f"{tag}{i}", "+") for i, p in enumerate(pos)]
    features = {n: ([(f[1], f[2]) for f in feats1[n]], [(f[1], f[2]) for f in feats2[n]]) for n in feats1}
    planned = perturbate.plan_windows(cfg, gen, deletion_size=60_000, features=features, max_tasks=10)
    ref = {}
    for ch, _ in gen:
        nrows, ncols = engine.band_shape(cfg, ch.simulated_size)
        ref[ch.name] = rng.integers(0, 5, nrows * ncols).astype(np.uint32)
    return cfg, planned, feats1, feats2, ref


def _oracle_windows(cfg, planned):
    """perturbate.run_windows with the oracle's window cell as the engine."""
    from _harness import load_oracle, make_chrom
    from modlefork_gb300 import _abi as abi
    from modlefork_gb300 import engine, perturbate

    lib = load_oracle()
    out = []
    for chrom, t in planned:
        ws, we = t["window"]
        nrows, ncols = engine.band_shape(cfg, we - ws)
        band = np.zeros(nrows * ncols, dtype=np.uint32)
        st = abi.CellStats()
        ch = make_chrom(chrom.start, chrom.end, chrom.size, chrom.name.encode())
        seed = engine.cell_seed(chrom.name, chrom.size, cfg.seed, t["cell_id"])
        rc = lib.orc_simulate_window_cell(C.byref(cfg), C.byref(ch), ws, we, abi.make_barriers(t["barriers"]),
                                          len(t["barriers"]), seed, t["target_contacts"], t["target_epochs"],
                                          t["nlefs"], band.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(st))
        assert rc == 0
        out.append(perturbate.WindowResult(chrom, t, band, st))
    return out


def _window_rank_main(rank, world, port, outdir):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cfg, planned, feats1, feats2, ref = _window_case()
        lines = sharding.perturbate_sharded(cfg, planned, feats1, feats2, ref, world, rank, _oracle_windows,
                                            block_size=3)
        with open(os.path.join(outdir, f"rec{rank}.txt"), "w") as f:
            f.write("\n".join(lines))
    finally:
        dist.destroy_process_group()


def test_window_queue_over_two_gloo_ranks_equals_one_process():
    import torch.multiprocessing as mp

    from modlefork_gb300 import perturbate

    world = 2
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_window_rank_main, args=(world, _free_port(), d), nprocs=world, start_method="spawn",
                           join=True)
        got = [open(os.path.join(d, f"rec{r}.txt")).read().split("\n") for r in range(world)]
    cfg, planned, feats1, feats2, ref = _window_case()
    assert len(planned) == 10 and len({t["task_id"] for _, t in planned}) == 10
    assert [t["task_id"] for _, t in sharding.shard_windows(planned, 2, 1)] == list(range(5, 10))
    want = perturbate.perturbate_records(cfg, feats1, feats2, ref, _oracle_windows(cfg, planned), block_size=3)
    assert want and got[0] == want and got[1] == want


def _perturbate_case():
    from modlefork_gb300 import engine, genome

    cfg = genome.parity_config(diagonal_width=500_000)
    rng = np.random.default_rng(12)
    gen, feats1, feats2 = [], {}, {}
    for k, L in enumerate((2_400_000, 1_800_000)):
        ch = engine.Chromosome(f"chrQ{k}", L)
        gen.append((ch, engine.barriers_from_bed(ch, genome.bed_records(rng, L, 30), 0.7, 0.7)))
        for feats, tag in ((feats1, "a"), (feats2, "b")):
            pos = np.sort(rng.integers(0, L - 1000, 25))
            feats[ch.name] = [(ch.name, int(p), int(p) + 500, f"{tag}{i}", "+") for i, p in enumerate(pos)]
    ref = {}
    for ch, _ in gen:
        nrows, ncols = engine.band_shape(cfg, ch.simulated_size)
        ref[ch.name] = rng.integers(0, 5, nrows * ncols).astype(np.uint32)
    return cfg, gen, feats1, feats2, ref


def _perturbate_rank_main(rank, world, port, outdir):
    import sys

    sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
    import torch
    import torch.distributed as dist

    from modlefork_gb300 import perturbate

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        cfg, gen, feats1, feats2, ref = _perturbate_case()
        lines, ntasks = perturbate.run(cfg, gen, feats1, feats2, deletion_size=60_000, block_size=3, max_tasks=10,
                                       world=world, rank=rank, reference=lambda c, g: ref,
                                       windows_fn=_oracle_windows)
        if rank == 0:
            perturbate.write_bedpe(os.path.join(outdir, "ranks.bedpe"), lines)
        # the reference bands' exact sum over ranks: uint32 counts as int32, wrapping like uint32
        band = np.array([1, 2**31 + 5, 2**32 - 1, 7], dtype=np.uint32) + np.uint32(rank)
        t = torch.from_numpy(band.view(np.int32).copy())
        from modlefork_gb300 import sharding

        summed = sharding.allreduce_band_(t).numpy().view(np.uint32)
        np.save(os.path.join(outdir, f"band{rank}.npy"), summed)
    finally:
        dist.destroy_process_group()


def test_perturbate_command_over_two_gloo_ranks_writes_the_single_rank_bedpe():
    import torch.multiprocessing as mp

    from modlefork_gb300 import perturbate

    world = 2
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_perturbate_rank_main, args=(world, _free_port(), d), nprocs=world,
                           start_method="spawn", join=True)
        got = open(os.path.join(d, "ranks.bedpe")).read()
        bands = [np.load(os.path.join(d, f"band{r}.npy")) for r in range(world)]
        cfg, gen, feats1, feats2, ref = _perturbate_case()
        lines, ntasks = perturbate.run(cfg, gen, feats1, feats2, deletion_size=60_000, block_size=3, max_tasks=10,
                                       reference=lambda c, g: ref, windows_fn=_oracle_windows)
        perturbate.write_bedpe(os.path.join(d, "one.bedpe"), lines)
        want = open(os.path.join(d, "one.bedpe")).read()
    assert ntasks == 10 and len(lines) > 0 and got == want
    base = np.array([1, 2**31 + 5, 2**32 - 1, 7], dtype=np.uint64)
    expect = ((2 * base + 1) % 2**32).astype(np.uint32)
    for b in bands:
        assert np.array_equal(b, expect)
