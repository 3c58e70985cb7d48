"""The batched workload's windows: uneven lengths, each window with its own bin size, LEF
density and barrier density, all advanced in one mgpu_simulate_batch launch.

Every window's cells must come out exactly as a plain per-window launch on an engine created
with that window's configuration gives them (bands, missed updates, per-cell results), and the
smallest windows are also checked against the oracle cell by cell.
"""

import ctypes as C

import numpy as np
import pytest

from modlefork_gb300 import _abi as abi
from modlefork_gb300 import engine, genome

from _harness import load_oracle, make_chrom

pytestmark = pytest.mark.gpu

NCELLS = 3


def _windows():
    return genome.batched_windows(seed=3, nwindows=10, min_len=1_000_000, max_len=12_000_000, cells=NCELLS)


def _tasks(cfg, chrom):
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, NCELLS)
    seeds = [engine.cell_seed(chrom.name, chrom.size, cfg.seed, i) for i in range(NCELLS)]
    return nl, seeds, [int(t) for t in targets], te


def _key(s):
    return (s.epochs, s.burnin_epochs, s.contacts, s.missed_updates, s.lef_epochs, s.rng_draws, s.status)


@pytest.mark.parametrize("smem_budget", [0, 12 * 1024])
def test_heterogeneous_windows_in_one_batch(smem_budget):
    wins = _windows()
    assert len({cfg.bin_size for cfg, _, _ in wins}) > 1  # the batch really mixes configurations
    want = []
    for cfg, chrom, bars in wins:
        nl, seeds, targets, te = _tasks(cfg, chrom)
        nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
        band = np.zeros(nrows * ncols, dtype=np.uint32)
        with engine.Engine(cfg) as eng:
            eng.set_debug_flags(0, smem_budget)
            cid = eng.upload_chrom(chrom, bars)
            m, st = eng.simulate_cells(cid, np.array(seeds, dtype=np.uint64), np.array(targets, dtype=np.uint64),
                                       te, nl, band)
        want.append((band, m, [_key(s) for s in st]))
    # one launch on an engine whose own configuration matches none of the windows
    with engine.Engine(genome.genome_config(bin_size=3000)) as eng:
        eng.set_debug_flags(0, smem_budget)
        tasks, bands = [], {}
        for cfg, chrom, bars in wins:
            cid = eng.upload_chrom(chrom, bars)
            eng.set_chrom_config(cid, cfg)
            nl, seeds, targets, te = _tasks(cfg, chrom)
            nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
            bands[cid] = np.zeros(nrows * ncols, dtype=np.uint32)
            tasks += [(cid, sd, tg, te, nl) for sd, tg in zip(seeds, targets)]
        perm = np.random.default_rng(2).permutation(len(tasks))
        missed, st = eng.simulate_batch([tasks[i] for i in perm], bands)
    got = [None] * len(tasks)
    for j, i in enumerate(perm):
        got[i] = _key(st[j])
    for w, (band, m, stats) in enumerate(want):
        assert got[w * NCELLS:(w + 1) * NCELLS] == stats, f"window {w}"
        assert np.array_equal(bands[w], band), f"window {w}"
        assert missed[w] == m
    assert all(s[-1] == 0 for s in got)


def test_heterogeneous_windows_match_the_oracle():
    lib = load_oracle()
    wins = sorted(_windows(), key=lambda w: w[1].size)[:3]
    with engine.Engine(genome.genome_config()) as eng:
        tasks, bands, cids = [], {}, []
        for cfg, chrom, bars in wins:
            cid = eng.upload_chrom(chrom, bars)
            eng.set_chrom_config(cid, cfg)
            nl, seeds, targets, te = _tasks(cfg, chrom)
            nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
            bands[cid] = np.zeros(nrows * ncols, dtype=np.uint32)
            tasks.append((cid, seeds[1], targets[1], te, nl))
            cids.append(cid)
        _, st = eng.simulate_batch(tasks, bands)
    for k, (cfg, chrom, bars) in enumerate(wins):
        _, seed, target, te, nl = tasks[k]
        band = np.zeros_like(bands[cids[k]])
        ost = abi.CellStats()
        rc = lib.orc_simulate_cell(C.byref(cfg), C.byref(make_chrom(chrom.start, chrom.end, chrom.size,
                                                                    chrom.name.encode())),
                                   abi.make_barriers(bars), len(bars), seed, target, te, nl,
                                   band.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(ost), None)
        assert rc == 0
        assert _key(st[k]) == _key(ost)
        assert np.array_equal(bands[cids[k]], band)


def test_chrom_config_is_validated_and_can_be_reset():
    cfg, gen = genome.parity_10mbp()
    chrom, bars = gen[0]
    with engine.Engine(cfg) as eng:
        cid = eng.upload_chrom(chrom, bars)
        bad = genome.parity_config()
        bad.bin_size = 0
        with pytest.raises(engine.EngineError) as e:
            eng.set_chrom_config(cid, bad)
        assert e.value.code == abi.MGPU_ERR_INVALID_ARG
        with pytest.raises(engine.EngineError):
            eng.set_chrom_config(cid + 5, cfg)
        # an override equal to the context's configuration and a reset both leave the cells as they were
        nl = engine.num_lefs(cfg, chrom.simulated_size)
        targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, 2)
        seeds = np.array([engine.cell_seed(chrom.name, chrom.size, cfg.seed, i) for i in range(2)], dtype=np.uint64)
        nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
        outs = []
        for step in range(3):
            if step == 1:
                eng.set_chrom_config(cid, genome.parity_config())
            if step == 2:
                eng.set_chrom_config(cid, None)
            band = np.zeros(nrows * ncols, dtype=np.uint32)
            m, st = eng.simulate_cells(cid, seeds, targets, te, nl, band)
            outs.append((band, m, [_key(s) for s in st]))
    for band, m, st in outs[1:]:
        assert np.array_equal(band, outs[0][0]) and m == outs[0][1] and st == outs[0][2]
