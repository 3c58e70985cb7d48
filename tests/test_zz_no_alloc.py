"""mgpu_simulate_cells_noalloc: the allocation-free variant of mgpu_simulate_cells.

It runs the same simulation kernel with its task list, work counter and cell slots in a
fixed scratch array of the library, so two calls in a row must each give exactly what the
allocating entry point gives for the same cells.  The file is named to be collected last, so
the test also runs after every other test of the session has used the device.
"""

import ctypes as C

import numpy as np
import pytest

from modlefork_gb300 import _abi as abi
from modlefork_gb300 import engine, genome

pytestmark = pytest.mark.gpu


def _cells(n, seed=9):
    cfg, gen = genome.parity_10mbp(seed=seed)
    chrom, bars = gen[0]
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, n)
    seeds = np.array([engine.cell_seed(chrom.name, chrom.size, cfg.seed, i) for i in range(n)], dtype=np.uint64)
    return cfg, chrom, bars, nl, seeds, targets, te


def _stats_tuple(s):
    return (s.epochs, s.burnin_epochs, s.contacts, s.missed_updates, s.lef_epochs, s.rng_draws, s.status)


@pytest.mark.parametrize("smem_budget", [0, 12 * 1024])
def test_noalloc_twice_matches_simulate_cells(smem_budget):
    """Also with the per-LEF arrays in global cell slots, which then live in the fixed scratch."""
    torch = pytest.importorskip("torch")
    n = 24
    cfg, chrom, bars, nl, seeds, targets, te = _cells(n)
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    ref_band = np.zeros(nrows * ncols, dtype=np.uint32)
    dev = torch.device("cuda", 0)
    d_seeds = torch.from_numpy(seeds.view(np.int64)).to(dev)
    d_targets = torch.from_numpy(targets.view(np.int64)).to(dev)
    stat_bytes = C.sizeof(abi.CellStats)
    outs = []
    for _ in range(2):
        outs.append(dict(band=torch.zeros(nrows * ncols, dtype=torch.int32, device=dev),
                         missed=torch.zeros(1, dtype=torch.int64, device=dev),
                         stats=torch.zeros(n * stat_bytes, dtype=torch.uint8, device=dev)))
    torch.cuda.synchronize()
    with engine.Engine(cfg) as eng:
        eng.set_debug_flags(0, smem_budget)
        cid = eng.upload_chrom(chrom, bars)
        ref_missed, ref_stats = eng.simulate_cells(cid, seeds, targets, te, nl, ref_band)
        for o in outs:  # two calls in a row on the context's stream, no sync in between
            eng.simulate_cells_noalloc(cid, d_seeds.data_ptr(), d_targets.data_ptr(), te, nl, n,
                                       o["band"].data_ptr(), o["missed"].data_ptr(), o["stats"].data_ptr())
        eng.sync()
    for o in outs:
        assert np.array_equal(o["band"].cpu().numpy().view(np.uint32), ref_band)
        assert int(o["missed"].item()) == ref_missed
        raw = o["stats"].cpu().numpy().tobytes()
        got = [abi.CellStats.from_buffer_copy(raw[i * stat_bytes:(i + 1) * stat_bytes]) for i in range(n)]
        assert [_stats_tuple(s) for s in got] == [_stats_tuple(s) for s in ref_stats]
    assert all(s.status == 0 for s in ref_stats)


def test_noalloc_rejects_what_it_cannot_hold():
    torch = pytest.importorskip("torch")
    n = 4
    cfg, chrom, bars, nl, seeds, targets, te = _cells(n)
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    dev = torch.device("cuda", 0)
    d_seeds = torch.from_numpy(seeds.view(np.int64)).to(dev)
    d_targets = torch.from_numpy(targets.view(np.int64)).to(dev)
    d_band = torch.zeros(nrows * ncols, dtype=torch.int32, device=dev)
    host_band = np.zeros(nrows * ncols, dtype=np.uint32)
    with engine.Engine(cfg) as eng:
        cid = eng.upload_chrom(chrom, bars)
        with pytest.raises(engine.EngineError) as e:
            eng.simulate_cells_noalloc(cid, d_seeds.data_ptr(), d_targets.data_ptr(), te, nl,
                                       abi.MGPU_NOALLOC_MAX_CELLS + 1, d_band.data_ptr())
        assert e.value.code == abi.MGPU_ERR_INVALID_ARG and "at most" in str(e.value)
        with pytest.raises(engine.EngineError) as e:
            eng.simulate_cells_noalloc(cid, d_seeds.data_ptr(), d_targets.data_ptr(), te, nl, n,
                                       host_band.ctypes.data)
        assert e.value.code == abi.MGPU_ERR_INVALID_ARG and "device pointer" in str(e.value)
        eng.sync()
    assert int(d_band.sum().item()) == 0  # nothing was issued
