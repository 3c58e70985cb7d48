"""1D LEF occupancy and model-state records on the GPU against the oracle, bit for bit."""

import numpy as np
import pytest

from test_outputs_cpu import run_oracle_cell, small_cell
from modlefork_gb300 import engine

pytestmark = pytest.mark.gpu

MODES = {"fast": (0, 0), "serial": (0xF, 0), "global_scratch": (0, 12 * 1024)}
FIELDS = ("epoch", "cell", "burnin", "barriers_occupied", "nbarriers", "num_lefs", "stalled_rev",
          "stalled_fwd", "stalled_both", "lef_bar", "lef_lef_primary", "lef_lef_secondary",
          "avg_loop_size")


@pytest.mark.parametrize("mode", list(MODES))
def test_occupancy_and_records_match_oracle(mode):
    cfg, chrom, bars, nl, target, te = small_cell(track_1d_lef_position=1, log_model_internal_state=1)
    n = 3
    seeds = np.array([101, 202, 303], dtype=np.uint64)
    targets = np.full(n, target, dtype=np.uint64)
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    band = np.zeros(nrows * ncols, dtype=np.uint32)
    occ = np.zeros((chrom.size + cfg.bin_size - 1) // cfg.bin_size, dtype=np.uint64)
    occ[5] = 7  # the counters are added to
    with engine.Engine(cfg) as eng:
        eng.set_debug_flags(*MODES[mode])
        cid = eng.upload_chrom(chrom, bars)
        missed, st, recs = eng.simulate_cells_ex(cid, seeds, targets, te, nl, band, occupancy=occ,
                                                 max_epoch_records=5000)
    want_band = np.zeros_like(band)
    want_occ = np.zeros_like(occ)
    want_occ[5] = 7
    for i, seed in enumerate(seeds):
        b, o, s, r = run_oracle_cell(cfg, chrom, bars, int(seed), target, te, nl, max_records=5000)
        want_band += b
        want_occ += o
        assert (st[i].epochs, st[i].contacts, st[i].rng_draws) == (s.epochs, s.contacts, s.rng_draws)
        got = [tuple(getattr(x, f) for f in FIELDS) for x in recs[i]]
        exp = [tuple((i if f == "cell" else getattr(x, f)) for f in FIELDS) for x in r]
        assert got == exp
    assert np.array_equal(band, want_band)
    assert np.array_equal(occ, want_occ)
