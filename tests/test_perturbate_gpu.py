"""modle perturbate windows on the batched GPU engine against the oracle's window cell."""

import ctypes as C

import numpy as np
import pytest

from _harness import load_oracle, make_chrom
from modlefork_gb300 import _abi as abi
from modlefork_gb300 import engine, genome, perturbate

pytestmark = pytest.mark.gpu


def test_windows_match_oracle():
    cfg = genome.parity_config(diagonal_width=500_000)
    rng = np.random.default_rng(4)
    chroms = []
    for k, L in enumerate((3_000_000, 2_200_000)):
        ch = engine.Chromosome(f"chrP{k}", L)
        chroms.append((ch, engine.barriers_from_bed(ch, genome.bed_records(rng, L, 40), 0.7, 0.7)))
    res = perturbate.simulate_windows(cfg, chroms, deletion_size=30_000, max_tasks=48)
    assert len(res) == 48
    lib = load_oracle()
    for r in res:
        t = r.task
        ws, we = t["window"]
        nrows, ncols = engine.band_shape(cfg, we - ws)
        band = np.zeros(nrows * ncols, dtype=np.uint32)
        st = abi.CellStats()
        bs = abi.make_barriers(t["barriers"])
        ch = make_chrom(r.chrom.start, r.chrom.end, r.chrom.size, r.chrom.name.encode())
        seed = engine.cell_seed(r.chrom.name, r.chrom.size, cfg.seed, t["cell_id"])
        rc = lib.orc_simulate_window_cell(C.byref(cfg), C.byref(ch), ws, we, bs, len(t["barriers"]), seed,
                                          t["target_contacts"], t["target_epochs"], t["nlefs"],
                                          band.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(st))
        assert rc == 0
        assert (r.stats.epochs, r.stats.contacts, r.stats.rng_draws, r.stats.missed_updates) == \
               (st.epochs, st.contacts, st.rng_draws, st.missed_updates), t["cell_id"]
        assert np.array_equal(r.band, band), t["cell_id"]
    assert any(r.task["active_barriers"] < len(r.task["barriers"]) for r in res)
