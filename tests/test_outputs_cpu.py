"""Optional outputs of a cell in the oracle: the 1D LEF occupancy (register_1d_lef_occupancy,
register_contacts.cpp:200-232) and the per-epoch model-state records (Simulation::dump_stats,
simulation.cpp:1166-1224).  Properties the reference's code implies."""

import ctypes as C

import numpy as np

from _harness import load_oracle, make_chrom
from modlefork_gb300 import _abi as abi
from modlefork_gb300 import genome


def run_oracle_cell(cfg, chrom, bars, seed, target, te, nl, max_records=0):
    lib = load_oracle()
    nrows = min((cfg.diagonal_width + cfg.bin_size - 1) // cfg.bin_size,
                (chrom.end - chrom.start + cfg.bin_size - 1) // cfg.bin_size)
    ncols = (chrom.end - chrom.start + cfg.bin_size - 1) // cfg.bin_size
    band = np.zeros(nrows * ncols, dtype=np.uint32)
    occ = np.zeros((chrom.size + cfg.bin_size - 1) // cfg.bin_size, dtype=np.uint64)
    st = abi.CellStats()
    recs = (abi.EpochRecord * max(1, max_records))()
    nrec = C.c_uint64()
    bs = abi.make_barriers(bars)
    ch = make_chrom(chrom.start, chrom.end, chrom.size, chrom.name.encode())
    rc = lib.orc_simulate_cell_ex(C.byref(cfg), C.byref(ch), bs, len(bars), seed, target, te, nl,
                                  band.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(st), None,
                                  occ.ctypes.data, C.addressof(recs), max_records, 3, C.byref(nrec))
    assert rc == 0
    return band, occ, st, [recs[k] for k in range(nrec.value)]


def small_cell(**overrides):
    cfg, gen = genome.parity_10mbp(seed=9, **overrides)
    chrom, bars = gen[0]
    from modlefork_gb300 import engine
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, 64)
    return cfg, chrom, bars, nl, int(targets[0]), te


def test_occupancy_counts_two_bins_per_sampling_event():
    cfg, chrom, bars, nl, target, te = small_cell(track_1d_lef_position=1)
    band, occ, st, _ = run_oracle_cell(cfg, chrom, bars, 77, target, te, nl)
    assert int(occ.sum()) == 2 * st.contacts
    # tracking consumes draws, so it changes the cell's contacts but not their number
    cfg0, *_ = small_cell()
    band0, occ0, st0, _ = run_oracle_cell(cfg0, chrom, bars, 77, target, te, nl)
    assert int(occ0.sum()) == 0
    assert st.contacts == st0.contacts
    assert st.rng_draws > st0.rng_draws


def test_model_state_records():
    cfg, chrom, bars, nl, target, te = small_cell(log_model_internal_state=1)
    _, _, st, recs = run_oracle_cell(cfg, chrom, bars, 78, target, te, nl, max_records=10_000)
    # one record per epoch that reached extrude: all but the last (which stops at the target)
    assert len(recs) == st.epochs
    assert [r.epoch for r in recs] == list(range(st.epochs))
    # the epoch whose run_burnin completes the burn-in counts as a burn-in epoch but logs False
    assert sum(r.burnin for r in recs) == st.burnin_epochs - 1
    for r in recs:
        assert r.cell == 3 and r.nbarriers == len(bars) and r.barriers_occupied <= r.nbarriers
        assert r.stalled_both <= min(r.stalled_rev, r.stalled_fwd)
        assert r.lef_bar + r.lef_lef_primary + r.lef_lef_secondary <= r.stalled_rev + r.stalled_fwd
        assert r.avg_loop_size >= 0
    # logging draws nothing: the cell is unchanged
    cfg0, *_ = small_cell()
    _, _, st0, recs0 = run_oracle_cell(cfg0, chrom, bars, 78, target, te, nl, max_records=10)
    assert (st0.epochs, st0.contacts, st0.rng_draws) == (st.epochs, st.contacts, st.rng_draws)
    assert recs0 == []
