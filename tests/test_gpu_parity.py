"""GPU parity: the CUDA path against the reference's known-answer tests and against the CPU
oracle, bit for bit.

* The reference's step-level unit tests (tests/golden) run through mgpu_run_phase.
* Whole cells run through mgpu_trace_cell; every epoch's state digest, draw count, burn-in
  and contact counters, and the cell's contact band must equal the oracle's.  The cell
  configurations stress the rare paths: full rank ties, chromosome ends, soft barriers,
  LEF bypass, Poisson PTRS and binomial BTRD, loop-only / TAD-only sampling, fixed speeds,
  the epoch stopping criterion.
* A batch of cells through mgpu_simulate_cells: per-cell statistics and the summed band.
"""

import ctypes as C

import numpy as np
import pytest

from _harness import (check_golden, golden_inputs, load_golden_cases, load_oracle, make_chrom,
                      run_golden_case)
from modlefork_gb300 import _abi as abi
from modlefork_gb300 import engine, genome

pytestmark = pytest.mark.gpu

CASES = load_golden_cases()


# execution modes of the engine: warp-parallel steps, the serial restatements forced, and the
# per-LEF arrays moved to global scratch (the layout of very large cells)
MODES = {"fast": (0, 0), "serial": (0xF, 0), "global_scratch": (0, 12 * 1024)}


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("case", CASES, ids=[c["name"] for c in CASES])
def test_gpu_matches_reference_unit_test(case, mode):
    overrides, chrom, barriers, _ = golden_inputs(case)
    cfg = engine.config_defaults(**overrides)
    with engine.Engine(cfg) as eng:
        eng.set_debug_flags(*MODES[mode])
        cid = eng.upload_chrom(engine.Chromosome("chr1", chrom["size"], chrom["start"], chrom["end"]),
                               barriers)
        st = run_golden_case(case, lambda phase, io: eng.run_phase(cid, phase, io))
    check_golden(case, st)


def oracle_trace(cfg, chrom, bars, seed, target, te, nl, max_epochs, max_records=0):
    lib = load_oracle()
    tr = abi.TraceRequest()
    hdr = (abi.TraceHeader * max_epochs)()
    tr.max_epochs = max_epochs
    tr.all_headers = hdr
    arrays = {}
    rec_h = (abi.TraceHeader * max(1, max_records))()
    if max_records:
        tr.max_records = max_records
        tr.headers = rec_h
        for name in abi.TRACE_ARRAYS:
            a = np.zeros(max_records * nl, dtype=np.uint64)
            arrays[name] = a
            setattr(tr, name, abi.ptr64(a))
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    band = np.zeros(nrows * ncols, dtype=np.uint32)
    st = abi.CellStats()
    bs = abi.make_barriers(bars)
    rc = lib.orc_simulate_cell(C.byref(cfg), C.byref(make_chrom(chrom.start, chrom.end, chrom.size,
                                                                chrom.name.encode())),
                               bs, len(bars), seed, target, te, nl,
                               band.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(st), C.byref(tr))
    return rc, st, hdr, tr.num_epochs_recorded, band, arrays


def first_divergence(g_arrays, o_arrays, nl, nrec):
    for k in range(nrec):
        for name in abi.TRACE_ARRAYS:
            a = g_arrays[name][k * nl:(k + 1) * nl]
            b = o_arrays[name][k * nl:(k + 1) * nl]
            if not np.array_equal(a, b):
                i = int(np.nonzero(a != b)[0][0])
                return f"epoch {k} {name}[{i}]: gpu {a[i]} oracle {b[i]}"
    return "no difference in the recorded arrays"


def compare_cell(cfg, chrom, bars, cell_id=0, nl=None, max_epochs=20000, target=None, mode="fast"):
    nl = nl or engine.num_lefs(cfg, chrom.simulated_size)
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, int(cfg.num_cells))
    target = int(targets[min(cell_id, len(targets) - 1)]) if target is None else target
    seed = engine.cell_seed(chrom.name, chrom.size, cfg.seed, cell_id)
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    gband = np.zeros(nrows * ncols, dtype=np.uint32)
    with engine.Engine(cfg) as eng:
        eng.set_debug_flags(*MODES[mode])
        cid = eng.upload_chrom(chrom, bars)
        gst, _, _, ghdr, gn = eng.trace_cell(cid, seed, target, te, nl, max_epochs=max_epochs, band=gband)
        rc, ost, ohdr, on, oband, _ = oracle_trace(cfg, chrom, bars, seed, target, te, nl, max_epochs)
        assert rc == 0
        assert gn == on, f"epochs recorded: gpu {gn} oracle {on}"
        for k in range(gn):
            g, o = ghdr[k], ohdr[k]
            if (g.digest, g.rng_draws, g.num_active_lefs, g.num_contacts, g.burnin_completed,
                    g.n5prime, g.n3prime) != (o.digest, o.rng_draws, o.num_active_lefs, o.num_contacts,
                                              o.burnin_completed, o.n5prime, o.n3prime):
                # re-run both with full records around the first divergent epoch for the report
                lo = k + 1
                _, _, garr, _, _ = eng.trace_cell(cid, seed, target, te, nl, max_records=lo)
                _, _, _, _, _, oarr = oracle_trace(cfg, chrom, bars, seed, target, te, nl, 1, lo)
                pytest.fail(f"epoch {k}: gpu (draws {g.rng_draws}, active {g.num_active_lefs}, "
                            f"contacts {g.num_contacts}) vs oracle (draws {o.rng_draws}, active "
                            f"{o.num_active_lefs}, contacts {o.num_contacts}); "
                            + first_divergence(garr, oarr, nl, lo))
    assert (gst.epochs, gst.burnin_epochs, gst.contacts, gst.missed_updates, gst.lef_epochs,
            gst.rng_draws) == (ost.epochs, ost.burnin_epochs, ost.contacts, ost.missed_updates,
                               ost.lef_epochs, ost.rng_draws)
    assert gst.status == 0
    assert np.array_equal(gband, oband)
    return gst


def small_genome(cfg, length, nbarriers, seed, occupancy=None, name="chrT", start=0):
    rng = np.random.default_rng(seed)
    chrom = engine.Chromosome(name, length + start, start, length + start)
    occ = rng.beta(8.0, 2.0, size=nbarriers) if occupancy == "beta" else None
    recs = genome.bed_records(rng, length, nbarriers, occ)
    recs = [(s + start, e + start, st, sc) for s, e, st, sc in recs]
    bars = engine.barriers_from_bed(chrom, recs, cfg.barrier_occupied_stp, cfg.barrier_not_occupied_stp)
    return chrom, bars


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("cell", [0, 1, 17, 63])
def test_parity_10mbp_cell(cell, mode):
    cfg, gen = genome.parity_10mbp(seed=7)
    chrom, bars = gen[0]
    st = compare_cell(cfg, chrom, bars, cell_id=cell, mode=mode)
    assert st.burnin_epochs > 100 and st.contacts > 0


STRESS = {
    # tiny chromosome crowded with LEFs: boundary pile-ups, full rank ties, many collisions
    "crowded": (dict(number_of_lefs_per_mbp=2000.0, avg_lef_processivity=20000, bin_size=1000,
                     diagonal_width=100000, num_cells=1), 50_000, 40, None),
    # soft barriers and frequent bypass: LEF-BAR trials that draw
    "soft_barriers": (dict(lef_bar_minor_collision_pblock=0.4, lef_bar_major_collision_pblock=0.8,
                           probability_of_extrusion_unit_bypass=0.3), 2_000_000, 300, "beta"),
    # many LEFs, short burn-in: Poisson PTRS (mean >= 10) and binomial BTRD (m >= 11)
    "ptrs_btrd": (dict(number_of_lefs_per_mbp=400.0, burnin_target_epochs_for_lef_activation=0,
                       contact_sampling_interval=2000, avg_lef_processivity=50000, num_cells=1),
                  1_000_000, 100, "beta"),
    "loop_only": (dict(contact_sampling_strategy=abi.CS_LOOP | abi.CS_NOISIFY), 2_000_000, 50, None),
    "tad_only_no_noise": (dict(contact_sampling_strategy=abi.CS_TAD), 2_000_000, 50, None),
    "fixed_speed": (dict(rev_extrusion_speed_std=0.0, fwd_extrusion_speed_std=0.0), 2_000_000, 80, None),
    "skip_burnin_epochs": (dict(skip_burnin=1, stop_on_epochs=1, target_simulation_epochs=300,
                                num_cells=4), 2_000_000, 80, "beta"),
    "offset_start": (dict(), 3_000_000, 60, None),
    # no barriers at all: LEF-BAR sweeps over an empty track
    "no_barriers": (dict(), 2_000_000, 0, None),
    # the 1D occupancy and model-state outputs enabled (more draws per epoch)
    "outputs_on": (dict(track_1d_lef_position=1, log_model_internal_state=1), 2_000_000, 40, "beta"),
}


@pytest.mark.parametrize("mode", list(MODES))
@pytest.mark.parametrize("name", list(STRESS))
def test_stress_cell(name, mode):
    ov, length, nb, occ = STRESS[name]
    ov = dict(ov)
    burn_target = ov.pop("burnin_target_epochs_for_lef_activation", None)
    cfg = genome.parity_config(**ov)
    if burn_target is not None:  # set after transform: a short activation phase
        cfg.burnin_target_epochs_for_lef_activation = 20
    start = 1_234_567 if name == "offset_start" else 0
    chrom, bars = small_genome(cfg, length, nb, seed=sum(map(ord, name)), occupancy=occ, start=start)
    for cell in (0, 5):
        compare_cell(cfg, chrom, bars, cell_id=cell, max_epochs=50000, mode=mode)


def test_batch_matches_oracle_cells():
    """64 cells in one launch: per-cell stats and the summed band equal the oracle's."""
    cfg, gen = genome.parity_10mbp(seed=9)
    chrom, bars = gen[0]
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    n = 64
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, n)
    seeds = np.array([engine.cell_seed(chrom.name, chrom.size, cfg.seed, i) for i in range(n)], dtype=np.uint64)
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    gband = np.zeros(nrows * ncols, dtype=np.uint32)
    with engine.Engine(cfg) as eng:
        cid = eng.upload_chrom(chrom, bars)
        gmissed, gst = eng.simulate_cells(cid, seeds, targets, te, nl, gband)
    lib = load_oracle()
    oband = np.zeros_like(gband)
    ost = (abi.CellStats * n)()
    omissed = C.c_uint64(0)
    bs = abi.make_barriers(bars)
    rc = lib.orc_simulate_cells_mt(C.byref(cfg), C.byref(make_chrom(0, chrom.end, chrom.size, b"chrS")), bs,
                                   len(bars), seeds.ctypes.data_as(C.POINTER(C.c_uint64)),
                                   targets.ctypes.data_as(C.POINTER(C.c_uint64)), te, nl, n, 8,
                                   oband.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(omissed), ost)
    assert rc == 0
    for i in range(n):
        g, o = gst[i], ost[i]
        assert (g.epochs, g.burnin_epochs, g.contacts, g.lef_epochs, g.rng_draws) == \
               (o.epochs, o.burnin_epochs, o.contacts, o.lef_epochs, o.rng_draws), i
    assert gmissed == omissed.value
    assert np.array_equal(gband, oband)
    assert int(gband.sum()) + gmissed == int(targets.sum())


def test_host_buffers_accumulate_into_band():
    """The band argument is added to, like the reference's shared ContactMatrixDense."""
    cfg, gen = genome.parity_10mbp(seed=9)
    chrom, bars = gen[0]
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, 4)
    seeds = np.arange(4, dtype=np.uint64) + 99
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    band = np.zeros(nrows * ncols, dtype=np.uint32)
    with engine.Engine(cfg) as eng:
        cid = eng.upload_chrom(chrom, bars)
        eng.simulate_cells(cid, seeds, targets, te, nl, band)
        once = band.copy()
        eng.simulate_cells(cid, seeds, targets, te, nl, band)
    assert np.array_equal(band, 2 * once)


def test_concurrent_contexts_match_one_context():
    """Chromosome launches from several contexts at once (threads, streams, a shared-memory
    budget that moves arrays to global slots) give the same bands and cells as one context."""
    from modlefork_gb300 import simulate

    cfg, gen = genome.genome_24chr(seed=5, nchroms=4, min_len=2_000_000, max_len=6_000_000)
    cfg.num_cells = 16
    one = simulate.simulate_genome(cfg, gen, workers=1)
    many = simulate.simulate_genome(cfg, gen, workers=3, smem_budget=12 * 1024)
    assert [r.chrom.name for r in one] == [r.chrom.name for r in many]
    for a, b in zip(one, many):
        assert np.array_equal(a.band, b.band), a.chrom.name
        assert a.missed == b.missed
        assert [(s.epochs, s.contacts, s.rng_draws) for s in a.stats] == \
               [(s.epochs, s.contacts, s.rng_draws) for s in b.stats]


def test_device_buffers_match_host_buffers():
    """Seeds, targets and band given as device pointers (torch tensors) give the same band
    and statistics as host arrays, on a caller's stream."""
    torch = pytest.importorskip("torch")
    cfg, gen = genome.parity_10mbp(seed=9)
    chrom, bars = gen[0]
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    n = 8
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, n)
    seeds = np.arange(n, dtype=np.uint64) + 1234
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    hband = np.zeros(nrows * ncols, dtype=np.uint32)
    dev = torch.device("cuda", 0)
    d_seeds = torch.from_numpy(seeds.view(np.int64)).to(dev)
    d_targets = torch.from_numpy(targets.view(np.int64)).to(dev)
    d_band = torch.zeros(nrows * ncols, dtype=torch.int32, device=dev)
    stream = torch.cuda.Stream()
    with engine.Engine(cfg) as eng:
        cid = eng.upload_chrom(chrom, bars)
        hm, hst = eng.simulate_cells(cid, seeds, targets, te, nl, hband)
        with pytest.raises(ValueError):
            eng.simulate_cells(cid, d_seeds.data_ptr(), d_targets.data_ptr(), te, nl, d_band.data_ptr())
        eng.set_stream(stream.cuda_stream)
        dm, dst = eng.simulate_cells(cid, d_seeds.data_ptr(), d_targets.data_ptr(), te, nl,
                                     d_band.data_ptr(), ncells=n)
    torch.cuda.synchronize()
    assert dm == hm
    assert [(s.epochs, s.contacts, s.rng_draws) for s in dst] == [(s.epochs, s.contacts, s.rng_draws) for s in hst]
    assert np.array_equal(d_band.cpu().numpy().view(np.uint32), hband)


def test_unreachable_contacts_end_with_timeout_status():
    """A chromosome where no LEF can ever be inside (start + 1, end - 1) would make the
    reference loop forever; the device gives up after its attempt budget and reports it."""
    cfg = genome.parity_config(skip_burnin=1)
    chrom = engine.Chromosome("chrZ", 3)
    with engine.Engine(cfg) as eng:
        cid = eng.upload_chrom(chrom, [])
        band = np.zeros(1, dtype=np.uint32)
        with pytest.raises(engine.EngineError) as e:
            eng.simulate_cells(cid, np.array([1], dtype=np.uint64), np.array([10], dtype=np.uint64), 0, 4, band)
    assert e.value.code == abi.MGPU_ERR_TIMEOUT


@pytest.mark.parametrize("mode", ["fast", "global_scratch"])
def test_largest_genome_chromosome_cell(mode):
    """The genome workload's largest chromosome (246 Mbp, 4918 LEFs and barriers): one whole
    cell, every epoch, against the oracle."""
    cfg, gen = genome.genome_24chr(seed=11)
    chrom, bars = max(gen, key=lambda cb: cb[0].size)
    assert chrom.size > 240_000_000
    compare_cell(cfg, chrom, bars, cell_id=3, max_epochs=5000, mode=mode)


@pytest.mark.parametrize("mode", list(MODES))
def test_batched_launch_matches_per_chromosome_launches(mode):
    """One batched launch over several chromosomes (and two LEF counts on one of them) gives
    the bands, missed updates and per-cell results of one launch per (chromosome, LEF count)."""
    cfg, gen = genome.genome_24chr(seed=5, nchroms=3, min_len=2_000_000, max_len=6_000_000)
    n = 12
    with engine.Engine(cfg) as eng:
        eng.set_debug_flags(*MODES[mode])
        tasks, bands, want = [], {}, []
        for chrom, bars in gen:
            cid = eng.upload_chrom(chrom, bars)
            nl = engine.num_lefs(cfg, chrom.simulated_size)
            nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
            for nl_k in ((nl, nl + 7) if cid == 1 else (nl,)):
                targets, te = engine.task_targets(cfg, chrom.simulated_size, nl_k, n)
                seeds = np.array([engine.cell_seed(chrom.name, chrom.size, cfg.seed, i) for i in range(n)],
                                 dtype=np.uint64) + nl_k
                band = np.zeros(nrows * ncols, dtype=np.uint32)
                m, st = eng.simulate_cells(cid, seeds, targets, te, nl_k, band)
                want.append((cid, band, m, [(s.epochs, s.contacts, s.rng_draws) for s in st]))
                bands.setdefault(cid, np.zeros(nrows * ncols, dtype=np.uint32))
                tasks += [(cid, int(sd), int(tg), te, nl_k) for sd, tg in zip(seeds, targets)]
        perm = np.random.default_rng(1).permutation(len(tasks))  # task order does not matter
        missed, st = eng.simulate_batch([tasks[i] for i in perm], bands)
    got = {}
    for j, i in enumerate(perm):
        got[i] = (st[j].epochs, st[j].contacts, st[j].rng_draws)
    k = 0
    sums, msums = {}, {}
    for cid, band, m, stats in want:
        assert [got[k + t] for t in range(n)] == stats
        k += n
        sums[cid] = sums.get(cid, 0) + band.astype(np.uint64)
        msums[cid] = msums.get(cid, 0) + m
    for cid in bands:
        assert np.array_equal(bands[cid].astype(np.uint64), sums[cid])
        assert missed[cid] == msums[cid]
