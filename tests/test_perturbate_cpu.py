"""Window and deletion generation of modle perturbate (scheduler_perturbate.cpp:186-372,
scheduler_common.cpp:51-127), restated in modlefork_gb300.perturbate."""

import numpy as np
import pytest

from modlefork_gb300 import engine, genome, perturbate


def test_generate_deletions_end_one_bp_after_each_barrier():
    bars = [dict(pos=p, stp_active=0.7, stp_inactive=0.7, blocking_dir=1) for p in (100, 0, 5)]
    assert perturbate.generate_deletions(bars, 10) == [(0, 1), (0, 6), (91, 101)]


def test_windows_advance_by_the_diagonal_width():
    chrom = engine.Chromosome("chrW", 10_000)
    w = list(perturbate.windows(chrom, 1_000))
    assert w[0] == (0, 4000, 0, 3000)
    assert w[1] == (0, 4000, 1000, 3000)
    assert w[2] == (1000, 5000, 2000, 4000)
    assert w[-1] == (8000, 10_000, 9000, 10_000)
    assert [a for _, _, a, _ in w] == list(range(0, 10_000, 1000))


def test_window_tasks():
    cfg = genome.parity_config(diagonal_width=500_000)
    rng = np.random.default_rng(3)
    chrom = engine.Chromosome("chrW", 3_000_000)
    bars = engine.barriers_from_bed(chrom, genome.bed_records(rng, chrom.size, 60), 0.7, 0.7)
    dels = perturbate.generate_deletions(bars, 20_000)
    tasks = perturbate.window_tasks(cfg, chrom, bars, dels)
    assert [t["cell_id"] for t in tasks] == list(range(len(tasks)))
    for t in tasks:
        ws, we = t["window"]
        db, de = t["deletion"]
        assert db < we and ws < de  # the deletion overlaps the outer window
        assert all(ws <= b["pos"] < we for b in t["barriers"])
        off = [b for b in t["barriers"] if db <= b["pos"] < de]
        assert all(b["stp_active"] == 0.0 and b["stp_inactive"] == 1.0 for b in off)
        assert t["active_barriers"] == len(t["barriers"]) - len(off)
        assert t["nlefs"] == round((we - ws) / 1e6 * cfg.number_of_lefs_per_mbp)
        npix = ((we - ws + cfg.bin_size - 1) // cfg.bin_size) * ((cfg.diagonal_width + cfg.bin_size - 1) // cfg.bin_size)
        assert t["target_contacts"] == max(1, round(cfg.target_contact_density * npix))
    # every deletion overlapping a window is simulated once per window
    n = sum(sum(1 for d in dels if d[0] < we and ws < d[1])
            for ws, we, _, _ in perturbate.windows(chrom, cfg.diagonal_width)
            if any(ws <= b["pos"] < we for b in bars))
    assert len(tasks) == n


def test_oracle_window_spanning_the_chromosome_is_the_plain_cell():
    import ctypes as C

    from _harness import load_oracle, make_chrom
    from modlefork_gb300 import _abi as abi

    cfg, gen = genome.parity_10mbp(seed=9)
    chrom, bars = gen[0]
    nl = engine.num_lefs(cfg, chrom.simulated_size)
    targets, te = engine.task_targets(cfg, chrom.simulated_size, nl, 64)
    lib = load_oracle()
    nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
    bs = abi.make_barriers(bars)
    ch = make_chrom(0, chrom.end, chrom.size, b"chrS")
    out = []
    for window in (False, True):
        band = np.zeros(nrows * ncols, dtype=np.uint32)
        st = abi.CellStats()
        if window:
            rc = lib.orc_simulate_window_cell(C.byref(cfg), C.byref(ch), 0, chrom.end, bs, len(bars), 11,
                                              int(targets[0]), te, nl, band.ctypes.data_as(C.POINTER(C.c_uint32)),
                                              C.byref(st))
        else:
            rc = lib.orc_simulate_cell(C.byref(cfg), C.byref(ch), bs, len(bars), 11, int(targets[0]), te, nl,
                                       band.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(st), None)
        assert rc == 0
        out.append((band, (st.epochs, st.contacts, st.rng_draws)))
    assert np.array_equal(out[0][0], out[1][0]) and out[0][1] == out[1][1]


def test_block_sums_extend_edges_and_stay_in_the_band():
    nrows, ncols = 3, 6
    band = np.arange(1, nrows * ncols + 1, dtype=np.uint32)  # column j, row r at j * nrows + r
    for j in range(ncols):
        for r in range(nrows):
            if r > j:
                band[j * nrows + r] = 0
    get = lambda i, j: perturbate.band_get(band, nrows, ncols, i, j)
    assert get(2, 4) == band[4 * nrows + 2] and get(4, 2) == get(2, 4) and get(0, 5) == 0
    # 3x3 block at the corner (0, 0): rows and columns -1 clamp to 0
    want = sum(get(min(max(i, 0), ncols - 1), min(max(j, 0), ncols - 1)) for i in (-1, 0, 1) for j in (-1, 0, 1))
    assert perturbate.band_block(band, nrows, ncols, 0, 0, 3) == want
    assert perturbate.band_block(band, nrows, ncols, 2, 3, 1) == get(2, 3)


def test_window_band_and_scores():
    cfg = genome.parity_config(diagonal_width=20_000, bin_size=5000)
    nrows, ncols = engine.band_shape(cfg, 100_000)
    rng = np.random.default_rng(2)
    full = rng.integers(0, 9, size=nrows * ncols).astype(np.uint32)
    win = perturbate.window_band_of(cfg, full, nrows, 20_000, 60_000)
    wr, wc = engine.band_shape(cfg, 40_000)
    for jr in range(wc):
        for r in range(min(wr, jr + 1)):
            assert win[jr * wr + r] == full[(4 + jr) * nrows + r]
    task = dict(window=(20_000, 60_000), active=(20_000, 40_000), deletion=(30_000, 31_000), cell_id=7, task_id=11,
                active_barriers=2, barriers=[{}, {}, {}])
    sim = win.copy()
    sim[0] += 5
    res = perturbate.WindowResult(engine.Chromosome("chrW", 100_000), task, sim, None)
    feats1 = [("chrW", 21_000, 21_001, "a", "+")]
    feats2 = [("chrW", 24_000, 24_001, "", "-"), ("chrW", 45_000, 45_001, "b", "+")]
    lines = perturbate.score_window(cfg, res, win, feats1, feats2, block_size=1)
    rows = [ln.split("\t") for ln in lines]
    assert all(r[6] in ("a;none", "a;b") for r in rows)
    for r in rows:
        ref, cont = int(r[10]), int(r[11])
        assert ref + cont > 0
        if ref and cont:
            assert abs(float(r[7]) - np.log2(cont / ref)) < 1e-3 * max(1.0, abs(np.log2(cont / ref)))
        assert r[13:] == ["30000", "31000", "2", "3", "20000", "40000", "20000", "60000", "11"]
    assert perturbate.binomial_test(5, 10) == 1.0
    assert abs(perturbate.binomial_test(0, 10) - 2 * 0.5 ** 10) < 1e-12


@pytest.mark.parametrize("block_size", [1, 3, 4, 9])
def test_vectorised_block_sums_equal_the_loop(block_size):
    rng = np.random.default_rng(block_size)
    nrows, ncols = 7, 40
    band = rng.integers(0, 100, nrows * ncols).astype(np.uint32)
    for j in range(ncols):
        for r in range(nrows):
            if r > j:
                band[j * nrows + r] = 0
    rows = rng.integers(0, ncols, 300)
    cols = rng.integers(0, ncols, 300)
    rows[:4], cols[:4] = [0, ncols - 1, 0, ncols - 1], [0, ncols - 1, ncols - 1, 0]
    got = perturbate.band_blocks(band, nrows, ncols, rows, cols, block_size)
    want = [perturbate.band_block(band, nrows, ncols, int(r), int(c), block_size) for r, c in zip(rows, cols)]
    assert got.tolist() == want


def test_task_sizes_round_halves_away_from_zero():
    """The LEF count and contact target use std::round (scheduler_perturbate.cpp:306-320)."""
    assert [perturbate.cpp_round(x) for x in (0.5, 1.5, 2.5, 2.4999999999999996, 60.5, -2.5, 0.0)] == \
        [1, 2, 3, 2, 61, -3, 0]
    cfg = genome.parity_config(diagonal_width=1_000_000, bin_size=5000, number_of_lefs_per_mbp=20.0)
    chrom = engine.Chromosome("chrR", 3_025_000)  # the outer window is 3.025 Mbp: 60.5 LEFs
    bars = [dict(pos=1_000_000, stp_active=0.9, stp_inactive=0.9, blocking_dir=1)]
    tasks = perturbate.window_tasks(cfg, chrom, bars, perturbate.generate_deletions(bars, 10_000))
    assert tasks[0]["window"] == (0, 3_025_000) and tasks[0]["nlefs"] == 61


def test_read_bed_features(tmp_path):
    import gzip

    text = "track name=x\n#c\nchr2\t50\t60\tb\t0\t-\nchr1\t10\t20\nchr1\t5\t8\ta\t1\t+\n"
    p = tmp_path / "f.bed"
    p.write_text(text)
    pz = tmp_path / "f.bed.gz"
    with gzip.open(pz, "wt") as f:
        f.write(text)
    for path in (p, pz):
        got = perturbate.read_bed_features(str(path))
        assert got == {"chr1": [("chr1", 5, 8, "a", "+"), ("chr1", 10, 20, "", ".")],
                       "chr2": [("chr2", 50, 60, "b", "-")]}
    bad = tmp_path / "bad.bed"
    bad.write_text("chr1\t10\n")
    with pytest.raises(ValueError):
        perturbate.read_bed_features(str(bad))


def test_records_take_the_active_window_features(tmp_path):
    """perturbate_records scores each window with the features of its active window, against
    the reference band restricted to the window, and writes (gzipped) bedpe."""
    cfg = genome.parity_config(diagonal_width=20_000, bin_size=5000)
    chrom = engine.Chromosome("chrW", 100_000)
    nrows, ncols = engine.band_shape(cfg, chrom.size)
    rng = np.random.default_rng(5)
    ref = rng.integers(0, 9, nrows * ncols).astype(np.uint32)
    feats1 = {"chrW": [("chrW", 15_000, 15_001, "a", "+"), ("chrW", 75_000, 75_001, "c", "+")]}
    feats2 = {"chrW": [("chrW", 24_000, 24_001, "", "-"), ("chrW", 35_000, 35_001, "b", "+"),
                       ("chrW", 78_000, 78_001, "d", "-")]}
    results = []
    for tid, (ws, we, a0, a1) in enumerate([(0, 80_000, 0, 60_000), (20_000, 100_000, 40_000, 100_000)]):
        wr, wc = engine.band_shape(cfg, we - ws)
        task = dict(window=(ws, we), active=(a0, a1), deletion=(30_000, 31_000), cell_id=tid, task_id=tid,
                    active_barriers=1, barriers=[{}, {}])
        results.append(perturbate.WindowResult(chrom, task, rng.integers(0, 9, wr * wc).astype(np.uint32), None))
    lines = perturbate.perturbate_records(cfg, feats1, feats2, {"chrW": ref}, results, block_size=3)
    want = []
    for r in results:
        a0, a1 = r.task["active"]
        ws, we = r.task["window"]
        win = perturbate.window_band_of(cfg, ref, nrows, ws, we)
        f1 = [f for f in feats1["chrW"] if a0 <= f[1] < a1]
        f2 = [f for f in feats2["chrW"] if a0 <= f[1] < a1]
        want += perturbate.score_window(cfg, r, win, f1, f2, block_size=3, last_window=a1 == chrom.end)
    assert lines == want and lines
    assert {ln.split("\t")[-1] for ln in lines} <= {"0", "1"}
    # the first window pairs feature a with the kind-2 features of its active window; the
    # second (the last window of the chromosome) pairs c with d
    names = [(ln.split("\t")[6], ln.split("\t")[-1]) for ln in lines]
    assert {n for n, t in names if t == "0"} <= {"a;none", "a;b"} and {n for n, t in names if t == "1"} <= {"c;d"}
    out = tmp_path / "x.bedpe.gz"
    perturbate.write_bedpe(str(out), lines)
    import gzip

    with gzip.open(out, "rt") as f:
        got = f.read().splitlines()
    assert got[0] == "#" + "\t".join(perturbate.BEDPE_COLUMNS) and got[1:] == lines
    assert all(len(ln.split("\t")) == len(perturbate.BEDPE_COLUMNS) for ln in lines)


def test_plan_windows_with_a_deletion_list(tmp_path):
    cfg = genome.parity_config(diagonal_width=500_000)
    chroms = [engine.Chromosome("chrD0", 2_000_000), engine.Chromosome("chrD1", 1_500_000)]
    rng = np.random.default_rng(6)
    gen = [(ch, engine.barriers_from_bed(ch, genome.bed_records(rng, ch.size, 12), 0.7, 0.7)) for ch in chroms]
    bed = tmp_path / "del.bed"
    bed.write_text("chrD0\t900000\t950000\nchrD0\t100000\t120000\nchrX\t1\t5\n")
    dels = perturbate.read_bed_intervals(str(bed))
    assert dels == {"chrD0": [(100_000, 120_000), (900_000, 950_000)], "chrX": [(1, 5)]}
    planned = perturbate.plan_windows(cfg, gen, deletions=dels)
    # chrD1 has no deletions and is skipped; every task carries one of the listed deletions
    assert {c.name for c, _ in planned} == {"chrD0"}
    assert {t["deletion"] for _, t in planned} <= set(dels["chrD0"])
    assert [t["task_id"] for _, t in planned] == list(range(len(planned)))
    for _, t in planned:
        ws, we = t["window"]
        db, de = t["deletion"]
        assert db < we and ws < de  # the deletion overlaps the window
        off = [b for b in t["barriers"] if b["stp_active"] == 0.0 and b["stp_inactive"] == 1.0]
        assert len(t["barriers"]) - len(off) == t["active_barriers"]
    # generated deletions: one per barrier, ending one bp after it
    gen_plan = perturbate.plan_windows(cfg, gen, deletion_size=30_000)
    assert {c.name for c, _ in gen_plan} == {"chrD0", "chrD1"}


def test_deletion_list_skipping_a_middle_chromosome_keeps_task_ids_contiguous(tmp_path):
    """A deletion list that omits a chromosome between two listed ones and names one the genome
    lacks (the reference looks deletions up per chromosome and skips chromosomes without any,
    scheduler_perturbate.cpp:202): the omitted and the unknown chromosome give no task, and the
    run-wide task ids run on without a gap from the first listed chromosome to the next."""
    cfg = genome.parity_config(diagonal_width=500_000)
    chroms = [engine.Chromosome(f"chrM{k}", 1_800_000) for k in range(3)]
    rng = np.random.default_rng(8)
    gen = [(ch, engine.barriers_from_bed(ch, genome.bed_records(rng, ch.size, 10), 0.7, 0.7)) for ch in chroms]
    bed = tmp_path / "del.bed"
    bed.write_text("chrM2\t300000\t330000\nchrUn\t5\t9\nchrM0\t700000\t720000\n")
    dels = perturbate.read_bed_intervals(str(bed))
    planned = perturbate.plan_windows(cfg, gen, deletions=dels)
    names = [c.name for c, _ in planned]
    assert set(names) == {"chrM0", "chrM2"} and "chrM1" not in names
    assert names == sorted(names, key=lambda n: int(n[-1]))  # genome order: chrM0's tasks first
    assert [t["task_id"] for _, t in planned] == list(range(len(planned)))
    first_m2 = names.index("chrM2")
    assert 0 < first_m2 and planned[first_m2][1]["task_id"] == planned[first_m2 - 1][1]["task_id"] + 1
