"""Barrier-deletion windows of ``modle perturbate`` on the batched engine.

The reference (src/libmodle/cpu/scheduler_perturbate.cpp:90-372, scheduler_common.cpp:51-127)
walks each chromosome with an outer window 4*D wide (D = diagonal width) whose central 2*D is the
active window, advancing by D; for every deletion overlapping the outer window it simulates one
cell of that window with the barriers inside the deletion switched off
(Simulation::simulate_window, :429-480).  Generated deletions end one bp after each barrier and
span ``deletion_size`` bp (generate_deletions).  Each (window, deletion) is one task: its seed is
the chromosome's hash of (seed, cell id) with cell ids counted per chromosome, its LEF count and
contact target follow from the window's size.

Here every task becomes a window upload (mgpu_upload_window) and all tasks of a run advance in
one batched launch (mgpu_simulate_batch).  ``score_window`` then compares a window's contacts
with a reference run's for every pair of features, as simulate_window's bedpe output does
(block sums with edge extension, log2 ratio, two-sided binomial test).
"""

import math

import numpy as np

from . import engine

MBP = 1.0e6


def cpp_round(x):
    """std::round: halves go away from zero (Python's round sends them to the even neighbour)."""
    x = float(x)
    if x < 0:
        return -cpp_round(-x)
    f = math.floor(x)
    return f + 1 if x - f >= 0.5 else f


def generate_deletions(barriers, deletion_size):
    """Simulation::generate_deletions: [pos + 1 - s, pos + 1) with s = min(pos + 1, size), in
    position order."""
    out = []
    for b in barriers:
        s = min(int(b["pos"]) + 1, int(deletion_size))
        begin = int(b["pos"]) + 1 - s
        out.append((begin, begin + s))
    return sorted(out)


def windows(chrom, diagonal_width):
    """Outer and active windows of one chromosome (TaskPW set-up and Simulation::advance_window):
    yields (window_start, window_end, active_start, active_end)."""
    d = int(diagonal_width)
    ws, we, a0, a1 = 0, 4 * d, 0, 3 * d
    end = chrom.end
    while True:
        yield ws, min(we, end), a0, min(a1, end)
        a0 += d
        a1 = min(a0 + 2 * d, end)
        ws = a0 - d
        we = min(a1 + d, end)
        if a0 >= end:
            return


def _features_in(features, lo, hi):
    return any(s < hi and lo < e for s, e in features)


def window_tasks(cfg, chrom, barriers, deletions, features=None):
    """Tasks of one chromosome in the reference's order: dicts with the window, the active
    window, the deletion, the cell id (counted per chromosome, it seeds the cell), the task id
    (counted over the whole run by simulate_windows; here equal to the cell id), the LEF count,
    the contact and epoch targets and the window's barriers with the deleted ones switched off."""
    bars = sorted(barriers, key=lambda b: b["pos"])
    d = int(cfg.diagonal_width)
    bin_size = int(cfg.bin_size)
    tasks, cell_id = [], 0
    for ws, we, a0, a1 in windows(chrom, d):
        wbars = [b for b in bars if ws <= b["pos"] < we]
        if not wbars:
            continue
        if features is not None and not (_features_in(features[0], a0, a1) and _features_in(features[1], a0, a1)):
            continue
        for db, de in (x for x in deletions if x[0] < we and ws < x[1]):
            tb = []
            for b in wbars:
                if db <= b["pos"] < de:
                    tb.append(dict(pos=b["pos"], stp_active=0.0, stp_inactive=1.0, blocking_dir=b["blocking_dir"]))
                else:
                    tb.append(dict(b))
            target = 0
            if cfg.target_contact_density != 0.0:
                npix1 = (we - ws + bin_size - 1) // bin_size
                npix2 = (d + bin_size - 1) // bin_size
                target = int(max(1.0, cpp_round(cfg.target_contact_density * float(npix1 * npix2))))
            nlefs = int(cpp_round((we - ws) / MBP * cfg.number_of_lefs_per_mbp))
            te = int(cfg.target_simulation_epochs) if target == 0 else (1 << 64) - 1
            tasks.append(dict(window=(ws, we), active=(a0, a1), deletion=(db, de), cell_id=cell_id,
                              task_id=cell_id,
                              nlefs=nlefs, target_contacts=target, target_epochs=te, barriers=tb,
                              active_barriers=sum(1 for b in wbars if not (db <= b["pos"] < de))))
            cell_id += 1
    return tasks


class WindowResult:
    def __init__(self, chrom, task, band, stats):
        self.chrom = chrom
        self.task = task
        self.band = band
        self.stats = stats


def plan_windows(cfg, genome, deletion_size=10_000, features=None, max_tasks=None, deletions=None):
    """Every (window, deletion) task of the genome in the reference's order, as (chrom, task)
    pairs with run-wide task ids (scheduler_perturbate.cpp:189, :298).  ``features`` maps a
    chromosome name to two lists of (start, end) intervals (the two feature kinds); chromosomes
    without barriers, or without features when ``features`` is given, are skipped, and without
    it no window is skipped for lack of features.  ``deletions`` maps a chromosome name to its
    (start, end) deletions (an imported --deletion-list, Simulation::import_deletions,
    scheduler_common.cpp:42-49); chromosomes it lacks are skipped.  Without it the deletions are
    generated from the barriers (generate_deletions)."""
    planned = []
    for chrom, bars in genome:
        if not bars:
            continue
        feats = features.get(chrom.name) if features is not None else None
        if features is not None and feats is None:
            continue
        if deletions is not None:
            if chrom.name not in deletions:
                continue
            dels = sorted((int(a), int(b)) for a, b in deletions[chrom.name])
        else:
            dels = generate_deletions(bars, deletion_size)
        for t in window_tasks(cfg, chrom, bars, dels, feats):
            if max_tasks is not None and len(planned) >= max_tasks:
                return planned
            t["task_id"] = len(planned)
            planned.append((chrom, t))
    return planned


def run_windows(cfg, planned, device=0):
    """Simulate the planned (chrom, task) pairs in one batched launch (mgpu_upload_window per
    task, mgpu_simulate_batch); returns one WindowResult per task, in the given order."""
    if not planned:
        return []
    from . import autotune

    with engine.Engine(cfg, device) as eng:
        autotune.apply_all(eng)
        batch, bands, cids = [], {}, []
        for chrom, t in planned:
            cid = eng.upload_window(chrom, t["window"][0], t["window"][1], t["barriers"])
            nrows, ncols = engine.band_shape(cfg, t["window"][1] - t["window"][0])
            bands[cid] = np.zeros(nrows * ncols, dtype=np.uint32)
            seed = engine.cell_seed(chrom.name, chrom.size, cfg.seed, t["cell_id"])
            batch.append((cid, seed, t["target_contacts"], t["target_epochs"], t["nlefs"]))
            cids.append(cid)
        _, stats = eng.simulate_batch(batch, bands)
    return [WindowResult(chrom, t, bands[cid], stats[k]) for k, ((chrom, t), cid) in enumerate(zip(planned, cids))]


def simulate_windows(cfg, genome, deletion_size=10_000, features=None, device=0, max_tasks=None):
    """Simulate every (window, deletion) task of the genome in one batched launch; returns one
    WindowResult per task, in task-id order (plan_windows, then run_windows)."""
    return run_windows(cfg, plan_windows(cfg, genome, deletion_size, features, max_tasks), device)


# ---------------------------------------------------------------------------------------------
# feature-pair scoring (Simulation::simulate_window, scheduler_perturbate.cpp:481-556)

def band_get(band, nrows, ncols, i, j):
    """ContactMatrixDense::unsafe_get: the count of bins (i, j), 0 outside the band."""
    if i > j:
        i, j = j, i
    r = j - i
    return 0 if r >= nrows else int(band[j * nrows + r])


def band_block(band, nrows, ncols, row, col, block_size):
    """ContactMatrixDense::unsafe_get_block (contact_matrix_dense_unsafe_impl.hpp:89-113): sum of
    the block_size x block_size pixels centred on (row, col), edges extended."""
    if block_size == 1:
        return band_get(band, nrows, ncols, row, col)
    h = block_size // 2
    tot = 0
    for i in range(row - h, row - h + block_size):
        for j in range(col - h, col - h + block_size):
            tot += band_get(band, nrows, ncols, min(max(i, 0), ncols - 1), min(max(j, 0), ncols - 1))
    return tot


def band_blocks(band, nrows, ncols, rows, cols, block_size):
    """band_block for many (row, col) centres at once (equal results): the block's indices are
    clamped to the matrix, mirrored into the upper triangle and read from the band, 0 outside
    it.  Centres are processed in chunks to bound the temporary arrays."""
    band = np.asarray(band)
    rows = np.asarray(rows, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int64)
    out = np.zeros(rows.size, dtype=np.int64)
    h = block_size // 2 if block_size > 1 else 0
    off = np.arange(block_size, dtype=np.int64) - h
    step = max(1, (1 << 22) // max(1, block_size * block_size))
    for k0 in range(0, rows.size, step):
        r = rows[k0:k0 + step]
        c = cols[k0:k0 + step]
        ii = np.clip(r[:, None, None] + off[None, :, None], 0, ncols - 1)
        jj = np.clip(c[:, None, None] + off[None, None, :], 0, ncols - 1)
        lo, hi = np.minimum(ii, jj), np.maximum(ii, jj)
        d = hi - lo
        inside = d < nrows
        vals = np.where(inside, band[np.where(inside, hi * nrows + d, 0)], 0).astype(np.int64)
        out[k0:k0 + step] = vals.sum(axis=(1, 2))
    return out


def window_band_of(cfg, band, nrows_full, window_start, window_end):
    """The reference run's contacts (a chromosome band with ``nrows_full`` rows) restricted to a
    window, in the window's own band layout (read_reference_contacts,
    scheduler_perturbate.cpp:76-87): pixels with both bins inside the window."""
    bin_size = int(cfg.bin_size)
    b0 = window_start // bin_size
    nrows_w, ncols_w = engine.band_shape(cfg, window_end - window_start)
    full = np.asarray(band).reshape(-1, nrows_full)
    out = np.zeros((ncols_w, nrows_w), dtype=np.uint32)
    for jr in range(max(0, min(ncols_w, full.shape[0] - b0))):
        r = np.arange(min(nrows_w, nrows_full, jr + 1))
        out[jr, r] = full[b0 + jr, r]
    return out.reshape(-1)


def binomial_test(k, n, p=0.5):
    """stats::binomial_test, two-sided (src/stats/tests_impl.hpp:17-110), which follows scipy's
    binomtest."""
    from scipy.stats import binomtest

    if n == 0:
        return 1.0
    return float(binomtest(int(k), int(n), p, alternative="two-sided").pvalue)


def score_window(cfg, result, ref_window_band, feats1, feats2, block_size=9, last_window=False):
    """bedpe records of one (window, deletion) task: for feature i of kind 1 and j >= i of kind
    2 (each (chrom, start, end, name, strand)), the block sums of the window's and the
    reference's contacts around their bins, their log2 ratio and binomial p-value, and the task's
    window, deletion and barrier counts and its task id.  Pairs with both features past the
    partition point are left to the next window (except in the last one), and pairs without
    contacts are skipped."""
    t = result.task
    ws, we = t["window"]
    a0, a1 = t["active"]
    d = int(cfg.diagonal_width)
    bin_size = int(cfg.bin_size)
    nrows, ncols = engine.band_shape(cfg, we - ws)
    part = a0 + d
    pairs = []
    for i, f1 in enumerate(feats1):
        for f2 in feats2[i:]:
            if not last_window and f1[1] >= part and f2[1] >= part:
                continue
            pairs.append((f1, f2))
    if not pairs:
        return []
    c1 = np.array([(f1[1] + f1[2] + 1) // 2 for f1, _ in pairs], dtype=np.int64)
    c2 = np.array([(f2[1] + f2[2] + 1) // 2 for _, f2 in pairs], dtype=np.int64)
    b1r, b2r = (c1 - ws) // bin_size, (c2 - ws) // bin_size
    conts = band_blocks(result.band, nrows, ncols, b1r, b2r, block_size)
    refs = band_blocks(ref_window_band, nrows, ncols, b1r, b2r, block_size)
    lines = []
    for k, (f1, f2) in enumerate(pairs):
        cont, ref = int(conts[k]), int(refs[k])
        if cont == 0 and ref == 0:
            continue
        if ref == 0:
            score = 999.0
        elif cont == 0:
            score = -999.0
        else:
            score = min(max(float(np.log2(cont / ref)), -999.0), 999.0)
        sig = binomial_test(cont, ref + cont)
        b1, b2 = int(c1[k]) // bin_size, int(c2[k]) // bin_size
        name = f"{f1[3] or 'none'};{f2[3] or 'none'}"
        lines.append("\t".join(str(x) for x in (
            f1[0], b1 * bin_size, (b1 + 1) * bin_size, f2[0], b2 * bin_size, (b2 + 1) * bin_size,
            name, format(score, ".4G"), f1[4], f2[4], ref, cont, format(sig, ".4G"),
            t["deletion"][0], t["deletion"][1], t["active_barriers"], len(t["barriers"]),
            a0, a1, ws, we, t["task_id"])))
    return lines


# ---------------------------------------------------------------------------------------------
# the modle perturbate run: features, reference contacts, window tasks, bedpe records

def read_bed_intervals(path):
    """BED3 intervals grouped by chromosome: {chrom: [(start, end)]} sorted, e.g. a deletion
    list (bed::BED_tree of BED3 records)."""
    return {c: [(f[1], f[2]) for f in fs] for c, fs in read_bed_features(path).items()}


def read_bed_features(path):
    """Features of a BED file as (chrom, start, end, name, strand) tuples grouped by chromosome
    and sorted by (start, end): BED3-BED6 fields, name "" and strand "." when absent; track,
    browser and comment lines are skipped (the --feature-beds inputs, cli.cpp:653-657)."""
    import gzip

    opener = gzip.open if str(path).endswith(".gz") else open
    out = {}
    with opener(path, "rt") as f:
        for line in f:
            if not line.strip() or line.startswith(("#", "track", "browser")):
                continue
            fs = line.rstrip("\n").split("\t")
            if len(fs) < 3:
                raise ValueError(f"{path}: a BED record needs at least 3 fields: {line!r}")
            start, end = int(fs[1]), int(fs[2])
            if end < start:
                raise ValueError(f"{path}: end before start: {line!r}")
            name = fs[3] if len(fs) > 3 else ""
            strand = fs[5] if len(fs) > 5 else "."
            out.setdefault(fs[0], []).append((fs[0], start, end, name, strand))
    for v in out.values():
        v.sort(key=lambda x: (x[1], x[2]))
    return out


def features_in(feats, lo, hi):
    """The features overlapping [lo, hi) (map_features_to_window, scheduler_common.cpp:82-111)."""
    return [f for f in feats if f[1] < hi and lo < f[2]]


def perturbate_records(cfg, feats1, feats2, ref_bands, results, block_size=9):
    """bedpe records of every window result, in task-id order: each window's features of both
    kinds in its active window, scored against the reference run's band of its chromosome
    restricted to the window.  ref_bands maps a chromosome name to its full band (chromosomes
    simulated from position 0, as the generated workloads are)."""
    lines = []
    for r in results:
        t = r.task
        a0, a1 = t["active"]
        ws, we = t["window"]
        nrows_full, _ = engine.band_shape(cfg, r.chrom.simulated_size)
        ref_win = window_band_of(cfg, ref_bands[r.chrom.name], nrows_full, ws, we)
        f1 = features_in(feats1.get(r.chrom.name, []), a0, a1)
        f2 = features_in(feats2.get(r.chrom.name, []), a0, a1)
        lines += score_window(cfg, r, ref_win, f1, f2, block_size=block_size,
                              last_window=a1 == r.chrom.end)
    return lines


# bedpe columns, the header line the reference writes when asked to (scheduler_perturbate.cpp:120-152)
BEDPE_COLUMNS = ("chrom1", "start1", "end1", "chrom2", "start2", "end2", "name", "score", "strand1",
                 "strand2", "reference_contacts", "contacts", "significance", "deletion_begin",
                 "deletion_end", "num_active_barriers", "total_num_barriers", "active_window_start",
                 "active_window_end", "window_start", "window_end", "task_id")


def write_bedpe(path, lines, header=True):
    """bedpe records (gzip when the path ends in .gz), after a '#'-prefixed column header."""
    import gzip

    opener = gzip.open if str(path).endswith(".gz") else open
    with opener(path, "wt") as f:
        if header:
            f.write("#" + "\t".join(BEDPE_COLUMNS) + "\n")
        for ln in lines:
            f.write(ln + "\n")


def reference_bands(cfg, genome, device=0, world=1, rank=0, group=None):
    """The reference run of simulate_window's comparison: every chromosome's band over all
    cells.  With several ranks each simulates its contiguous range of cell ids and the bands are
    summed exactly over the ranks (sharding.allreduce_band_)."""
    import torch

    from . import sharding
    from .simulate import simulate_genome_batched

    lo, hi = sharding.cell_range(int(cfg.num_cells), world, rank)
    res = simulate_genome_batched(cfg, genome, device=device, cell_range=(lo, hi))
    bands = {r.chrom.name: r.band for r in res}
    if world > 1:
        dev = torch.device("cuda", device) if torch.cuda.is_available() else torch.device("cpu")
        for name, b in bands.items():
            t = torch.from_numpy(b.view(np.int32)).to(dev)
            bands[name] = sharding.allreduce_band_(t, group).cpu().numpy().view(np.uint32)
    return bands


def run(cfg, g, feats1, feats2, deletion_size=10_000, deletion_list=None, block_size=9, max_tasks=None, device=0,
        world=1, rank=0, group=None, reference=None, windows_fn=None):
    """The command's work on one rank: the reference bands, the planned (window, deletion) cells
    (every rank plans the same queue), this rank's block of the queue simulated and scored, and
    the records of all ranks in task-id order (every rank returns them).  ``reference(cfg, g)``
    and ``windows_fn(cfg, planned)`` replace the GPU's reference run and window launch (tests run
    them with the oracle)."""
    from . import sharding

    names = {c.name for c, _ in g}
    features = {n: ([(f[1], f[2]) for f in feats1[n]], [(f[1], f[2]) for f in feats2[n]])
                for n in names if n in feats1 and n in feats2}
    ref = reference(cfg, g) if reference else reference_bands(cfg, g, device, world, rank, group)
    dels = read_bed_intervals(deletion_list) if deletion_list else None
    planned = plan_windows(cfg, g, deletion_size, features, max_tasks, dels)
    win = windows_fn or (lambda c, p: run_windows(c, p, device=device))
    if world == 1:
        return perturbate_records(cfg, feats1, feats2, ref, win(cfg, planned), block_size), len(planned)
    return sharding.perturbate_sharded(cfg, planned, feats1, feats2, ref, world, rank, win, block_size,
                                       group), len(planned)


def _main(argv=None):
    """modle perturbate on a generated workload: a reference run of the whole genome, then one
    cell per (window, deletion) in one batched launch, scored for every pair of features of the
    two BED files.  Under torchrun (WORLD_SIZE > 1) every rank simulates its share of the
    reference cells and a contiguous block of the window queue on GPU LOCAL_RANK; rank 0 writes
    the bedpe.  Example:

    python -m modlefork_gb300.perturbate --workload parity --features a.bed b.bed --out x.bedpe.gz
    """
    import argparse
    import json
    import os
    import time

    from . import genome as gen

    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--workload", choices=["parity", "genome"], default="parity")
    ap.add_argument("--chroms", type=int, default=24, help="chromosomes of the generated genome workload")
    ap.add_argument("--features", nargs=2, required=True, metavar=("BED1", "BED2"))
    dg = ap.add_mutually_exclusive_group()
    dg.add_argument("--deletion-size", type=int, default=10_000)
    dg.add_argument("--deletion-list", default=None, help="BED file of the deletions to perform")
    ap.add_argument("--block-size", type=int, default=9)
    ap.add_argument("--max-tasks", type=int, default=None)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--out", required=True, help="bedpe output (gzip when it ends in .gz)")
    ap.add_argument("--no-header", action="store_true", help="omit the bedpe column header")
    args = ap.parse_args(argv)
    if args.block_size < 1 or args.block_size % 2 == 0:
        ap.error("--block-size must be a positive odd number")
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    device = int(os.environ.get("LOCAL_RANK", args.device)) if world > 1 else args.device
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(device)
        dist.init_process_group("nccl", init_method="env://")
    cfg, g = gen.parity_10mbp() if args.workload == "parity" else gen.genome_24chr(nchroms=args.chroms)
    feats1, feats2 = read_bed_features(args.features[0]), read_bed_features(args.features[1])
    t0 = time.perf_counter()
    lines, ntasks = run(cfg, g, feats1, feats2, args.deletion_size, args.deletion_list, args.block_size,
                        args.max_tasks, device, world, rank)
    if rank == 0:
        write_bedpe(args.out, lines, header=not args.no_header)
        print(json.dumps({"workload": args.workload, "tasks": ntasks, "records": len(lines), "ranks": world,
                          "seconds": time.perf_counter() - t0}))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    _main()
