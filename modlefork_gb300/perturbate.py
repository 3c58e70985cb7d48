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
one batched launch (mgpu_simulate_batch).  The feature-pair scoring and bedpe output of the
reference (reference cooler, block aggregation, binomial test) are not part of this module.
"""

import numpy as np

from . import engine

MBP = 1.0e6


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
    window, the deletion, the cell id, the LEF count, the contact and epoch targets and the
    window's barriers with the deleted ones switched off."""
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
                target = int(max(1.0, round(cfg.target_contact_density * float(npix1 * npix2))))
            nlefs = int(round((we - ws) / MBP * cfg.number_of_lefs_per_mbp))
            te = int(cfg.target_simulation_epochs) if target == 0 else (1 << 64) - 1
            tasks.append(dict(window=(ws, we), active=(a0, a1), deletion=(db, de), cell_id=cell_id,
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


def simulate_windows(cfg, genome, deletion_size=10_000, features=None, device=0, max_tasks=None):
    """Simulate every (window, deletion) task of the genome in one batched launch; returns one
    WindowResult per task, in task-id order.  ``features`` maps a chromosome name to two lists
    of (start, end) intervals (the two feature kinds); without it no window is skipped for
    lack of features."""
    results = []
    with engine.Engine(cfg, device) as eng:
        batch, bands, meta = [], {}, []
        for chrom, bars in genome:
            if not bars:
                continue
            dels = generate_deletions(bars, deletion_size)
            feats = features.get(chrom.name) if features is not None else None
            if features is not None and feats is None:
                continue
            for t in window_tasks(cfg, chrom, bars, dels, feats):
                if max_tasks is not None and len(batch) >= max_tasks:
                    break
                cid = eng.upload_window(chrom, t["window"][0], t["window"][1], t["barriers"])
                nrows, ncols = engine.band_shape(cfg, t["window"][1] - t["window"][0])
                bands[cid] = np.zeros(nrows * ncols, dtype=np.uint32)
                seed = engine.cell_seed(chrom.name, chrom.size, cfg.seed, t["cell_id"])
                batch.append((cid, seed, t["target_contacts"], t["target_epochs"], t["nlefs"]))
                meta.append((chrom, t, cid))
        if not batch:
            return results
        _, stats = eng.simulate_batch(batch, bands)
    for k, (chrom, t, cid) in enumerate(meta):
        results.append(WindowResult(chrom, t, bands[cid], stats[k]))
    return results
