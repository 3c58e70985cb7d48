"""Parameter-sweep data generation for the learned surrogate, on the batched simulator.

Each parameter set k is one 20 Mbp window (4000 bins of 5 kb, a 3 Mbp band of 600 diagonals)
with its own seeded barrier track and extrusion parameters:

* barriers: density U(10, 60)/Mbp at distinct uniform positions, strand +/- with p = 0.5,
  occupancy ~ Beta(8, 2) written to the BED score (as the genome workload);
* LEFs: density U(5, 40)/Mbp, average lifetime (processivity) U(50, 500) kb, extrusion speed
  U(1, 5) kb/epoch in both directions (standard deviation 5 % of the speed);
* cells: ``cells`` per set (1024 in the full sweep), contact density ``density``.

All windows of a chunk advance in one ``mgpu_simulate_batch`` launch, each with its own
configuration (``mgpu_set_chrom_config``).  The summed band of a window is turned into the
training target on the device (``msur_band_target``: per bin, log1p of the band row scaled to
mean 1, the row-normalised log1p of the mean over cells, in FP32), and every target is checked
against an FP64 host reduction of the same band.

The network's input for a window is a 4-channel track over its 4000 bins (summed barrier
occupancy, number of + motifs, number of - motifs, LEF density) plus a 4-vector of the
parameters (LEF density, lifetime, speed, barrier density), scaled to O(1).
"""

import os

import numpy as np

from . import engine, genome

WINDOW_BP = 20_000_000
BIN = 5000
DIAG = 3_000_000
NCOLS = WINDOW_BP // BIN  # 4000 bins
NROWS = DIAG // BIN       # 600 diagonals
PARAM_SCALE = np.array([40.0, 500e3, 5e3, 60.0])


def parameter_set(k, seed=2024):
    """The k-th parameter set of a sweep: a pure function of (seed, k), so any index can be
    regenerated (and a sweep resumed) without the ones before it."""
    rng = np.random.default_rng([seed, k])
    return {
        "bar_density": float(rng.uniform(10.0, 60.0)),
        "lef_density": float(rng.uniform(5.0, 40.0)),
        "lifetime": int(round(rng.uniform(50e3, 500e3))),
        "speed": int(round(rng.uniform(1e3, 5e3))),
        "track_seed": int(rng.integers(0, 2**62)),
    }


def window_config(ps, cells, density, seed, api=None):
    api = api or engine
    return genome.genome_config(api=api, bin_size=BIN, diagonal_width=DIAG, number_of_lefs_per_mbp=ps["lef_density"],
                                avg_lef_processivity=ps["lifetime"], rev_extrusion_speed=ps["speed"],
                                fwd_extrusion_speed=ps["speed"], rev_speed_set=1, fwd_speed_set=1,
                                rev_extrusion_speed_std=0.05, fwd_extrusion_speed_std=0.05, num_cells=cells,
                                target_contact_density=density, seed=seed)


def window(k, seed=2024, cells=1024, density=10.0, api=None):
    """(cfg, chrom, barriers, track[4, NCOLS] float32, params[4] float32) of parameter set k."""
    api = api or engine
    ps = parameter_set(k, seed)
    cfg = window_config(ps, cells, density, seed + k, api)
    rng = np.random.default_rng(ps["track_seed"])
    chrom = api.Chromosome(f"sweep{k}", WINDOW_BP)
    nb = int(round(WINDOW_BP / 1e6 * ps["bar_density"]))
    occ = rng.beta(8.0, 2.0, size=nb)
    recs = genome.bed_records(rng, WINDOW_BP, nb, occ)
    bars = api.barriers_from_bed(chrom, recs, cfg.barrier_occupied_stp, cfg.barrier_not_occupied_stp)
    track = barrier_track(recs)
    track[3] = ps["lef_density"] / PARAM_SCALE[0]
    params = np.array([ps["lef_density"], ps["lifetime"], ps["speed"], ps["bar_density"]]) / PARAM_SCALE
    return cfg, chrom, bars, track, params.astype(np.float32)


def barrier_track(records):
    """Channels 0-2 of the input track from BED records (start, end, strand, occupancy): summed
    occupancy, + motifs and - motifs per bin of the barrier (its midpoint, genome.cpp:199)."""
    track = np.zeros((4, NCOLS), dtype=np.float32)
    for s, e, strand, occ in records:
        b = min(NCOLS - 1, ((s + e + 1) // 2) // BIN)
        track[0, b] += occ
        track[1 if strand == "+" else 2, b] += 1.0
    return track


def target_fp64(band):
    """FP64 host reduction of a summed band (column-major [NCOLS][NROWS]): the reference the
    device targets are checked against."""
    b = np.asarray(band, dtype=np.float64).reshape(-1, NROWS)
    s = b.sum(1, keepdims=True)
    scale = np.divide(NROWS, s, out=np.zeros_like(s), where=s > 0)
    return np.log1p(b * scale)


def simulate_sets(ks, seed=2024, cells=1024, density=10.0, device=0, smem_budget=None, check=True):
    """Simulate parameter sets ks on the GPU in one batched launch.  Returns a dict with
    track [n, 4, NCOLS], params [n, 4], target [n, NCOLS, NROWS] (torch float32 on the device),
    the FP64 check's largest deviation, the launch's time and its statistics."""
    import torch

    from . import surrogate_ops as ops

    dev = torch.device("cuda", device)
    wins = [window(k, seed, cells, density) for k in ks]
    targets = torch.empty(len(ks), NCOLS, NROWS, dtype=torch.float32, device=dev)
    from . import autotune

    with engine.Engine(genome.genome_config(), device) as eng:
        autotune.apply_all(eng)
        if smem_budget is not None:
            eng.set_debug_flags(0, smem_budget)
        tasks, bands = [], {}
        for cfg, chrom, bars, _, _ in wins:
            cid = eng.upload_chrom(chrom, bars)
            eng.set_chrom_config(cid, cfg)
            nl = engine.num_lefs(cfg, chrom.simulated_size)
            tg, te = engine.task_targets(cfg, chrom.simulated_size, nl, cells)
            bands[cid] = torch.zeros(NCOLS * NROWS, dtype=torch.int32, device=dev)
            tasks += [(cid, engine.cell_seed(chrom.name, chrom.size, cfg.seed, i), int(tg[i]), te, nl)
                      for i in range(cells)]
        dbands = {c: b.data_ptr() for c, b in bands.items()}
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        _, st = eng.simulate_batch(tasks, dbands)
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
        max_dev = 0.0
        for j, cid in enumerate(sorted(bands)):
            ops.band_target(bands[cid], NCOLS, NROWS, targets[j])
        torch.cuda.synchronize()
        if check:
            for j, cid in enumerate(sorted(bands)):
                want = target_fp64(bands[cid].cpu().numpy().view(np.uint32))
                got = targets[j].double().cpu().numpy()
                max_dev = max(max_dev, float(np.max(np.abs(got - want) / (1.0 + np.abs(want)))))
    track = torch.from_numpy(np.stack([w[3] for w in wins])).to(dev)
    params = torch.from_numpy(np.stack([w[4] for w in wins])).to(dev)
    return {"track": track, "params": params, "target": targets, "fp64_max_rel_dev": max_dev, "ms": ms,
            "cells": len(st), "lef_epochs": int(sum(s.lef_epochs for s in st)),
            "contacts": int(sum(s.contacts for s in st))}


def generate(n, out_dir=None, start=0, chunk=32, seed=2024, cells=1024, density=10.0, device=0, log=None):
    """Simulate parameter sets start .. n - 1 in chunks.  With out_dir, each chunk is written as
    shard_<first index>.npz (track, params, target in FP32) and existing shards are skipped, so
    an interrupted sweep resumes where it stopped.  Returns the in-memory sets (when out_dir is
    None) and the run's totals."""
    sets, totals = [], {"ms": 0.0, "cells": 0, "lef_epochs": 0, "contacts": 0, "fp64_max_rel_dev": 0.0,
                        "maps": 0, "skipped": 0}
    for k0 in range(start, n, chunk):
        ks = list(range(k0, min(n, k0 + chunk)))
        path = os.path.join(out_dir, f"shard_{k0:06d}.npz") if out_dir else None
        if path and os.path.exists(path):
            totals["skipped"] += len(ks)
            continue
        r = simulate_sets(ks, seed, cells, density, device)
        for key in ("ms", "cells", "lef_epochs", "contacts"):
            totals[key] += r[key]
        totals["fp64_max_rel_dev"] = max(totals["fp64_max_rel_dev"], r["fp64_max_rel_dev"])
        totals["maps"] += len(ks)
        if log:
            log(f"sweep sets {ks[0]}..{ks[-1]}: {r['ms'] / 1e3:.1f} s, FP64 check {r['fp64_max_rel_dev']:.2e}")
        if path:
            os.makedirs(out_dir, exist_ok=True)
            tmp = path + ".tmp.npz"
            np.savez(tmp, track=r["track"].cpu().numpy(), params=r["params"].cpu().numpy(),
                     target=r["target"].cpu().numpy(), ks=np.array(ks))
            os.replace(tmp, path)
        else:
            sets.append(r)
    return sets, totals


def load_shards(out_dir):
    """The shards of a sweep directory in index order: (ks, track, params, target) numpy arrays."""
    names = sorted(f for f in os.listdir(out_dir) if f.startswith("shard_") and f.endswith(".npz"))
    parts = [np.load(os.path.join(out_dir, f)) for f in names]
    if not parts:
        return None
    return tuple(np.concatenate([p[key] for p in parts]) for key in ("ks", "track", "params", "target"))
