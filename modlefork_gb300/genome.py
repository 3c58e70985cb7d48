"""Seeded synthetic genomes for the workloads the engine is measured and checked on.

The reference benchmarks on no public dataset (its integration test's GRCh38 inputs are
not shipped), so every workload is generated here from a fixed seed with the shapes of the
parity and genome-scale workloads:

* ``parity_10mbp``: one 10 Mbp chromosome, 5 kb bins, 3 Mbp band (600 x 2000 uint32 band),
  100 barriers at uniform positions with +/- strands (p = 0.5), stp 0.7/0.7 (occupancy 0.5),
  20 LEFs/Mbp, 200 kb lifetime, 2.5 kb/epoch speeds with 5 % std, 64 cells, contact density 1,
  probability normalisation factor 5000 (keeps the stps as stated).
* ``genome_24chr``: 24 chromosomes with lengths uniform in [50, 250] Mbp, one barrier per
  50 kb on average at uniform positions, random strands, occupancy ~ Beta(8, 2) written to
  the BED score, 20 LEFs/Mbp, 200 kb lifetime, default speeds (0.8 x bin), 512 cells each.
* ``batched_windows``: windows of uneven length (log-uniform in [1, 250] Mbp, 4096 of them at
  full size), each with its own configuration: bin size uniform_int{1..10} kb, LEF density
  U(5, 40)/Mbp, barrier density U(5, 40)/Mbp, barriers and the rest as ``genome_24chr``.

Barriers are produced as BED records [p, p + 1) (so the reference's midpoint rule
(start + end + 1) / 2 of genome.cpp:199 puts the barrier at p + 1) in IITree order (sorted by
start, distinct positions), then converted with mgpu_barrier_from_bed.

Every generator takes ``api``: the module or object answering config_defaults,
config_transform, Chromosome and barriers_from_bed (the engine by default).  The CPU arm of the
benchmark passes the oracle's helpers instead, so that it never loads the product library.
"""

import numpy as np

from . import engine


def _distinct_positions(rng, lo, hi, k):
    pos = np.unique(rng.integers(lo, hi, size=k, dtype=np.int64))
    while len(pos) < k:
        extra = rng.integers(lo, hi, size=k - len(pos), dtype=np.int64)
        pos = np.unique(np.concatenate([pos, extra]))
    return np.sort(pos[:k])


def bed_records(rng, length, nbarriers, occupancy=None):
    """BED6-like records (start, end, strand, score) of barriers on [0, length)."""
    starts = _distinct_positions(rng, 0, length - 1, nbarriers)
    strands = np.where(rng.random(nbarriers) < 0.5, "+", "-")
    scores = occupancy if occupancy is not None else np.zeros(nbarriers)
    return [(int(s), int(s) + 1, str(st), float(sc)) for s, st, sc in zip(starts, strands, scores)]


def parity_config(api=None, **overrides):
    """Transformed Config of the 10 Mbp parity workload."""
    api = api or engine
    cfg = api.config_defaults(
        bin_size=5000, diagonal_width=3_000_000, rev_extrusion_speed=2500, fwd_extrusion_speed=2500,
        rev_speed_set=1, fwd_speed_set=1, rev_extrusion_speed_std=0.05, fwd_extrusion_speed_std=0.05,
        number_of_lefs_per_mbp=20.0, avg_lef_processivity=200_000, barrier_occupied_stp=0.7,
        barrier_not_occupied_stp=0.7, probability_normalization_factor=5000, num_cells=64,
        seed=20231203, target_contact_density=1.0)
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return api.config_transform(cfg)


def parity_10mbp(seed=7, api=None, **overrides):
    api = api or engine
    cfg = parity_config(api=api, **overrides)
    rng = np.random.default_rng(seed)
    chrom = api.Chromosome("chrS", 10_000_000)
    recs = bed_records(rng, chrom.size, 100)
    bars = api.barriers_from_bed(chrom, recs, cfg.barrier_occupied_stp, cfg.barrier_not_occupied_stp)
    return cfg, [(chrom, bars)]


def genome_config(api=None, **overrides):
    """Transformed Config of the genome-scale workload (defaults except lifetime, 512 cells)."""
    api = api or engine
    cfg = api.config_defaults(bin_size=5000, diagonal_width=3_000_000, number_of_lefs_per_mbp=20.0,
                              avg_lef_processivity=200_000, num_cells=512, seed=20231203,
                              target_contact_density=1.0)
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return api.config_transform(cfg)


def genome_24chr(seed=11, nchroms=24, min_len=50_000_000, max_len=250_000_000, api=None, **overrides):
    api = api or engine
    cfg = genome_config(api=api, **overrides)
    rng = np.random.default_rng(seed)
    lengths = rng.integers(min_len, max_len + 1, size=nchroms)
    out = []
    for k, L in enumerate(lengths):
        chrom = api.Chromosome(f"chr{k + 1}", int(L))
        nb = int(round(L / 50_000))
        occ = rng.beta(8.0, 2.0, size=nb)
        recs = bed_records(rng, int(L), nb, occ)
        bars = api.barriers_from_bed(chrom, recs, cfg.barrier_occupied_stp, cfg.barrier_not_occupied_stp)
        out.append((chrom, bars))
    return cfg, out


def batched_windows(seed=13, nwindows=4096, min_len=1_000_000, max_len=250_000_000, cells=256, api=None,
                    **overrides):
    """Windows of the batched workload, each a sequence of its own with its own transformed
    configuration; returns a list of (cfg, chrom, barriers)."""
    api = api or engine
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nwindows):
        L = int(round(float(np.exp(rng.uniform(np.log(min_len), np.log(max_len))))))
        bin_size = 1000 * int(rng.integers(1, 11))
        lef_density = float(rng.uniform(5.0, 40.0))
        bar_density = float(rng.uniform(5.0, 40.0))
        cfg = genome_config(api=api, bin_size=bin_size, number_of_lefs_per_mbp=lef_density, num_cells=cells,
                            **overrides)
        chrom = api.Chromosome(f"win{k + 1}", L)
        nb = int(round(L / 1e6 * bar_density))
        occ = rng.beta(8.0, 2.0, size=nb)
        recs = bed_records(rng, L, nb, occ)
        bars = api.barriers_from_bed(chrom, recs, cfg.barrier_occupied_stp, cfg.barrier_not_occupied_stp)
        out.append((cfg, chrom, bars))
    return out
