"""Host driver of a genome-wide run: the task fan-out of Simulation::run_simulate
(src/libmodle/cpu/scheduler_simulate.cpp:110-166) over the engine's batched call.

Per chromosome: the number of LEFs (simulation.cpp:1253-1257), the per-cell contact targets
(scheduler_simulate.cpp:129-153), the per-cell seeds (genome.cpp:317-335), then one
``mgpu_simulate_cells`` call for all of its cells (one launch per chromosome).  Chromosomes
without barriers are skipped unless ``simulate_chromosomes_wo_barriers`` is set
(scheduler_simulate.cpp:114-121).
"""

import gzip

import numpy as np

from . import engine


def _open_text(path):
    """A text file for writing, gzip-compressed when the path ends in .gz."""
    return gzip.open(path, "wt") if str(path).endswith(".gz") else open(path, "w")


class ChromResult:
    def __init__(self, chrom, nlefs, band, missed, stats, occupancy=None, records=None):
        self.chrom = chrom
        self.nlefs = nlefs
        self.band = band
        self.missed = missed
        self.stats = stats
        self.occupancy = occupancy  # 1D LEF occupancy counters (track_1d_lef_position)
        self.records = records      # per-cell lists of model-state records (log_model_internal_state)

    @property
    def lef_epochs(self):
        return int(sum(s.lef_epochs for s in self.stats))

    @property
    def contacts(self):
        return int(sum(s.contacts for s in self.stats))


def prepare_chrom(eng, cfg, chrom, barriers, ncells):
    """Upload one chromosome and compute its task list; returns a dict of launch inputs."""
    size = chrom.simulated_size
    nlefs = engine.num_lefs(cfg, size)
    targets, target_epochs = engine.task_targets(cfg, size, nlefs, ncells)
    seeds = np.array([engine.cell_seed(chrom.name, chrom.size, cfg.seed, i) for i in range(ncells)],
                     dtype=np.uint64)
    cid = eng.upload_chrom(chrom, barriers)
    nrows, ncols = engine.band_shape(cfg, size)
    return dict(chrom=chrom, cid=cid, nlefs=nlefs, targets=targets, target_epochs=target_epochs,
                seeds=seeds, nrows=nrows, ncols=ncols)


# Shared-memory budget per cell when several chromosome launches run at once, and the share of
# the SM's unified memory given to shared memory (the rest is L1 for the per-LEF arrays that
# live in global slots): six cells per SM with a 70 KB L1 measured best on the genome workload.
CONCURRENT_SMEM_BUDGET = 24 * 1024
CONCURRENT_CARVEOUT = 70


def simulate_genome(cfg, genome, ncells=None, device=0, simulate_wo_barriers=False, workers=1,
                    smem_budget=None, max_epoch_records=4096):
    """Run every cell of every chromosome; returns a list of ChromResult in genome order.

    With ``workers`` > 1, that many host threads each drive their own engine context (own
    CUDA stream), taking chromosomes from a queue largest first, so several one-chromosome
    launches share the GPU at once, as the reference's worker threads share its cores.
    ``smem_budget`` caps each cell's shared memory (bytes; default: the device limit with one
    worker, CONCURRENT_SMEM_BUDGET with several)."""
    import queue
    import threading

    ncells = int(cfg.num_cells if ncells is None else ncells)
    jobs = [(i, c, b) for i, (c, b) in enumerate(genome) if b or simulate_wo_barriers]
    if smem_budget is None:
        smem_budget = 0 if workers <= 1 else CONCURRENT_SMEM_BUDGET
    todo = queue.Queue()
    for job in sorted(jobs, key=lambda j: -j[1].simulated_size):
        todo.put(job)
    results, errors = {}, []

    def worker():
        try:
            with engine.Engine(cfg, device) as eng:
                eng.set_debug_flags((CONCURRENT_CARVEOUT << 8) if workers > 1 else 0, smem_budget)
                while True:
                    try:
                        i, chrom, barriers = todo.get_nowait()
                    except queue.Empty:
                        return
                    t = prepare_chrom(eng, cfg, chrom, barriers, ncells)
                    band = np.zeros(t["nrows"] * t["ncols"], dtype=np.uint32)
                    occ, recs = None, None
                    if cfg.track_1d_lef_position or cfg.log_model_internal_state:
                        if cfg.track_1d_lef_position:
                            occ = np.zeros((chrom.size + cfg.bin_size - 1) // cfg.bin_size, dtype=np.uint64)
                        missed, stats, recs = eng.simulate_cells_ex(
                            t["cid"], t["seeds"], t["targets"], t["target_epochs"], t["nlefs"], band,
                            occupancy=occ, max_epoch_records=max_epoch_records if cfg.log_model_internal_state else 0)
                    else:
                        missed, stats = eng.simulate_cells(t["cid"], t["seeds"], t["targets"],
                                                           t["target_epochs"], t["nlefs"], band)
                    results[i] = ChromResult(chrom, t["nlefs"], band, missed, stats, occ, recs)
        except BaseException as e:  # surfaced to the caller below
            errors.append(e)

    threads = [threading.Thread(target=worker) for _ in range(max(1, workers))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    if errors:
        raise errors[0]
    return [results[i] for i, _, _ in jobs]

def simulate_genome_batched(cfg, genome, ncells=None, device=0, simulate_wo_barriers=False, cell_range=None,
                            smem_budget=None, carveout=None):
    """simulate_genome with every chromosome's cells in one batched launch (mgpu_simulate_batch):
    one persistent kernel and one work queue for the whole genome, largest chromosomes first.
    Same results as one launch per chromosome.  cell_range = (lo, hi) simulates only cell ids
    lo .. hi - 1 of each chromosome (one rank's share); their seeds and targets are those of the
    full run.  smem_budget (bytes per cell) and carveout (percent of the SM's unified memory as
    shared memory) replace the tuned launch table's choice when given."""
    ncells = int(cfg.num_cells if ncells is None else ncells)
    lo, hi = cell_range if cell_range is not None else (0, ncells)
    jobs = [(c, b) for c, b in genome if b or simulate_wo_barriers]
    from . import autotune

    with engine.Engine(cfg, device) as eng:
        autotune.apply_all(eng)
        if smem_budget is not None or carveout is not None:
            eng.set_debug_flags((int(carveout or 0) & 0xFF) << 8, int(smem_budget or 0))
        preps, tasks, bands = [], [], {}
        for chrom, barriers in jobs:
            t = prepare_chrom(eng, cfg, chrom, barriers, ncells)
            preps.append(t)
            bands[t["cid"]] = np.zeros(t["nrows"] * t["ncols"], dtype=np.uint32)
            for seed, target in zip(t["seeds"][lo:hi], t["targets"][lo:hi]):
                tasks.append((t["cid"], int(seed), int(target), t["target_epochs"], t["nlefs"]))
        missed, stats = eng.simulate_batch(tasks, bands) if tasks else ({t["cid"]: 0 for t in preps}, [])
    out, k = [], 0
    for t in preps:
        st = stats[k:k + hi - lo]
        k += hi - lo
        out.append(ChromResult(t["chrom"], t["nlefs"], bands[t["cid"]], missed[t["cid"]], st))
    return out


def write_lef_occupancy(path, cfg, results):
    """The 1D LEF occupancy track as bedGraph (chrom, start, end, value), with the values the
    reference writes to its bigwig (Simulation::write_1d_lef_occupancy_to_disk,
    simulation.cpp:214-262): each chromosome's counters divided by its maximum, as float32, one
    interval per bin from the chromosome's start."""
    bin_size = int(cfg.bin_size)
    with _open_text(path) as f:
        for r in results:
            if r.occupancy is None:
                continue
            mx = int(r.occupancy.max()) if r.occupancy.size else 0
            vals = (r.occupancy.astype(np.float64) / float(mx)).astype(np.float32) if mx else \
                np.zeros(r.occupancy.size, np.float32)
            for k, v in enumerate(vals.tolist()):
                s0 = r.chrom.start + k * bin_size
                f.write(f"{r.chrom.name}\t{s0}\t{min(s0 + bin_size, r.chrom.size)}\t{v!r}\n")


def occupancy_values(occupancy):
    """The values Simulation::write_1d_lef_occupancy_to_disk writes (simulation.cpp:245-255):
    each counter divided by the chromosome's largest, in double, then rounded to float32 (an
    all-zero track gives NaN, as 0.0 / 0.0 does there)."""
    occ = np.asarray(occupancy, dtype=np.float64)
    mx = float(occ.max()) if occ.size else 0.0
    with np.errstate(invalid="ignore", divide="ignore"):
        return (occ / mx).astype(np.float32)


def write_lef_occupancy_bigwig(path, cfg, results, chroms):
    """The 1D LEF occupancy track as the reference's bigWig: every chromosome of `chroms`
    (Chromosome objects, the genome's list) in the chromosome tree, and for each result with a
    track one fixed-step run of span = step = bin size from the chromosome's start
    (io::bigwig::Writer::write_range, bigwig_impl.hpp:72-97)."""
    from . import bigwig

    bin_size = int(cfg.bin_size)
    tracks = [bigwig.Track(r.chrom.name, r.chrom.start, bin_size, bin_size, occupancy_values(r.occupancy))
              for r in results if r.occupancy is not None]
    bigwig.write_bigwig(path, [(c.name, int(c.size)) for c in chroms], tracks)


def write_model_state(path, results):
    """Model-state log with the columns of Simulation::dump_stats (simulation.cpp:1166-1224):
    task, epoch, cell, chrom, burn-in, effective barrier occupancy, LEFs, stalled rev / fwd /
    both, LEF-BAR, primary and secondary LEF-LEF collisions, mean loop size.  The task id is the
    chromosome's index in the run times the cell count plus the cell."""
    with _open_text(path) as f:
        for ci, r in enumerate(results):
            if r.records is None:
                continue
            ncells = len(r.records)
            for cell, recs in enumerate(r.records):
                for x in recs:
                    occ = x.barriers_occupied / x.nbarriers if x.nbarriers else float("nan")
                    f.write("\t".join(str(v) for v in (
                        ci * ncells + cell, x.epoch, cell, r.chrom.name, "True" if x.burnin else "False", occ,
                        x.num_lefs, x.stalled_rev, x.stalled_fwd, x.stalled_both, x.lef_bar,
                        x.lef_lef_primary, x.lef_lef_secondary, x.avg_loop_size)) + "\n")


def genome_pixels(cfg, results, genome_chroms=None):
    """Genome-wide pixel table of a run, as a cooler stores it (Cooler::write_or_append_cmatrix_to_file,
    src/libmodle_io/cooler_write_impl.hpp:141-330): bins are numbered across the genome in
    chromosome order, ceil(size / bin) per chromosome, and a band's first bin is its chromosome's
    offset plus ceil(start / bin).  Returns (bin1, bin2, count) numpy arrays sorted by (bin1, bin2).

    ``genome_chroms`` lists every chromosome of the genome in order (default: the simulated ones),
    so that chromosomes skipped by the run still take their bins."""
    chroms = genome_chroms if genome_chroms is not None else [r.chrom for r in results]
    bin_size = int(cfg.bin_size)
    first_bin, acc = {}, 0
    for ch in chroms:
        first_bin[ch.name] = acc
        acc += (ch.size + bin_size - 1) // bin_size
    b1s, b2s, cs = [], [], []
    with engine.Engine(cfg) as eng:
        for r in results:
            nrows, ncols = engine.band_shape(cfg, r.chrom.simulated_size)
            off = first_bin[r.chrom.name] + (r.chrom.start + bin_size - 1) // bin_size
            _, b1, b2, c = eng.band_to_pixels(r.band, nrows, ncols, off)
            b1s.append(b1)
            b2s.append(b2)
            cs.append(c)
    cat = (lambda xs, dt: np.concatenate(xs) if xs else np.zeros(0, dt))
    return cat(b1s, np.int64), cat(b2s, np.int64), cat(cs, np.uint32)


def _main(argv=None):
    """Run one workload and print its throughput, e.g. for profiling one launch:

    python -m modlefork_gb300.simulate --workload genome --chrom 0 --cells 64
    """
    import argparse
    import json
    import time

    from . import genome as gen

    ap = argparse.ArgumentParser(description=_main.__doc__)
    ap.add_argument("--workload", choices=["parity", "genome"], default="genome")
    ap.add_argument("--chrom", type=int, action="append", help="chromosome index (repeatable)")
    ap.add_argument("--chroms", type=int, default=24, help="chromosomes of the generated genome workload")
    ap.add_argument("--contact-density", type=float, default=None, help="target contact density")
    ap.add_argument("--cells", type=int, default=None)
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--workers", type=int, default=1, help="concurrent chromosome launches")
    ap.add_argument("--batched", action="store_true", help="all chromosomes in one batched launch")
    ap.add_argument("--smem-budget", type=int, default=None, help="shared memory per cell (bytes)")
    ap.add_argument("--carveout", type=int, default=None,
                    help="batched launch: percent of the SM's unified memory used as shared memory")
    ap.add_argument("--pixels", default=None, help="write the pixel table (bin1_id, bin2_id, count) as TSV")
    ap.add_argument("--lef-occupancy", default=None,
                    help="track the 1D LEF occupancy, write it as bigWig (.bw, .bigwig) or bedGraph")
    ap.add_argument("--model-state", default=None, help="log the per-epoch model state as TSV")
    args = ap.parse_args(argv)
    ov = {} if args.contact_density is None else {"target_contact_density": args.contact_density}
    cfg, g = gen.parity_10mbp(**ov) if args.workload == "parity" else gen.genome_24chr(nchroms=args.chroms, **ov)
    if args.chrom:
        g = [g[i] for i in args.chrom]
    if args.cells is not None:
        cfg.num_cells = args.cells
    cfg.track_1d_lef_position = 1 if args.lef_occupancy else 0
    cfg.log_model_internal_state = 1 if args.model_state else 0
    t0 = time.perf_counter()
    if args.batched:
        res = simulate_genome_batched(cfg, g, device=args.device, smem_budget=args.smem_budget,
                                      carveout=args.carveout)
    else:
        res = simulate_genome(cfg, g, device=args.device, workers=args.workers, smem_budget=args.smem_budget)
    dt = time.perf_counter() - t0
    if args.pixels:
        b1, b2, cnt = genome_pixels(cfg, res, [c for c, _ in g])
        with _open_text(args.pixels) as f:
            f.write("bin1_id\tbin2_id\tcount\n")
            for a, b, c in zip(b1.tolist(), b2.tolist(), cnt.tolist()):
                f.write(f"{a}\t{b}\t{c}\n")
    if args.lef_occupancy:
        if args.lef_occupancy.lower().endswith((".bw", ".bigwig")):
            write_lef_occupancy_bigwig(args.lef_occupancy, cfg, res, [c for c, _ in g])
        else:
            write_lef_occupancy(args.lef_occupancy, cfg, res)
    if args.model_state:
        write_model_state(args.model_state, res)
    le = sum(r.lef_epochs for r in res)
    print(json.dumps({"workload": args.workload, "chromosomes": [r.chrom.name for r in res],
                      "cells": int(cfg.num_cells), "workers": args.workers, "lef_epochs": le, "contacts": sum(r.contacts for r in res),
                      "wall_s": dt, "lef_epochs_per_s": le / dt}))


if __name__ == "__main__":
    _main()
