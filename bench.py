#!/usr/bin/env python3
"""Benchmark of the loop-extrusion epoch engine on the genome-scale workload.

Workload: 24 synthetic chromosomes, lengths uniform in [50, 250] Mbp, 5 kb bins, 3 Mbp band,
one barrier per 50 kb (Beta(8, 2) occupancy), 20 LEFs/Mbp, 200 kb lifetime, 512 cells per
chromosome, contact density 1, one engine launch per chromosome.  One step is the whole genome:
the 24 launches run at once from 24 engine contexts (host threads, CUDA streams), each cell
with a 24 KiB shared-memory budget and a 70 % shared-memory carveout.  The metric is
LEF-epochs/s (sum over cells and epochs of active LEFs, burn-in included), with cells/s and
contacts/s reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``value`` is timed with CUDA events around K steps whose inputs (seeds, targets, bands)
are already in device memory; ``e2e`` repeats the step through the C ABI with host buffers
(host-to-device copies of the inputs and the band, device-to-host copies of the band and the
per-cell statistics inside the timed region).  ``--impl reference`` times the reference
algorithm on the host cores instead (the CPU oracle, a restatement of the reference, since
the reference's own build needs dependencies this machine does not have) on a bounded sample
of the same workload.
"""

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "genome_24chr_50-250Mbp_5kb_512cells"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cells", type=int, default=512, help="cells per chromosome")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU baseline time budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--serial-every", type=int, default=3,
                    help="plain path one launch at a time over every n-th chromosome (0 = skip)")
    ap.add_argument("--workers", type=int, default=24, help="concurrent engine contexts")
    ap.add_argument("--wave", type=int, default=24, help="chromosome launches per step")
    ap.add_argument("--smem-budget", type=int, default=None, help="shared memory per cell (bytes)")
    ap.add_argument("--carveout", type=int, default=None, help="shared-memory carveout percent")
    ap.add_argument("--wave-steps", type=int, default=1,
                    help="timed steps of the plain path (one-chromosome launches from concurrent contexts)")
    ap.add_argument("--windows", type=int, default=16,
                    help="windows of the batched uneven-window workload timed in one launch (0 = skip)")
    ap.add_argument("--surrogate", type=int, default=1, help="also time the learned surrogate against the simulator")
    ap.add_argument("--sur-maps", type=int, default=16, help="fresh simulator maps the surrogate is scored on")
    return ap.parse_args()


# ---------------------------------------------------------------------------------------------
def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """nvidia-smi sampler for the timed region (SM clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
            os.close(fd)
            self.out = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.out,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.out.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[4:]))
            except ValueError:
                continue
        os.remove(self.path)
        if not rows:
            return None
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = set()
        for _, _, flags in rows:
            for name, v in zip(names[1:], flags[1:]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": sorted(reasons), "samples": len(rows)}


def measured_peak(key="hbm_gbs"):
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return float(d[key]), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}[key], "fallback"


SUR_HELD_BASE = 2_000_000  # parameter sets neither the training nor its evaluation used


def run_windows(args, device, log):
    """The batched workload of uneven windows: the first ``args.windows`` of the 4096 seeded
    windows (lengths log-uniform in [1, 250] Mbp, bin 1-10 kb, LEF and barrier densities
    U(5, 40)/Mbp, each with its own configuration) x 256 cells in one batched launch.  A sample
    of cells is re-simulated by plain per-window launches on engines created with each window's
    configuration and must give identical per-cell results."""
    import torch

    from modlefork_gb300 import engine, genome

    cells = 256
    wins = genome.batched_windows(seed=13, nwindows=args.windows, cells=cells)
    dev = torch.device("cuda", device)
    from modlefork_gb300 import autotune

    with engine.Engine(genome.genome_config(), device) as eng:
        autotune.apply_all(eng)
        tasks, bands, meta = [], {}, []
        for cfg, chrom, bars in wins:
            cid = eng.upload_chrom(chrom, bars)
            eng.set_chrom_config(cid, cfg)
            nl = engine.num_lefs(cfg, chrom.simulated_size)
            tg, te = engine.task_targets(cfg, chrom.simulated_size, nl, cells)
            nrows, ncols = engine.band_shape(cfg, chrom.simulated_size)
            bands[cid] = torch.zeros(nrows * ncols, dtype=torch.int32, device=dev)
            seeds = [engine.cell_seed(chrom.name, chrom.size, cfg.seed, i) for i in range(cells)]
            meta.append((cfg, chrom, bars, nl, seeds, [int(x) for x in tg], te, len(tasks)))
            tasks += [(cid, sd, int(t), te, nl) for sd, t in zip(seeds, tg)]
        dbands = {c: b.data_ptr() for c, b in bands.items()}
        torch.cuda.synchronize()
        log(f"uneven windows: {len(wins)} windows x {cells} cells in one batched launch")
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        _, st = eng.simulate_batch(tasks, dbands)
        ev1.record()
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1)
    # sampled bit-exactness: the cheapest windows' first two cells through plain launches
    order = sorted(range(len(meta)), key=lambda k: meta[k][3] * meta[k][6])[:4]
    compared = equal = 0
    for k in order:
        cfg, chrom, bars, nl, seeds, tg, te, first = meta[k]
        with engine.Engine(cfg, device) as eng:
            cid = eng.upload_chrom(chrom, bars)
            _, pst = eng.simulate_cells(cid, np.array(seeds[:2], dtype=np.uint64), np.array(tg[:2], dtype=np.uint64),
                                        te, nl)
        for i in range(2):
            a, b = pst[i], st[first + i]
            compared += 1
            equal += int((a.epochs, a.burnin_epochs, a.contacts, a.missed_updates, a.lef_epochs, a.rng_draws) ==
                         (b.epochs, b.burnin_epochs, b.contacts, b.missed_updates, b.lef_epochs, b.rng_draws))
    le = sum(x.lef_epochs for x in st)
    return {"windows": len(wins), "of_windows": 4096, "cells_per_window": cells, "cells": len(st),
            "window_mbp": float(sum(w[1].size for w in wins) / 1e6),
            "bin_sizes_kb": sorted({int(w[0].bin_size // 1000) for w in wins}),
            "ms": ms, "value": le / (ms / 1e3), "unit": "LEF-epochs/s", "cells_per_s": len(st) / (ms / 1e3),
            "contacts_per_s": sum(x.contacts for x in st) / (ms / 1e3), "launches": 1,
            "parity_sample": {"cells": compared, "equal": equal,
                              "against": "plain per-window launches on engines with each window's configuration"},
            "note": "the first windows of the seeded 4096-window workload (a stated subset); the whole "
                    "workload is about 2e12 LEF-epochs.  One warp advances one cell, so the launch's tail "
                    "is the longest cell: the fourth window (170 Mbp at 1 kb bins, 6450 LEFs, about 1e4 epochs per "
                    "cell) sets this subset's time"}


def run_surrogate(args, log):
    """The learned surrogate against the batched simulator on fresh 20 Mbp windows: the
    committed network (modlefork_gb300/data/surrogate_unet.npz) predicts each window's map,
    scored by Pearson r and relative L2 against the simulator's map of the same window (1024
    cells, contact density 10); maps below the r gate fall back to the simulator.  maps/s of the
    surrogate at inference batch 256 (inputs resident, CUDA events) and end to end (host inputs
    in, predicted maps back to host memory), against the simulator's maps/s on these windows."""
    import torch

    from modlefork_gb300 import surrogate as S
    from modlefork_gb300 import sweep
    from modlefork_gb300 import train_surrogate as T

    from modlefork_gb300 import autotune

    autotune.apply_all()
    net = T.load_weights(os.path.join(ROOT, "modlefork_gb300", "data", "surrogate_unet.npz"))
    n = args.sur_maps
    log(f"surrogate: simulating {n} fresh windows")
    sims = sweep.simulate_sets(list(range(SUR_HELD_BASE, SUR_HELD_BASE + n)), cells=1024, density=10.0)
    data = S.Dataset(sims["track"], sims["params"], sims["target"], net.dev)
    r, rel = S.evaluate(S.predict(net, data.x), data.target)
    sim_mps = n / (sims["ms"] / 1e3)
    log("surrogate: inference")
    mps, ms, tf = T.inference_rate(net, data.x, batch=256, reps=20)
    # end to end: host tracks and parameters in, predicted maps back to pinned host memory through
    # S.predict_host (batches of 256; each batch's copy back overlaps the next batch's forward)
    B, nbatch = 256, 4
    idx = np.arange(B * nbatch) % n
    pin_track = torch.from_numpy(sims["track"].cpu().numpy()[idx].copy()).pin_memory()
    pin_params = torch.from_numpy(sims["params"].cpu().numpy()[idx].copy()).pin_memory()
    pin_out = torch.empty(B * nbatch, net.length, S.NROWS, dtype=torch.float32).pin_memory()
    S.predict_host(net, pin_track, pin_params, pin_out, batch=B)  # warm-up: every part of the buffers
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    S.predict_host(net, pin_track, pin_params, pin_out, batch=B)
    torch.cuda.synchronize()
    e2e_mps = B * nbatch / (time.perf_counter() - t0)
    # the link that bounds it: one batch of maps copied device-to-host into each batch's part of
    # the same pinned buffer (the rate depends on where the host placed those pinned pages, which
    # varies between runs and can differ between parts of one large buffer)
    d_maps = torch.empty(B, net.length, S.NROWS, dtype=torch.float32, device=net.dev)
    d2h_parts = []
    for k in range(nbatch):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pin_out[k * B:(k + 1) * B].copy_(d_maps, non_blocking=True)
        torch.cuda.synchronize()
        d2h_parts.append(d_maps.numel() * 4 / (time.perf_counter() - t0) / 1e9)
    d2h_gbs = nbatch / sum(1.0 / g for g in d2h_parts)
    del d_maps
    passed = r >= 0.95
    tpeak, tkind = measured_peak("bf16_tflops")
    eff = 1.0 / (1.0 / mps + (1.0 - passed.mean()) / sim_mps)
    return {
        "metric": "maps/s", "value": mps, "unit": "maps/s", "batch": B, "ms_per_batch": ms,
        "maps_scored": n, "mean_r": float(r.mean()), "min_r": float(r.min()), "mean_rel_l2": float(rel.mean()),
        "gate_r": 0.95, "maps_passing_gate": int(passed.sum()),
        "gated_maps_per_s": eff, "simulator_maps_per_s": sim_mps, "over_simulator": mps / sim_mps,
        "gated_over_simulator": eff / sim_mps,
        "simulator_config": "20 Mbp windows of the sweep generator, 1024 cells, contact density 10, one batched "
                            "launch (CUDA events around the launch)",
        "fp64_target_check_max_rel_dev": sims["fp64_max_rel_dev"],
        "e2e": {"value": e2e_mps, "unit": "maps/s", "batches": nbatch, "d2h_gb_per_s": d2h_gbs,
                "d2h_gb_per_s_by_batch": d2h_parts,
                "d2h_bound_maps_per_s": d2h_gbs * 1e9 / (net.length * S.NROWS * 4),
                "h2d_bytes_per_step": int((pin_track.numel() + pin_params.numel()) * 4) // nbatch,
                "d2h_bytes_per_step": int(pin_out.numel() * 4) // nbatch},
        "roofline": {"bound": "tensor", "achieved": tf, "peak": tpeak, "unit": "TFLOP/s", "frac": tf / tpeak,
                     "peak_source": f"{tkind} bf16_tflops", "flops_model": "2 x multiply-adds of the network's "
                     f"convolutions per map ({net.flops_per_map() / 1e9:.2f} GFLOP) x maps / time",
                     "traffic": None},
        "nparams": net.nparams, "dtype": "bf16 operands, fp32 accumulate",
    }


def dram_traffic_per_launch(lef_epochs_per_launch, kernel="simulate_kernel"):
    """DRAM bytes per launch of a simulation kernel, from the committed ncu capture's bytes per
    LEF-epoch (one launch of the same kernel and layout) scaled to this run's launches."""
    path = os.path.join(ROOT, "profiles", f"{kernel}_traffic.json")
    if os.path.exists(path):
        d = json.load(open(path))
        return d["bytes_per_lef_epoch"] * lef_epochs_per_launch, d
    return None, None


# ---------------------------------------------------------------------------------------------
def build_workload(cells, rank, api=None):
    """The genome workload's tasks.  ``api`` answers the host helpers (seeds, LEF counts, task
    targets, band shapes): the engine for our arm, the oracle's helpers for the CPU arm, which
    must not load the product library."""
    from modlefork_gb300 import genome

    if api is None:
        from modlefork_gb300 import engine as api
    cfg, gen = genome.genome_24chr(seed=11, api=api)
    tasks = []
    for chrom, bars in gen:
        size = chrom.simulated_size
        nl = api.num_lefs(cfg, size)
        targets, te = api.task_targets(cfg, size, nl, cells)
        base = rank * cells  # weak scaling: each rank simulates its own cell ids
        seeds = np.array([api.cell_seed(chrom.name, chrom.size, cfg.seed, base + i) for i in range(cells)],
                         dtype=np.uint64)
        nrows, ncols = api.band_shape(cfg, size)
        tasks.append(dict(chrom=chrom, bars=bars, nlefs=nl, targets=targets, te=te, seeds=seeds,
                          nrows=nrows, ncols=ncols))
    return cfg, tasks


def algorithmic_bytes(stats, nbarriers):
    """B_epoch = 24 A + 6 N_b + 8 C summed over the cell-epochs of one launch."""
    lef_epochs = sum(s.lef_epochs for s in stats)
    epochs = sum(s.epochs for s in stats)
    contacts = sum(s.contacts for s in stats)
    return 24 * lef_epochs + 6 * nbarriers * epochs + 8 * contacts


def cpu_sample(cfg, task, budget_s, threads):
    """Time the oracle on whole cells of one chromosome with all host threads."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _harness import load_oracle, make_chrom
    from modlefork_gb300 import _abi as abi

    lib = load_oracle()
    chrom = task["chrom"]
    bs = abi.make_barriers(task["bars"])
    ch = make_chrom(chrom.start, chrom.end, chrom.size, chrom.name.encode())
    band = np.zeros(task["nrows"] * task["ncols"], dtype=np.uint32)
    done_cells = lef_epochs = contacts = 0
    per_cell = []
    t0 = time.perf_counter()
    i0 = 0
    while i0 < len(task["seeds"]) and (done_cells == 0 or time.perf_counter() - t0 < budget_s):
        n = min(threads, len(task["seeds"]) - i0)
        st = (abi.CellStats * n)()
        missed = C.c_uint64(0)
        seeds = np.ascontiguousarray(task["seeds"][i0:i0 + n])
        targets = np.ascontiguousarray(task["targets"][i0:i0 + n])
        rc = lib.orc_simulate_cells_mt(C.byref(cfg), C.byref(ch), bs, len(task["bars"]),
                                       seeds.ctypes.data_as(C.POINTER(C.c_uint64)),
                                       targets.ctypes.data_as(C.POINTER(C.c_uint64)), task["te"],
                                       task["nlefs"], n, threads,
                                       band.ctypes.data_as(C.POINTER(C.c_uint32)), C.byref(missed), st)
        if rc != 0:
            raise RuntimeError(f"oracle failed with {rc}")
        done_cells += n
        lef_epochs += sum(s.lef_epochs for s in st)
        contacts += sum(s.contacts for s in st)
        per_cell += [(i0 + j, st[j].epochs, st[j].contacts, st[j].rng_draws, st[j].lef_epochs) for j in range(n)]
        i0 += n
    dt = time.perf_counter() - t0
    return dict(seconds=dt, cells=done_cells, lef_epochs=lef_epochs, contacts=contacts, per_cell=per_cell,
                sample=f"{chrom.name} ({chrom.size / 1e6:.1f} Mbp, {task['nlefs']} LEFs, "
                       f"{len(task['bars'])} barriers): cells 0..{done_cells - 1} of {len(task['seeds'])}, "
                       f"{threads} threads")


def cpu_sample_genome(cfg, tasks, budget_s, threads, first=0):
    """Time the oracle on the genome's mix: one batch of ``threads`` whole cells from each
    chromosome in turn (chromosome ``first`` onwards, largest and smallest alike) until the
    budget is spent."""
    total = dict(seconds=0.0, cells=0, lef_epochs=0, contacts=0, per_cell={})
    names, k = [], first
    while total["seconds"] < budget_s and len(names) < len(tasks):
        t = tasks[k % len(tasks)]
        s = cpu_sample(cfg, t, 0.0, threads)  # one batch
        for key in ("seconds", "cells", "lef_epochs", "contacts"):
            total[key] += s[key]
        total["per_cell"][k % len(tasks)] = s["per_cell"]
        names.append(t["chrom"].name)
        k += 1
    total["sample"] = (f"{threads} whole cells (ids 0..{threads - 1}) of each of {len(names)} chromosomes "
                       f"({names[0]}..{names[-1]}, {sum(tasks[(first + i) % len(tasks)]['nlefs'] for i in range(len(names))) // len(names)} "
                       f"LEFs on average), {threads} threads")
    return total


# ---------------------------------------------------------------------------------------------
def run_reference(args):
    world, rank, _ = dist_env()
    if world > 1 and rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _harness import OracleHelpers

    # the workload's seeds, targets and barriers come from the oracle's own helpers: this arm
    # loads liboracle.so and nothing of the product
    cfg, tasks = build_workload(args.cells, 0, api=OracleHelpers())
    threads = os.cpu_count() or 1
    per_step = max(1.0, args.cpu_seconds / 2)
    for _ in range(args.warmup):
        cpu_sample(cfg, tasks[0], 0.1, threads)  # one batch
    rates, samples, secs = [], [], 0.0
    for i in range(args.steps):
        s = cpu_sample_genome(cfg, tasks, per_step, threads, first=i * 7)
        rates.append(s["lef_epochs"] / s["seconds"])
        samples.append(s)
        secs += s["seconds"]
    value = sum(s["lef_epochs"] for s in samples) / secs
    line = {
        "impl": "reference", "metric": "LEF-epochs/s", "value": value, "unit": "LEF-epochs/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1000 * secs / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64+f64", "data": "synthetic",
        "config": {"workload": WORKLOAD, "sample_per_step": samples[0]["sample"],
                   "same_config_note": "the same genome workload as our arm; each step times a bounded "
                                       "sample of it (whole cells of every chromosome in turn), so the "
                                       "rate is comparable while the cells timed are a subset"},
        "cpu_baseline": {"value": value, "unit": "LEF-epochs/s", "cores": threads, "kind": "port",
                         "sample": samples[0]["sample"]},
        "e2e": {"value": value, "unit": "LEF-epochs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "cells_per_s": sum(s["cells"] for s in samples) / secs,
        "contacts_per_s": sum(s["contacts"] for s in samples) / secs,
    }
    print(json.dumps(line), flush=True)


def log(msg):
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def run_ours(args):
    import queue
    import threading

    import torch

    world, rank, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    from modlefork_gb300 import autotune
    from modlefork_gb300 import build as mbuild
    from modlefork_gb300 import engine
    from modlefork_gb300.simulate import CONCURRENT_CARVEOUT, CONCURRENT_SMEM_BUDGET

    mbuild.build()
    cfg, tasks = build_workload(args.cells, rank)
    log("workload ready")
    dev = torch.device("cuda", local)
    budget = args.smem_budget if args.smem_budget is not None else (
        0 if args.workers == 1 else CONCURRENT_SMEM_BUDGET)
    carveout = args.carveout if args.carveout is not None else (0 if args.workers == 1 else CONCURRENT_CARVEOUT)
    for t in tasks:
        t["d_seeds"] = torch.from_numpy(t["seeds"].view(np.int64)).to(dev)
        t["d_targets"] = torch.from_numpy(t["targets"].view(np.int64)).to(dev)
        t["d_band"] = torch.zeros(t["nrows"] * t["ncols"], dtype=torch.int32, device=dev)
    workers = []
    for _ in range(args.workers):
        eng = engine.Engine(cfg, local)
        eng.set_debug_flags((carveout & 0xFF) << 8, budget)
        stream = torch.cuda.Stream(device=dev)
        eng.set_stream(stream.cuda_stream)
        cids = [eng.upload_chrom(t["chrom"], t["bars"]) for t in tasks]
        workers.append(dict(eng=eng, stream=stream, cids=cids))
    torch.cuda.synchronize()
    wave = max(1, min(args.wave, len(tasks)))

    def run_wave(i, device_inputs):
        """Step i: chromosomes (i*wave + j) mod 24, j < wave, largest first over the workers."""
        ids = sorted({(i * wave + j) % len(tasks) for j in range(wave)}, key=lambda k: -tasks[k]["nlefs"])
        todo = queue.Queue()
        for k in ids:
            todo.put(k)
        done, errors = [], []

        def work(w):
            try:
                while True:
                    try:
                        k = todo.get_nowait()
                    except queue.Empty:
                        return
                    t = tasks[k]
                    if device_inputs:
                        _, st = w["eng"].simulate_cells(w["cids"][k], t["d_seeds"].data_ptr(),
                                                        t["d_targets"].data_ptr(), t["te"], t["nlefs"],
                                                        t["d_band"].data_ptr(), ncells=len(t["seeds"]))
                    else:
                        _, st = w["eng"].simulate_cells(w["cids"][k], t["seeds"], t["targets"], t["te"],
                                                        t["nlefs"], t["h_band"])
                    done.append((k, st, w["eng"].last_kernel_ms()))
            except BaseException as e:
                errors.append(e)

        threads = [threading.Thread(target=work, args=(w,)) for w in workers]
        for th in threads:
            th.start()
        for th in threads:
            th.join()
        if errors:
            raise errors[0]
        return done

    def tally(done):
        agg = dict(lef_epochs=0, cells=0, contacts=0, bytes=0, kernel_ms=0.0, launches=0)
        for k, st, kms in done:
            agg["lef_epochs"] += sum(s.lef_epochs for s in st)
            agg["contacts"] += sum(s.contacts for s in st)
            agg["cells"] += len(st)
            agg["bytes"] += algorithmic_bytes(st, len(tasks[k]["bars"]))
            agg["kernel_ms"] += kms
            agg["launches"] += 1
        return agg

    # ---- headline: the whole genome in one batched launch per step (mgpu_simulate_batch) -------
    # One persistent kernel and one work queue over every chromosome's cells, largest first: the
    # GB300 form of the reference's task queue of (chromosome, cell) tasks over worker threads.
    w0 = workers[0]
    w0["eng"].set_debug_flags(0, 0)
    tuning = autotune.apply_all(w0["eng"])
    btasks = [(w0["cids"][k], int(sd), int(tg), t["te"], t["nlefs"])
              for k, t in enumerate(tasks) for sd, tg in zip(t["seeds"], t["targets"])]
    dbands = {w0["cids"][k]: t["d_band"].data_ptr() for k, t in enumerate(tasks)}

    def batched_tally(bst):
        agg = dict(lef_epochs=0, cells=len(bst), contacts=0, bytes=0, launches=1)
        off = 0
        for t in tasks:
            st = bst[off:off + len(t["seeds"])]
            agg["lef_epochs"] += sum(x.lef_epochs for x in st)
            agg["contacts"] += sum(x.contacts for x in st)
            agg["bytes"] += algorithmic_bytes(st, len(t["bars"]))
            off += len(t["seeds"])
        return agg

    for i in range(args.warmup):
        log(f"warm-up step {i}")
        w0["eng"].simulate_batch(btasks, dbands)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(w0["stream"])
    first_step, agg = None, dict(lef_epochs=0, cells=0, contacts=0, bytes=0, launches=0)
    for i in range(args.steps):
        log(f"timed step {i}")
        _, bst = w0["eng"].simulate_batch(btasks, dbands)
        first_step = first_step if first_step is not None else bst
        for key, v in batched_tally(bst).items():
            agg[key] += v
    ev1.record(w0["stream"])
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    log(f"timed region: {ms:.1f} ms")
    if world > 1:
        from modlefork_gb300 import sharding

        ms, sums = sharding.reduce_timing(ms, {k: agg[k] for k in ("lef_epochs", "cells", "contacts", "bytes",
                                                                    "launches")}, device=dev)
        agg.update(sums)
        torch.distributed.barrier()
    done = []  # (chromosome, stats) of the first timed step, for the parity check
    off = 0
    for k, t in enumerate(tasks):
        done.append((k, first_step[off:off + len(t["seeds"])], 0.0))
        off += len(t["seeds"])

    # end to end through the C ABI with host buffers (copies inside the timed region)
    e2e = None
    if args.e2e_steps > 0:
        hb = {w0["cids"][k]: np.zeros(t["nrows"] * t["ncols"], dtype=np.uint32) for k, t in enumerate(tasks)}
        torch.cuda.synchronize()
        step_rates, dt, ele, ecells = [], 0.0, 0, 0
        for i in range(args.e2e_steps):
            log(f"e2e step {i}")
            for b in hb.values():
                b[:] = 0
            t0 = time.perf_counter()
            _, est = w0["eng"].simulate_batch(btasks, hb)
            torch.cuda.synchronize()
            sdt = time.perf_counter() - t0
            dt += sdt
            sle = sum(x.lef_epochs for x in est)
            step_rates.append(sle / sdt)
            ele += sle
            ecells += len(est)
        e2e = {"value": ele / dt, "unit": "LEF-epochs/s",
               "h2d_bytes_per_step": int(sum(b.nbytes for b in hb.values()) + len(btasks) * 40),
               "d2h_bytes_per_step": int(sum(b.nbytes for b in hb.values()) + len(btasks) * 64),
               "steps": args.e2e_steps, "cells_per_s": ecells / dt,
               "step_rates": {"min": min(step_rates), "median": statistics.median(step_rates),
                              "max": max(step_rates)},
               "timing": "host clock around each step's C-ABI call (task list, band buffers and per-cell "
                         "stats copied in and out inside it) and a device synchronisation"}

    # the plain path: one-chromosome launches (mgpu_simulate_cells) from concurrent contexts
    wave_line = None
    if args.wave_steps > 0:
        for w in workers:
            w["eng"].set_debug_flags((carveout & 0xFF) << 8, budget)
        log("plain wave warm-up")
        run_wave(0, True)
        torch.cuda.synchronize()
        main = torch.cuda.current_stream()
        wev0, wev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        wev0.record(main)
        for w in workers:
            w["stream"].wait_event(wev0)
        wdone = []
        for i in range(args.wave_steps):
            log(f"plain wave step {i}")
            wdone += run_wave(i, True)
        for w in workers:
            main.wait_stream(w["stream"])
        wev1.record(main)
        torch.cuda.synchronize()
        wms = wev0.elapsed_time(wev1)
        wagg = tally(wdone)
        wave_line = {"value": wagg["lef_epochs"] / (wms / 1e3), "unit": "LEF-epochs/s", "steps": args.wave_steps,
                     "warmup": 1, "ms_per_step": wms / args.wave_steps, "cells_per_s": wagg["cells"] / (wms / 1e3),
                     "launches": int(wagg["launches"]),
                     "step": f"one wave of {wave} one-chromosome launches ({args.cells} cells each) over "
                             f"{args.workers} concurrent contexts",
                     "smem_budget_per_cell": budget, "smem_carveout_pct": carveout,
                     "bytes": wagg["bytes"], "ms": wms}

    # the plain path one launch at a time: one context, every n-th chromosome's 512 cells in
    # one blocking call after another (the reference's drop-in used from a single worker), and
    # the batched engine on exactly the same cells
    serial = None
    if args.serial_every > 0:
        w0 = workers[0]
        w0["eng"].set_debug_flags(0, 0)
        ks = list(range(0, len(tasks), args.serial_every))
        log(f"plain path one launch at a time over {len(ks)} chromosomes")
        torch.cuda.synchronize()
        sev0, sev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        sev0.record(w0["stream"])
        sst = []
        for k in ks:
            t = tasks[k]
            _, st = w0["eng"].simulate_cells(w0["cids"][k], t["d_seeds"].data_ptr(), t["d_targets"].data_ptr(),
                                             t["te"], t["nlefs"], t["d_band"].data_ptr(), ncells=len(t["seeds"]))
            sst += list(st)
        sev1.record(w0["stream"])
        torch.cuda.synchronize()
        sms = sev0.elapsed_time(sev1)
        btasks_s = [(w0["cids"][k], int(sd), int(tg), tasks[k]["te"], tasks[k]["nlefs"])
                    for k in ks for sd, tg in zip(tasks[k]["seeds"], tasks[k]["targets"])]
        log("batched launch over the same chromosomes")
        bs0, bs1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        bs0.record(w0["stream"])
        _, bsst = w0["eng"].simulate_batch(btasks_s, {w0["cids"][k]: tasks[k]["d_band"].data_ptr() for k in ks})
        bs1.record(w0["stream"])
        torch.cuda.synchronize()
        bsms = bs0.elapsed_time(bs1)
        same = all(a.epochs == b.epochs and a.contacts == b.contacts and a.rng_draws == b.rng_draws
                   for a, b in zip(sst, bsst))
        serial = {"chromosomes": [tasks[k]["chrom"].name for k in ks], "cells": len(sst), "ms": sms,
                  "value": sum(x.lef_epochs for x in sst) / (sms / 1e3), "unit": "LEF-epochs/s",
                  "cells_per_s": len(sst) / (sms / 1e3), "launches": len(ks),
                  "batched_same_cells": {"ms": bsms, "cells_per_s": len(bsst) / (bsms / 1e3),
                                         "value": sum(x.lef_epochs for x in bsst) / (bsms / 1e3),
                                         "per_cell_stats_equal": bool(same)},
                  "batched_over_serial_cells_per_s": (len(bsst) / bsms) / (len(sst) / sms)}

    if rank != 0:
        return
    peak, peak_kind = measured_peak()
    achieved = agg["bytes"] / (ms / 1e3) / 1e9
    traffic, tinfo = dram_traffic_per_launch(agg["lef_epochs"] / max(1, agg["launches"]), "simulate_batch_kernel")
    line = {
        "metric": "LEF-epochs/s", "value": agg["lef_epochs"] / (ms / 1e3), "unit": "LEF-epochs/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32+f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "chromosomes": len(tasks), "cells_per_chromosome": args.cells,
                   "step": f"one batched launch (mgpu_simulate_batch) of all {len(tasks)} chromosomes x "
                           f"{args.cells} cells, one work queue, largest chromosomes first",
                   "launch_settings": ("the tuned table (modlefork_gb300/data/tuning_gb300.json)" if tuning
                                       else "16 KiB per cell, 60% carveout"),
                   "genome_bp": int(sum(t["chrom"].size for t in tasks)),
                   "lefs": int(sum(t["nlefs"] for t in tasks)),
                   "barriers": int(sum(len(t["bars"]) for t in tasks)),
                   "l2": "inputs larger than L2 (contact bands total "
                         f"{sum(t['nrows'] * t['ncols'] * 4 for t in tasks) / 1e9:.2f} GB)"},
        "cells_per_s": agg["cells"] / (ms / 1e3), "contacts_per_s": agg["contacts"] / (ms / 1e3),
        "gpu_launches": int(agg["launches"]),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": f"{peak_kind} hbm_gbs", "kernel": "simulate_batch_kernel",
                     "bytes_model": "24*LEF_epochs + 6*barriers*epochs + 8*contacts per launch / launch time",
                     "traffic_note": "DRAM bytes per launch: ncu bytes per LEF-epoch of a one-wave batched "
                                     "launch (profiles/simulate_batch_kernel_traffic.json) x this launch's "
                                     "LEF-epochs; above the algorithmic bytes because the resident cells' "
                                     "arrays exceed L2",
                     "traffic_over_algorithmic": None},
        "e2e": e2e, "clocks": clk, "plain_wave": wave_line, "plain_serial": serial,
    }
    if traffic is not None and agg["bytes"]:
        line["roofline"]["traffic_over_algorithmic"] = traffic * agg["launches"] / agg["bytes"]
        line["roofline"]["captured_launch_lef_epochs_per_s"] = tinfo.get("lef_epochs_per_s")
    if wave_line is not None:
        wach = wave_line.pop("bytes") / (wave_line["ms"] / 1e3) / 1e9
        wtraffic, _ = dram_traffic_per_launch(wagg["lef_epochs"] / max(1, wagg["launches"]))
        wave_line["roofline"] = {
            "bound": "hbm", "achieved": wach, "peak": peak, "unit": "GB/s", "frac": wach / peak,
            "traffic": wtraffic, "peak_source": f"{peak_kind} hbm_gbs", "kernel": "simulate_kernel",
            "traffic_note": "DRAM bytes per launch: ncu bytes per LEF-epoch of one launch that fills every "
                            "SM with 24 KiB cells as the concurrent wave does "
                            "(profiles/simulate_kernel_traffic.json) x this run's LEF-epochs per launch"}
        wave_line["batched_over_wave_cells_per_s"] = line["cells_per_s"] / wave_line["cells_per_s"]
    if args.windows > 0:
        line["batched_windows"] = run_windows(args, local, log)
    if args.surrogate:
        line["surrogate"] = run_surrogate(args, log)
    if not args.no_cpu_baseline:
        log("cpu baseline")
        threads = os.cpu_count() or 1
        s = cpu_sample_genome(cfg, tasks, args.cpu_seconds, threads)
        line["cpu_baseline"] = {"value": s["lef_epochs"] / s["seconds"], "unit": "LEF-epochs/s",
                                "cores": threads, "kind": "port", "sample": s["sample"]}
        # the CPU leg doubles as a parity check: its cells are the GPU's cells of the same ids
        gpu_cells = {}
        for k, st, _ in done:
            if k not in gpu_cells:
                gpu_cells[k] = st
        compared = equal = 0
        for k, cells in s["per_cell"].items():
            if k not in gpu_cells:
                continue
            for (i, ep, ct, dr, le) in cells:
                g = gpu_cells[k][i]
                compared += 1
                equal += int((g.epochs, g.contacts, g.rng_draws, g.lef_epochs) == (ep, ct, dr, le))
        line["parity"] = {"cells": compared, "equal": equal,
                          "fields": "epochs, contacts, rng_draws, lef_epochs of each CPU-oracle cell against "
                                    "the GPU cell of the same chromosome and cell id in the first timed step"}
    print(json.dumps(line), flush=True)
    for w in workers:
        w["eng"].close()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
