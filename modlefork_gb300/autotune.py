"""Autotuner of the GPU paths' launch settings, measured on the device it runs on.

  python -m modlefork_gb300.autotune [--out FILE] [--quick]

1. Batched simulator, per cell-size bucket (LEFs per cell): the engine's own workloads of that
   size (sweep windows; the genome workload's chromosomes grouped by LEF count, with their
   burn-in and contacts), one batched launch per candidate (shared-memory budget per cell,
   shared-memory carveout, cap of resident cells per SM), timed with CUDA events; the fastest in
   LEF-epochs/s becomes the bucket's entry of the table that mgpu_set_launch_table installs,
   unless it beats the engine's default (16 KiB, 60 %) by less than 5 %, the trials' spread, in
   which case the default stays.  The settings only move per-LEF arrays between
   shared memory and global slots, so every candidate simulates the same cells.
2. Surrogate convolutions: the kernel form (one CTA per tile or persistent, outputs per thread or
   staged through shared memory and TMA stores) and pipeline depth (2-4 stages) per N tile width
   of msur_conv_forward, then per forward layer of the network, by coordinate descent on the
   network's inference time at batch 256.

The result is a JSON file keyed by the device's name and SM count; ``load_table`` and
``apply_all`` read it back (engine contexts and the surrogate library take it from there).  The
tuned table measured on a GB300 ships as modlefork_gb300/data/tuning_gb300.json.
"""

import argparse
import json
import os
import sys
import time

import numpy as np

DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data")
DEFAULT_FILE = os.path.join(DATA, "tuning_gb300.json")

# (bucket upper bound on LEFs per cell, chromosome length of its trial workload in bp at 20 LEFs/Mbp)
BUCKETS = [(512, 16_000_000), (2048, 64_000_000), (4096, 160_000_000), (1 << 40, 250_000_000)]
FULL = 1 << 30  # a budget above the device limit: as much shared memory per cell as a block may have
DEFAULT = (16384, 60, 0)  # the engine's setting of large batches without a table
CANDIDATES = [DEFAULT, (FULL, 0, 0), (12288, 60, 0), (20480, 60, 0), (24576, 60, 0), (24576, 80, 0),
              (32768, 80, 0)]
QUICK_CANDIDATES = [DEFAULT, (FULL, 0, 0), (24576, 70, 0), (12288, 80, 0), (32768, 80, 0)]
MARGIN = 1.05  # a candidate replaces the default only when it is this much faster


def log(msg):
    print(f"[autotune {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def device_key():
    import torch

    p = torch.cuda.get_device_properties(0)
    return f"{p.name}|{p.multi_processor_count}"


def bucket_workloads():
    """The workloads each bucket is tuned on, the engine's own: sweep windows for small cells, and
    the genome workload's chromosomes grouped by LEF count (with their burn-in and contacts, as
    the batched genome launch runs them).  Yields (max_lefs, description, [(cfg, chrom, barriers,
    cells)])."""
    from . import engine, genome, sweep

    wins = [sweep.window(k, cells=1024, density=5.0) for k in range(12)]
    yield 512, "sweep windows 0-11 (20 Mbp, 1024 cells, contact density 5)", [(w[0], w[1], w[2], 1024) for w in wins]
    for lo, hi, cells in ((0, 2048, 1536), (2048, 4096, 1024), (4096, 1 << 40, 1024)):
        cfg, gen = genome.genome_24chr(seed=11, num_cells=cells)  # per-cell targets split over `cells`
        nl = {c.name: engine.num_lefs(cfg, c.simulated_size) for c, _ in gen}
        chroms = [(cfg, c, b, cells) for c, b in gen if lo < nl[c.name] <= hi]
        yield hi, (f"genome chromosomes with {lo + 1}-{min(hi, 99999)} LEFs ({len(chroms)}) x {cells} cells, "
                   "contact density 1"), chroms


def tune_simulator(candidates, device=0):
    """One batched launch of each bucket's workload per candidate, timed with CUDA events."""
    from . import engine, genome

    table, trials = [], []
    for max_lefs, what, items in bucket_workloads():
        best, default_rate = None, 0.0
        with engine.Engine(genome.genome_config(), device) as eng:
            tasks, bands = [], {}
            for cfg, chrom, bars, cells in items:
                cid = eng.upload_chrom(chrom, bars)
                eng.set_chrom_config(cid, cfg)
                n = engine.num_lefs(cfg, chrom.simulated_size)
                tg, te = engine.task_targets(cfg, chrom.simulated_size, n, cells)
                bands[cid] = None
                tasks += [(cid, engine.cell_seed(chrom.name, chrom.size, cfg.seed, i), int(tg[i]), te, n)
                          for i in range(cells)]
            import torch

            dbands = {}
            for (cfg, chrom, _, _), cid in zip(items, sorted(bands)):
                dbands[cid] = torch.zeros(int(np.prod(engine.band_shape(cfg, chrom.simulated_size))),
                                          dtype=torch.int32, device=f"cuda:{device}")
            ptrs = {c: t.data_ptr() for c, t in dbands.items()}
            log(f"bucket <= {max_lefs} LEFs: {what}, {len(tasks)} cells")
            for budget, carveout, cap in candidates:
                eng.set_debug_flags(((carveout & 0xFF) << 8) | ((cap & 0xFF) << 16), budget)
                try:
                    _, st = eng.simulate_batch(tasks, ptrs)
                except engine.EngineError as e:  # a budget below a cell's fixed shared memory
                    log(f"  budget {budget // 1024} KiB rejected ({e})")
                    continue
                ms = eng.last_kernel_ms()
                rate = sum(x.lef_epochs for x in st) / (ms / 1e3)
                trials.append({"bucket_max_lefs": max_lefs, "workload": what, "smem_budget": budget,
                               "carveout_pct": carveout, "max_cells_per_sm": cap, "ms": ms, "lef_epochs_per_s": rate})
                log(f"  budget {min(budget, 1 << 20) // 1024} KiB, carveout {carveout} %, cap {cap}: "
                    f"{rate:.3e} LEF-epochs/s")
                if (budget, carveout, cap) == DEFAULT:
                    default_rate = rate
                if best is None or rate > best[0]:
                    best = (rate, budget, carveout, cap)
        if best[0] < MARGIN * default_rate:  # within the measurement's spread: keep the default
            best = (default_rate,) + DEFAULT
        table.append({"max_lefs": max_lefs, "smem_budget": best[1], "carveout_pct": best[2],
                      "max_cells_per_sm": best[3], "lef_epochs_per_s": best[0],
                      "default_lef_epochs_per_s": default_rate, "workload": what})
    return table, trials


def tune_surrogate(batch=256, reps=5):
    import torch

    from . import surrogate as S
    from . import surrogate_ops as ops

    S.LAYER_CFG.clear()  # start from the per-width settings alone
    net = S.UNet(seed=0)
    x = torch.zeros(batch, net.length, S.IN_CH, dtype=torch.bfloat16, device=net.dev)
    x[:, :, :8].normal_()

    def timed():
        net.forward(x)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record()
        for _ in range(reps):
            net.forward(x)
        ev1.record()
        torch.cuda.synchronize()
        return ev0.elapsed_time(ev1) / reps

    choice = {bn: (ops.conv_get_form(bn), ops.conv_get_stages(bn)) for bn in (64, 128, 256)}
    trials = []
    base = timed()
    for _ in range(2):  # two rounds of coordinate descent over (kernel form, stages) per N tile
        for bn in (256, 128, 64):
            times = {}
            for form in (0, 1, 2, 3):
                for stages in (2, 3, 4):
                    ops.conv_set_form(bn, form)
                    ops.conv_set_stages(bn, stages)
                    times[(form, stages)] = timed()
                    trials.append({"bn": bn, "form": form, "stages": stages,
                                   "others": {str(k): list(v) for k, v in choice.items()},
                                   "ms_per_batch": times[(form, stages)]})
            choice[bn] = min(times, key=times.get)
            ops.conv_set_form(bn, choice[bn][0])
            ops.conv_set_stages(bn, choice[bn][1])
            log(f"conv N tile {bn}: {times} -> {choice[bn]}")
    per_width = timed()
    # then per forward layer (the network sets the layer's choice before its call), starting
    # from the per-width choices, one round of coordinate descent over the layers
    layers = {}
    for name, spec in net.specs.items():
        layers[name] = choice[S.tile_width(spec.cout)]
    S.LAYER_CFG.clear()
    S.LAYER_CFG.update(layers)
    cur = timed()
    for name in net.specs:
        times = {}
        for form in (0, 1, 2, 3):
            for stages in (2, 3, 4):
                S.LAYER_CFG[name] = (form, stages)
                times[(form, stages)] = timed()
        best_cfg = min(times, key=times.get)
        S.LAYER_CFG[name] = best_cfg
        trials.append({"layer": name, "times": {f"{k[0]},{k[1]}": v for k, v in times.items()}})
        log(f"layer {name}: -> {best_cfg} ({times[best_cfg]:.3f} ms)")
    best = timed()
    out = {"stages": {str(k): v[1] for k, v in choice.items()},
           "form": {str(k): v[0] for k, v in choice.items()},
           "layers": {k: list(v) for k, v in S.LAYER_CFG.items()}, "ms_per_batch_default": base,
           "ms_per_batch_per_width": per_width, "ms_per_batch_tuned": best, "batch": batch}
    S.LAYER_CFG.clear()
    return out, trials


def load_table(path=DEFAULT_FILE):
    """The tuned settings for the current device, or None when the file has none for it."""
    if not os.path.exists(path):
        return None
    try:
        d = json.load(open(path))
        return d.get("devices", {}).get(device_key())
    except (OSError, ValueError):
        return None


def apply_engine(eng, tuned):
    """Install the simulator table of `tuned` (load_table's result) on an engine context."""
    if tuned and tuned.get("simulator"):
        eng.set_launch_table([(e["max_lefs"], e["smem_budget"], e["carveout_pct"], e["max_cells_per_sm"])
                              for e in tuned["simulator"]])


def apply_all(eng=None, path=DEFAULT_FILE):
    """Apply the shipped tuning for this device (if it has any) to an engine and the surrogate
    library; returns the settings applied or None."""
    tuned = load_table(path)
    if tuned:
        if eng is not None:
            apply_engine(eng, tuned)
        apply_surrogate(tuned)
    return tuned


def apply_surrogate(tuned):
    """Set the convolution pipeline depths of `tuned` in the surrogate library."""
    from . import surrogate_ops as ops

    if tuned and tuned.get("surrogate"):
        for bn, stages in tuned["surrogate"]["stages"].items():
            ops.conv_set_stages(int(bn), int(stages))
        if "form" in tuned["surrogate"]:
            for bn, form in tuned["surrogate"]["form"].items():
                ops.conv_set_form(int(bn), int(form))
        else:  # tables written before the staged epilogue: bit 0 alone
            for bn, on in tuned["surrogate"].get("persistent", {}).items():
                ops.conv_set_form(int(bn), int(on))
        from . import surrogate as S

        S.LAYER_CFG.clear()
        S.LAYER_CFG.update({k: (int(v[0]), int(v[1])) for k, v in tuned["surrogate"].get("layers", {}).items()})


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--out", default="tuning.json")
    ap.add_argument("--quick", action="store_true", help="five simulator candidates instead of nineteen")
    ap.add_argument("--only", choices=["simulator", "surrogate"], default=None,
                    help="tune one part and keep the other's entry from --out")
    args = ap.parse_args(argv)
    from . import build

    build.build()
    out = {"devices": {}}
    if os.path.exists(args.out):
        out = json.load(open(args.out))
    entry = dict(out.setdefault("devices", {}).get(device_key(), {}))
    entry.setdefault("trials", {})
    if args.only != "surrogate":
        cands = QUICK_CANDIDATES if args.quick else CANDIDATES
        entry["simulator"], entry["trials"]["simulator"] = tune_simulator(cands)
    if args.only != "simulator":
        entry["surrogate"], entry["trials"]["surrogate"] = tune_surrogate()
    entry["measured"] = time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())
    entry["command"] = "python -m modlefork_gb300.autotune" + (" --quick" if args.quick else "")
    out["devices"][device_key()] = entry
    sim_table, sur = entry.get("simulator"), entry.get("surrogate")
    with open(args.out, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({"device": device_key(), "simulator": sim_table, "surrogate": sur}))


if __name__ == "__main__":
    main()
