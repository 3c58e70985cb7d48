"""Train and evaluate the surrogate end to end on one GPU.

  python -m modlefork_gb300.train_surrogate --train-sets 256 --held-sets 32 --out DIR

1. Sweep: parameter sets 0 .. train_sets - 1 on the batched simulator (sweep.py), targets on the
   device with their FP64 host check.
2. Train the U-Net with the project's own kernels (Adam, cosine schedule).
3. Held-out evaluation: fresh simulator runs of parameter sets the network never saw (indices
   from HELD_BASE on: new barrier tracks, parameters and cell seeds), each scored by Pearson r
   and relative L2 against the network's map, with the distance-decay baseline and the
   untrained network beside it; maps with r below the gate are answered by the simulator.
4. Throughput: surrogate maps/s at inference batch 256 (inputs in device memory, CUDA events)
   against the batched simulator's maps/s on the same windows.

Writes DIR/surrogate_unet.npz (weights: BF16 convolution weights, FP32 biases) and
DIR/surrogate_report.json.
"""

import argparse
import json
import os
import sys
import time

import numpy as np
import torch

from . import surrogate as S
from . import sweep

HELD_BASE = 1_000_000
GATE = 0.95


def log(msg):
    print(f"[surrogate {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def save_weights(net, path):
    """Convolution weights as BF16 bit patterns (what the tensor cores read), biases in FP32."""
    arrays = {"widths": np.array(net.widths), "mid": np.array(net.mid), "length": np.array(net.length)}
    for name in net.specs:
        arrays[f"w_{name}"] = net.wb[name].cpu().view(torch.int16).numpy()
        arrays[f"b_{name}"] = net.b32[name].cpu().numpy()
    np.savez_compressed(path, **arrays)


def load_weights(path, device=0):
    z = np.load(path)
    net = S.UNet(widths=tuple(int(w) for w in z["widths"]), mid=int(z["mid"]), length=int(z["length"]),
                 device=device)
    host = torch.zeros(net.p.numel(), dtype=torch.float32)
    for name, s in net.specs.items():
        w = torch.from_numpy(z[f"w_{name}"].copy()).view(torch.bfloat16).float().reshape(-1)
        wo = (net.w32[name].data_ptr() - net.p.data_ptr()) // 4
        bo = (net.b32[name].data_ptr() - net.p.data_ptr()) // 4
        host[wo:wo + s.wsize] = w
        host[bo:bo + s.cout] = torch.from_numpy(z[f"b_{name}"])
    net.load_state({"params": host.numpy()})
    return net


def concat_sets(sets, device):
    track = torch.cat([s["track"] for s in sets])
    params = torch.cat([s["params"] for s in sets])
    target = torch.cat([s["target"] for s in sets])
    return S.Dataset(track, params, target, device)


def inference_rate(net, x, batch=256, reps=5):
    """Surrogate maps/s at the given batch: inputs already on the device, CUDA events, one
    warm-up batch; returns (maps/s, ms per batch, achieved TFLOP/s)."""
    xb = x[torch.arange(batch, device=x.device) % x.shape[0]].contiguous()
    net.forward(xb)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(reps):
        net.forward(xb)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / reps
    return batch / (ms / 1e3), ms, net.flops_per_map() * batch / (ms / 1e3) / 1e12


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--train-sets", type=int, default=256)
    ap.add_argument("--held-sets", type=int, default=32)
    ap.add_argument("--cells", type=int, default=1024)
    ap.add_argument("--density", type=float, default=5.0)
    ap.add_argument("--held-density", type=float, default=10.0)
    ap.add_argument("--steps", type=int, default=3000)
    ap.add_argument("--batch", type=int, default=16)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--chunk", type=int, default=32)
    ap.add_argument("--out", default="surrogate_out")
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)
    from . import build

    build.build()
    from . import autotune

    autotune.apply_all()
    os.makedirs(args.out, exist_ok=True)
    dev = torch.device("cuda", 0)
    report = {"config": vars(args)}

    log(f"sweep: {args.train_sets} sets x {args.cells} cells, contact density {args.density}")
    sets, totals = sweep.generate(args.train_sets, chunk=args.chunk, cells=args.cells, density=args.density,
                                  log=log)
    report["sweep"] = {k: v for k, v in totals.items()}
    report["sweep"]["maps_per_s"] = totals["maps"] / (totals["ms"] / 1e3)
    data = concat_sets(sets, dev)
    del sets
    log(f"held-out: {args.held_sets} sets at contact density {args.held_density}")
    held_sets, held_totals = sweep.generate(HELD_BASE + args.held_sets, start=HELD_BASE, chunk=args.chunk,
                                            cells=args.cells, density=args.held_density, log=log)
    held = concat_sets(held_sets, dev)
    del held_sets
    report["held_sweep"] = dict(held_totals)
    report["held_sweep"]["maps_per_s"] = held_totals["maps"] / (held_totals["ms"] / 1e3)

    net = S.UNet(seed=args.seed, head_bias=data.diagonal_mean())
    report["nparams"] = net.nparams
    r0, l0 = S.evaluate(S.predict(net, held.x), held.target)
    log(f"train: {args.steps} steps, batch {args.batch}")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = S.train(net, data, steps=args.steps, batch=args.batch, lr=args.lr, warmup=min(200, args.steps // 10),
                     seed=args.seed, log=log, log_every=500)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    report["train"] = {"seconds": train_s, "steps": args.steps, "final_loss": float(losses[-50:].mean()),
                       "first_loss": float(losses[:10].mean()),
                       "tflops": net.flops_per_map(backward=True) * args.batch * args.steps / train_s / 1e12}
    pred = S.predict(net, held.x)
    r1, l1 = S.evaluate(pred, held.target)
    rt, lt = S.evaluate(S.predict(net, data.x[:64]), data.target[:64])
    base = S.baseline_prediction(data.diagonal_mean(), len(held), net.length, dev)
    rb, lb = S.evaluate(base, held.target)
    passed = r1 >= GATE
    report["held_out"] = {
        "maps": int(len(r1)), "pearson_r": r1.tolist(), "rel_l2": l1.tolist(),
        "mean_r": float(r1.mean()), "min_r": float(r1.min()), "mean_rel_l2": float(l1.mean()),
        "gate": GATE, "maps_passing_gate": int(passed.sum()),
        "untrained": {"mean_r": float(r0.mean()), "mean_rel_l2": float(l0.mean())},
        "distance_decay_baseline": {"mean_r": float(rb.mean()), "mean_rel_l2": float(lb.mean())},
        "train_maps_first_64": {"mean_r": float(rt.mean()), "mean_rel_l2": float(lt.mean())},
    }
    log(f"held-out: mean r {r1.mean():.4f} (min {r1.min():.4f}), rel-L2 {l1.mean():.4f}; "
        f"{int(passed.sum())}/{len(r1)} pass r >= {GATE}; baseline r {rb.mean():.4f} rel-L2 {lb.mean():.4f}")
    mps, ms, tf = inference_rate(net, held.x)
    sim_mps = report["held_sweep"]["maps_per_s"]
    # the gate's effective rate: maps that fail are simulated instead
    fail_frac = 1.0 - passed.mean()
    eff = 1.0 / (1.0 / mps + fail_frac / sim_mps)
    report["throughput"] = {"surrogate_maps_per_s": mps, "ms_per_batch_256": ms, "achieved_tflops": tf,
                            "simulator_maps_per_s": sim_mps, "surrogate_over_simulator": mps / sim_mps,
                            "gated_maps_per_s": eff, "gated_over_simulator": eff / sim_mps}
    log(f"surrogate {mps:.0f} maps/s ({tf:.1f} TFLOP/s), simulator {sim_mps:.2f} maps/s: {mps / sim_mps:.0f}x")
    save_weights(net, os.path.join(args.out, "surrogate_unet.npz"))
    with open(os.path.join(args.out, "surrogate_report.json"), "w") as f:
        json.dump(report, f, indent=1)
    print(json.dumps({k: report[k] for k in ("train", "throughput")} | {
        "held_out": {k: v for k, v in report["held_out"].items() if k not in ("pearson_r", "rel_l2")}}))


if __name__ == "__main__":
    main()
