"""Surrogate inference from the command line: predict banded contact maps for sweep windows.

  python -m modlefork_gb300.surrogate_cli [--batch 256] [--reps 3] [--first 0] [--out maps.npy]

Loads the committed network (modlefork_gb300/data/surrogate_unet.npz), builds the inputs of
sweep windows first .. first + batch - 1 on the host (barrier tracks and parameters; no
simulation), runs one warm-up batch and `reps` timed batches on the GPU and prints maps/s.
With --out the last batch's maps ([batch, 4000, 600] float32, row-normalised log1p) are saved.
"""

import argparse
import json
import os

import numpy as np
import torch

from . import autotune, build
from . import surrogate as S
from . import sweep
from . import train_surrogate as T

WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "surrogate_unet.npz")


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--batch", type=int, default=256)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--first", type=int, default=0)
    ap.add_argument("--weights", default=WEIGHTS)
    ap.add_argument("--out", default=None)
    args = ap.parse_args(argv)
    build.build()
    autotune.apply_all()
    net = T.load_weights(args.weights)
    wins = [sweep.window(k, cells=1, density=1.0) for k in range(args.first, args.first + args.batch)]
    track = torch.from_numpy(np.stack([w[3] for w in wins])).to(net.dev)
    params = torch.from_numpy(np.stack([w[4] for w in wins])).to(net.dev)
    x = torch.empty(args.batch, net.length, S.IN_CH, dtype=torch.bfloat16, device=net.dev)
    S.ops.assemble_input(track, params, x)
    out = net.forward(x)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(args.reps):
        out = net.forward(x)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / max(1, args.reps)
    if args.out:
        np.save(args.out, out.cpu().numpy())
    print(json.dumps({"batch": args.batch, "ms_per_batch": ms, "maps_per_s": args.batch / (ms / 1e3),
                      "tflops": net.flops_per_map() * args.batch / (ms / 1e3) / 1e12}))


if __name__ == "__main__":
    main()
