"""The surrogate's FP64 oracle (oracle/surrogate_ref.py) against finite differences, and its
architecture against the GPU network's specification.  No GPU needed."""

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import surrogate_ref as ref  # noqa: E402


def _tiny(seed=0, widths=(64, 64), mid=64, length=16):
    rng = np.random.default_rng(seed)
    net = ref.RefUNet(widths, mid, length)
    params = {}
    for name, cout, taps, cin, act in net.specs:
        gain = 1.6 if act else 0.3
        params[name] = (rng.standard_normal((cout, taps, cin)) * gain / np.sqrt(taps * cin),
                        rng.standard_normal(cout) * 0.1)
    net.set_params(params)
    x = np.zeros((2, length, ref.IN_CH))
    x[:, :, :8] = rng.standard_normal((2, length, 8))
    t = rng.standard_normal((2, length, ref.NROWS)) * 0.5
    return net, x, t, rng


def test_oracle_gradients_match_finite_differences():
    net, x, t, rng = _tiny()
    _, grads = net.gradients(x, t)
    h = 1e-6
    for name, *_ in net.specs:
        w, b = net.params[name]
        dw, db = grads[name]
        for arr, garr in ((w, dw), (b, db)):
            flat, gflat = arr.reshape(-1), garr.reshape(-1)
            for k in rng.choice(flat.size, size=min(6, flat.size), replace=False):
                old = flat[k]
                flat[k] = old + h
                lp = net.loss(x, t)
                flat[k] = old - h
                lm = net.loss(x, t)
                flat[k] = old
                num = (lp - lm) / (2 * h)
                assert abs(num - gflat[k]) <= 1e-6 * max(1.0, abs(num)) + 1e-9, (name, k, num, gflat[k])


def test_oracle_architecture_equals_the_gpu_network():
    pytest.importorskip("torch")
    from modlefork_gb300 import surrogate

    widths, mid = (64, 128, 256, 384, 512), 512
    gpu = [(s.name, s.cout, s.taps, s.cin, s.act) for s in surrogate.conv_specs(widths, mid)]
    assert gpu == ref.RefUNet(widths, mid, 4000).specs
    n = sum(c * t * i + c for _, c, t, i, _ in gpu)
    assert 8e6 < n < 1e7  # about 8 M parameters


def test_shipped_per_layer_tuning_names_every_convolution():
    """The shipped table gives each forward convolution of the network a kernel form and depth,
    and apply_surrogate installs them where the network reads them (argument checks only: the
    setters run no device work)."""
    pytest.importorskip("torch")
    import json

    from modlefork_gb300 import autotune, surrogate, surrogate_ops

    table = json.load(open(autotune.DEFAULT_FILE))["devices"]
    names = [s.name for s in surrogate.conv_specs((64, 128, 256, 384, 512), 512)]
    saved = {bn: (surrogate_ops.conv_get_form(bn), surrogate_ops.conv_get_stages(bn)) for bn in (64, 128, 256)}
    try:
        for tuned in table.values():
            layers = tuned["surrogate"]["layers"]
            assert sorted(layers) == sorted(names)
            assert all(f in (0, 1, 2, 3) and s in (2, 3, 4) for f, s in layers.values())
            autotune.apply_surrogate(tuned)
            assert surrogate.LAYER_CFG == {k: tuple(v) for k, v in layers.items()}
            for bn, stages in tuned["surrogate"]["stages"].items():
                assert surrogate_ops.conv_get_stages(int(bn)) == stages
    finally:
        surrogate.LAYER_CFG.clear()
        for bn, (f, s) in saved.items():
            surrogate_ops.conv_set_form(bn, f)
            surrogate_ops.conv_set_stages(bn, s)
    assert {surrogate.tile_width(c) for c in (64, 128, 256, 384, 512, 640)} == {64, 128, 256}


def test_sweep_parameter_sets_are_reproducible_and_in_range():
    from modlefork_gb300 import sweep

    sets = [sweep.parameter_set(k) for k in range(200)]
    assert sets[17] == sweep.parameter_set(17)  # a pure function of the index (resumable)
    assert all(10 <= s["bar_density"] <= 60 and 5 <= s["lef_density"] <= 40 for s in sets)
    assert all(50e3 <= s["lifetime"] <= 500e3 and 1e3 <= s["speed"] <= 5e3 for s in sets)
    assert len({s["track_seed"] for s in sets}) == 200


def test_sweep_window_track_and_fp64_target():
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _harness import OracleHelpers
    from modlefork_gb300 import sweep

    cfg, chrom, bars, track, params = sweep.window(3, cells=8, density=1.0, api=OracleHelpers())
    assert chrom.size == sweep.WINDOW_BP and cfg.bin_size == sweep.BIN
    assert track.shape == (4, sweep.NCOLS) and params.shape == (4,)
    assert int(track[1].sum() + track[2].sum()) == len(bars)
    assert np.all(track[3] == track[3][0])
    band = np.zeros((sweep.NCOLS, sweep.NROWS), dtype=np.uint32)
    band[5, :3] = [4, 2, 0]
    t = sweep.target_fp64(band.reshape(-1))
    assert np.allclose(t[5, :3], np.log1p(np.array([4, 2, 0]) * sweep.NROWS / 6.0))
    assert not t[6].any()


def test_sweep_resumes_from_its_shards(tmp_path, monkeypatch):
    """An interrupted sweep re-run with the same output directory simulates only the chunks
    whose shard is missing, and load_shards returns every set in index order."""
    from modlefork_gb300 import sweep

    calls = []

    class FakeTensor:
        def __init__(self, a):
            self.a = a

        def cpu(self):
            return self

        def numpy(self):
            return self.a

    def fake(ks, seed, cells, density, device):
        calls.append(list(ks))
        n = len(ks)
        return {"track": FakeTensor(np.full((n, 4, 3), ks[0], np.float32)),
                "params": FakeTensor(np.asarray(ks, np.float32)[:, None].repeat(4, 1)),
                "target": FakeTensor(np.zeros((n, 2, 2), np.float32)), "fp64_max_rel_dev": 0.0, "ms": 1.0,
                "cells": n * cells, "lef_epochs": 0, "contacts": 0}

    monkeypatch.setattr(sweep, "simulate_sets", fake)
    out = str(tmp_path / "sweep")
    sweep.generate(10, out_dir=out, chunk=4, cells=2)
    assert calls == [[0, 1, 2, 3], [4, 5, 6, 7], [8, 9]]
    os.remove(os.path.join(out, "shard_000004.npz"))  # the run that lost a chunk
    calls.clear()
    _, totals = sweep.generate(10, out_dir=out, chunk=4, cells=2)
    assert calls == [[4, 5, 6, 7]] and totals["skipped"] == 6 and totals["maps"] == 4
    ks, track, params, target = sweep.load_shards(out)
    assert list(ks) == list(range(10)) and params[:, 0].tolist() == list(range(10))
