"""The surrogate network on the GPU: forward and backward against the FP64 oracle
(oracle/surrogate_ref.py, itself checked by finite differences), training that lowers the loss,
and the gain of the trained network over the method without it on simulated maps.

Tolerances: the GPU keeps activations and gradients in BF16 (FP32 accumulation), the oracle in
FP64; per tensor the relative L2 error must stay below 5 % and the cosine similarity above 0.995.
"""

import os
import sys

import numpy as np
import pytest
import torch

from modlefork_gb300 import surrogate as S
from modlefork_gb300 import surrogate_ops as ops

sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
import surrogate_ref as ref  # noqa: E402

pytestmark = pytest.mark.gpu


def _bf16_round(a):
    return torch.from_numpy(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).float().numpy().astype(np.float64)


def _inputs(rng, B, L):
    x = np.zeros((B, L, S.IN_CH), dtype=np.float32)
    x[:, :, :8] = rng.standard_normal((B, L, 8))
    return x


def _ref_for(net):
    r = ref.RefUNet(net.widths, net.mid, net.length)
    r.set_params({k: (_bf16_round(w), b.astype(np.float64)) for k, (w, b) in net.params_dict().items()})
    return r


@pytest.fixture(autouse=True)
def _no_timeouts():
    yield
    torch.cuda.synchronize()
    assert ops.take_error() == 0


def _agree(got, want, name):
    got, want = got.ravel(), want.ravel()
    rel = np.linalg.norm(got - want) / (np.linalg.norm(want) + 1e-30)
    cos = got @ want / (np.linalg.norm(got) * np.linalg.norm(want) + 1e-30)
    assert rel < 0.05 and cos > 0.995, f"{name}: relative L2 {rel:.4f}, cosine {cos:.5f}"


def test_gradients_match_the_fp64_oracle():
    rng = np.random.default_rng(1)
    B, L = 2, 256
    net = S.UNet(widths=(64, 128), mid=128, length=L, seed=3,
                 head_bias=rng.standard_normal(S.NROWS) * 0.1)
    x = _inputs(rng, B, L)
    t = (rng.standard_normal((B, L, S.NROWS)) * 0.5).astype(np.float32)
    xg = torch.from_numpy(x).to(net.dev, torch.bfloat16)
    tg = torch.from_numpy(t).to(net.dev)
    loss = net.loss_and_grad(xg, tg).item()
    torch.cuda.synchronize()
    r = _ref_for(net)
    rloss, rgrads = r.gradients(xg.float().cpu().numpy().astype(np.float64), t.astype(np.float64))
    assert abs(loss - rloss) < 0.01 * rloss
    for name in net.specs:
        dw = net.gw[name].cpu().numpy() / S.LOSS_SCALE
        db = net.gb[name].cpu().numpy() / S.LOSS_SCALE
        want_w, want_b = rgrads[name]
        _agree(dw, want_w, f"{name} weights")
        _agree(db, want_b, f"{name} bias")


def test_full_size_forward_matches_the_fp64_oracle():
    rng = np.random.default_rng(2)
    net = S.UNet(seed=5, head_bias=np.linspace(3, 0, S.NROWS))
    assert 8e6 < net.nparams < 1e7
    x = _inputs(rng, 1, net.length)
    xg = torch.from_numpy(x).to(net.dev, torch.bfloat16)
    out = net.forward(xg).cpu().numpy()
    want = _ref_for(net).forward(xg.float().cpu().numpy().astype(np.float64))
    _agree(out, want, "network output")


def test_fused_concatenation_equals_the_upcat_path():
    """Inference with the concatenation buffers filled by the producing convolutions (no upcat
    step) gives the maps of the unfused forward bit for bit, in the default kernel forms and in
    the shipped table's."""
    from modlefork_gb300 import autotune

    rng = np.random.default_rng(4)
    net = S.UNet(seed=9, head_bias=np.linspace(2, 0, S.NROWS))
    x = torch.from_numpy(_inputs(rng, 3, net.length)).to(net.dev, torch.bfloat16)
    saved = {bn: (ops.conv_get_form(bn), ops.conv_get_stages(bn)) for bn in (64, 128, 256)}
    try:
        for table in (None, autotune.load_table()):
            if table:
                autotune.apply_surrogate(table)
            assert net.fusable()
            fused = net.forward(x).clone()
            plain = net.forward(x, fuse=False).clone()
            torch.cuda.synchronize()
            assert torch.equal(fused, plain)
    finally:
        S.LAYER_CFG.clear()
        for bn, (f, st) in saved.items():
            ops.conv_set_form(bn, f)
            ops.conv_set_stages(bn, st)


def test_host_prediction_path_equals_device_prediction():
    """predict_host (host inputs, host outputs, batches alternating between two device slots with
    the copies back on a second stream, a short last batch) gives the maps predict gives from
    the same inputs assembled on the device, bit for bit."""
    rng = np.random.default_rng(8)
    net = S.UNet(seed=3, head_bias=np.linspace(2, 0, S.NROWS))
    N = 5
    track = rng.random((N, 4, net.length)).astype(np.float32)
    params = rng.random((N, 4)).astype(np.float32)
    data = S.Dataset(track, params, np.zeros((N, net.length, S.NROWS), np.float32), net.dev)
    want = S.predict(net, data.x, batch=2).cpu()
    out = torch.full((N, net.length, S.NROWS), 7.0).pin_memory()
    S.predict_host(net, torch.from_numpy(track).pin_memory(), torch.from_numpy(params).pin_memory(), out, batch=2)
    torch.cuda.synchronize()
    assert torch.equal(out, want)


def test_training_lowers_the_loss():
    rng = np.random.default_rng(3)
    N, L = 12, 256
    track = rng.random((N, 4, L)).astype(np.float32)
    params = rng.random((N, 4)).astype(np.float32)
    # a target that depends on the track smoothly: a distance decay modulated by the input
    d = np.arange(S.NROWS)
    target = (np.exp(-d / 50.0)[None, None, :] * (1 + track[:, 0, :, None]) + params[:, None, :1]).astype(
        np.float32)
    assert target.shape == (N, L, S.NROWS)
    data = S.Dataset(track, params, target)
    net = S.UNet(widths=(64, 128), mid=128, length=L, seed=1, head_bias=data.diagonal_mean())
    losses = S.train(net, data, steps=150, batch=4, lr=2e-3, warmup=10)
    assert np.isfinite(losses).all()
    assert losses[-20:].mean() < 0.5 * losses[:5].mean()


def test_trained_network_beats_the_method_without_it():
    """Gain test on simulated maps: sweep windows simulated on the GPU, a network trained on 28
    of them, and scored on 8 held-out windows against (a) the distance-decay baseline (the
    training maps' mean per diagonal, what one predicts without the network) and (b) the same
    network untrained."""
    from modlefork_gb300 import sweep

    train_sets = sweep.simulate_sets(list(range(28)), cells=128, density=5.0)
    test_sets = sweep.simulate_sets(list(range(1000, 1008)), cells=128, density=5.0)
    assert train_sets["fp64_max_rel_dev"] < 1e-6 and test_sets["fp64_max_rel_dev"] < 1e-6
    data = S.Dataset(train_sets["track"], train_sets["params"], train_sets["target"])
    held = S.Dataset(test_sets["track"], test_sets["params"], test_sets["target"])
    net = S.UNet(seed=7, head_bias=data.diagonal_mean())
    r0, l0 = S.evaluate(S.predict(net, held.x), held.target)
    S.train(net, data, steps=400, batch=8, lr=1e-3, warmup=40)
    r1, l1 = S.evaluate(S.predict(net, held.x), held.target)
    base = S.baseline_prediction(data.diagonal_mean(), len(held), net.length, net.dev)
    rb, lb = S.evaluate(base, held.target)
    print(f"held-out mean r / relL2: trained {r1.mean():.4f} / {l1.mean():.4f}, untrained {r0.mean():.4f} / "
          f"{l0.mean():.4f}, distance decay {rb.mean():.4f} / {lb.mean():.4f}")
    assert l1.mean() < lb.mean() and r1.mean() > rb.mean()
    assert l1.mean() < l0.mean()
