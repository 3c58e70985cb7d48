"""The surrogate's kernels against plain FP32/FP64 references of the same ops.

The tensor-core convolutions (tcgen05.mma on BF16 operands staged by TMA, FP32 accumulators)
are compared with an FP64 evaluation of the same convolution on the same BF16-rounded inputs:
the FP32 outputs must agree to 2e-5 of the outputs' scale (accumulation order only), the BF16
outputs to BF16 rounding (2^-8 relative) on top.  Shapes cover every tile width (64, 128, 256),
several output-channel tiles, a ragged last position tile, batches, one- and three-tap
convolutions, the masked head (600 of 640 channels), the SiLU epilogue and the gated data
gradient.  The memory-bound kernels are checked against numpy.
"""

import numpy as np
import pytest
import torch

from modlefork_gb300 import surrogate_ops as ops

pytestmark = pytest.mark.gpu
DEV = "cuda"


def _bf16(a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).to(torch.bfloat16)


def _np(t):
    return t.detach().float().cpu().numpy().astype(np.float64)


def _conv_ref(x, w, bias=None):
    """y[b, l, n] = sum_t sum_c x[b, l + t - pad, c] w[n, t, c] (FP64)."""
    B, L, _ = x.shape
    N, taps, _ = w.shape
    pad = (taps - 1) // 2
    xp = np.zeros((B, L + 2 * pad, x.shape[2]))
    xp[:, pad:pad + L] = x
    y = np.zeros((B, L, N))
    for t in range(taps):
        y += np.einsum("blc,nc->bln", xp[:, t:t + L], w[:, t])
    if bias is not None:
        y += bias
    return y


def _silu(z):
    return z / (1 + np.exp(-z))


def _dsilu(z):
    s = 1 / (1 + np.exp(-z))
    return s * (1 + z * (1 - s))


def _close(got, ref, rel_bf16):
    scale = np.sqrt(np.mean(ref ** 2)) + 1e-30
    tol = (2.0 ** -8 if rel_bf16 else 0.0) * np.abs(ref) + 2e-5 * scale
    bad = np.abs(got - ref) > tol
    assert not bad.any(), f"{bad.sum()} of {bad.size} differ; max err {np.abs(got - ref).max():.3e} scale {scale:.3e}"


@pytest.fixture(autouse=True)
def _no_timeouts():
    torch.cuda.synchronize()
    yield
    torch.cuda.synchronize()
    assert ops.take_error() == 0, "a tensor-core kernel's barrier wait ran out"


CONV_SHAPES = [
    # (B, L, Cin, Cout, taps)
    (2, 300, 64, 64, 3),
    (3, 257, 128, 256, 3),
    (2, 130, 192, 384, 3),
    (1, 128, 512, 512, 3),
    (2, 70, 64, 128, 1),
]


@pytest.fixture(params=[0, 1, 2, 3], ids=["tile", "persistent", "tile-staged", "persistent-staged"])
def conv_form(request):
    """Every kernel form of msur_conv_forward (per-thread or staged epilogue, one CTA per tile or
    persistent) for all N tile widths, restored afterwards."""
    saved = {bn: ops.conv_get_form(bn) for bn in (64, 128, 256)}
    for bn in saved:
        ops.conv_set_form(bn, request.param)
    yield request.param
    for bn, f in saved.items():
        ops.conv_set_form(bn, f)


@pytest.mark.parametrize("B,L,Cin,Cout,taps", CONV_SHAPES)
def test_conv_forward_matches_fp64(B, L, Cin, Cout, taps, conv_form):
    rng = np.random.default_rng(B * 1000 + L + Cin + Cout)
    xb = _bf16(rng.standard_normal((B, L, Cin)))
    wb = _bf16(rng.standard_normal((Cout, taps, Cin)) / np.sqrt(taps * Cin))
    bias = rng.standard_normal(Cout).astype(np.float32) * 0.1
    x, w = xb.to(DEV), wb.to(DEV)
    db = torch.from_numpy(bias).to(DEV)
    pre = torch.empty(B, L, Cout, dtype=torch.bfloat16, device=DEV)
    post = torch.empty_like(pre)
    f32 = torch.empty(B, L, Cout, dtype=torch.float32, device=DEV)
    ops.conv_forward(x, w, bias=db, act=ops.ACT_SILU, out_pre=pre, out_post=post, out_f32=f32)
    torch.cuda.synchronize()
    ref = _conv_ref(_np(xb), _np(wb), bias.astype(np.float64))
    _close(_np(f32), ref, False)
    _close(_np(pre), ref, True)
    _close(_np(post), _silu(ref), True)


def test_conv_forward_head_masks_padded_channels(conv_form):
    """The output head: one tap, 640 weight rows of which 600 are written, FP32, row stride 600;
    the buffer's guard value must survive beyond the 600 columns of the last row."""
    rng = np.random.default_rng(11)
    B, L, Cin, N, NV = 2, 260, 64, 640, 600
    xb = _bf16(rng.standard_normal((B, L, Cin)))
    wb = _bf16(rng.standard_normal((N, 1, Cin)) / 8)
    bias = (rng.standard_normal(N) * 0.1).astype(np.float32)
    buf = torch.full((B * L * NV + 64,), 7.0, dtype=torch.float32, device=DEV)
    out = buf[:B * L * NV].view(B, L, NV)
    ops.conv_forward(xb.to(DEV), wb.to(DEV), bias=torch.from_numpy(bias).to(DEV), out_f32=out, n_valid=NV,
                     out_stride=NV)
    torch.cuda.synchronize()
    ref = _conv_ref(_np(xb), _np(wb), bias.astype(np.float64))[:, :, :NV]
    _close(_np(out), ref, False)
    assert torch.all(buf[B * L * NV:] == 7.0)


@pytest.mark.parametrize("form", [2, 3], ids=["tile-staged", "persistent-staged"])
@pytest.mark.parametrize("Cout,C1", [(64, 128), (128, 64), (256, 128)])
def test_fused_copies_equal_the_post_output(form, Cout, C1):
    """msur_conv_forward_fused: the post-activation value written as usual, into the skip half of
    a concatenation buffer, upsampled by two into the other half of another one and average-pooled
    by two, bit for bit what conv_forward writes plus the copies and the pooling made separately;
    refused without the staged form.  L = 150 leaves a ragged last row tile (and a pooled one)."""
    rng = np.random.default_rng(Cout + C1 + form)
    B, L, Cin = 2, 150, 128
    x = _bf16(rng.standard_normal((B, L, Cin))).to(DEV)
    w = _bf16(rng.standard_normal((Cout, 3, Cin)) / 16).to(DEV)
    bias = torch.from_numpy(rng.standard_normal(Cout).astype(np.float32)).to(DEV)
    bn = 64 if Cout <= 64 else (256 if Cout % 256 == 0 else 128)
    saved = ops.conv_get_form(bn)
    try:
        ops.conv_set_form(bn, form)
        want = torch.empty(B, L, Cout, dtype=torch.bfloat16, device=DEV)
        ops.conv_forward(x, w, bias=bias, act=ops.ACT_SILU, out_post=want)
        post = torch.full((B, L, Cout), 3.0, dtype=torch.bfloat16, device=DEV)
        cat = torch.full((B, L, C1 + Cout), 5.0, dtype=torch.bfloat16, device=DEV)
        up = torch.full((B, 2 * L, Cout + C1), 5.0, dtype=torch.bfloat16, device=DEV)
        pooled = torch.full((B, L // 2, Cout), 5.0, dtype=torch.bfloat16, device=DEV)
        want_pool = torch.empty_like(pooled)
        ops.pool2(want, want_pool)
        ops.conv_forward_fused(x, w, bias=bias, act=ops.ACT_SILU, out_post=post, skip=cat[:, :, C1:],
                               dup=up[:, :, :Cout], pool=pooled)
        torch.cuda.synchronize()
        assert torch.equal(post, want)
        assert torch.equal(pooled, want_pool)
        assert torch.equal(cat[:, :, C1:], want) and torch.all(cat[:, :, :C1] == 5.0)
        assert torch.equal(up[:, 0::2, :Cout], want) and torch.equal(up[:, 1::2, :Cout], want)
        assert torch.all(up[:, :, Cout:] == 5.0)
        ops.conv_set_form(bn, form & 1)
        with pytest.raises(ops.SurrogateKernelError):
            ops.conv_forward_fused(x, w, bias=bias, act=ops.ACT_SILU, skip=cat[:, :, C1:])
    finally:
        ops.conv_set_form(bn, saved)


def test_data_gradient_through_silu_gate(conv_form):
    """dx = conv(dz, transpose(w)) * silu'(z_prev): the gradient of a SiLU-activated input."""
    rng = np.random.default_rng(12)
    B, L, Cin, Cout = 2, 190, 192, 256
    wb = _bf16(rng.standard_normal((Cout, 3, Cin)) / np.sqrt(3 * Cin))
    dzb = _bf16(rng.standard_normal((B, L, Cout)))
    zb = _bf16(rng.standard_normal((B, L, Cin)))
    w, dz, z = wb.to(DEV), dzb.to(DEV), zb.to(DEV)
    wt = torch.empty(Cin, 3, Cout, dtype=torch.bfloat16, device=DEV)
    ops.weight_transpose(w, wt)
    dx = torch.empty(B, L, Cin, dtype=torch.bfloat16, device=DEV)
    dxf = torch.empty(B, L, Cin, dtype=torch.float32, device=DEV)
    ops.conv_forward(dz, wt, out_post=dx, out_f32=dxf, gate=z)
    torch.cuda.synchronize()
    assert np.array_equal(_np(wt), np.transpose(_np(wb)[:, ::-1, :], (2, 1, 0)))
    # reference: the adjoint of the forward convolution, then the SiLU derivative
    wn, dzn = _np(wb), _np(dzb)
    ref = np.zeros((B, L, Cin))
    dzp = np.zeros((B, L + 2, Cout))
    dzp[:, 1:1 + L] = dzn
    for t in range(3):  # x[l + t - 1] feeds y[l]  =>  dx[j] += dz[j - t + 1] w[t]
        ref += np.einsum("bln,nc->blc", dzp[:, 2 - t:2 - t + L], wn[:, t])
    ref *= _dsilu(_np(zb))
    _close(_np(dxf), ref, True)  # the gate is applied to BF16-rounded z: relative BF16 tolerance
    _close(_np(dx), ref, True)


WGRAD_SHAPES = [
    # (B, L, Cin, Cout, taps)
    (2, 300, 64, 64, 3),
    (3, 257, 256, 128, 3),
    (2, 190, 192, 384, 3),
    (2, 130, 64, 640, 1),
]


@pytest.mark.parametrize("B,L,Cin,Cout,taps", WGRAD_SHAPES)
def test_weight_gradient_matches_fp64(B, L, Cin, Cout, taps):
    rng = np.random.default_rng(B + L + Cin + Cout + taps)
    xb = _bf16(rng.standard_normal((B, L, Cin)))
    dzb = _bf16(rng.standard_normal((B, L, Cout)))
    dw = torch.full((Cout, taps, Cin), 0.5, dtype=torch.float32, device=DEV)  # accumulated into
    ops.conv_wgrad(xb.to(DEV), dzb.to(DEV), dw)
    torch.cuda.synchronize()
    x, dz = _np(xb), _np(dzb)
    pad = (taps - 1) // 2
    xp = np.zeros((B, L + 2 * pad, Cin))
    xp[:, pad:pad + L] = x
    ref = np.stack([np.einsum("bln,blc->nc", dz, xp[:, t:t + L]) for t in range(taps)], axis=1) + 0.5
    _close(_np(dw), ref, False)


def test_weight_gradient_split_counts_agree():
    rng = np.random.default_rng(21)
    B, L, Cin, Cout = 4, 500, 128, 256
    x = _bf16(rng.standard_normal((B, L, Cin))).to(DEV)
    dz = _bf16(rng.standard_normal((B, L, Cout))).to(DEV)
    outs = []
    for splits in (1, 3, 32):
        dw = torch.zeros(Cout, 3, Cin, dtype=torch.float32, device=DEV)
        ops.conv_wgrad(x, dz, dw, splits=splits)
        outs.append(_np(dw))
    torch.cuda.synchronize()
    for o in outs[1:]:
        _close(o, outs[0], False)


# ---- memory-bound kernels ------------------------------------------------------------------

def test_pool_upcat_and_their_gradients():
    rng = np.random.default_rng(31)
    B, L, C1, C2 = 2, 100, 64, 128
    x = _bf16(rng.standard_normal((B, L, C2)))
    y = torch.empty(B, L // 2, C2, dtype=torch.bfloat16, device=DEV)
    ops.pool2(x.to(DEV), y)
    xn = _np(x)
    _close(_np(y), 0.5 * (xn[:, 0::2] + xn[:, 1::2]), True)
    h = _bf16(rng.standard_normal((B, L // 2, C1)))
    cat = torch.empty(B, L, C1 + C2, dtype=torch.bfloat16, device=DEV)
    ops.upcat(h.to(DEV), x.to(DEV), cat)
    cn = _np(cat)
    assert np.array_equal(cn[:, :, :C1], np.repeat(_np(h), 2, axis=1)) and np.array_equal(cn[:, :, C1:], xn)
    dcat = _bf16(rng.standard_normal((B, L, C1 + C2)))
    zh = _bf16(rng.standard_normal((B, L // 2, C1)))
    dzh = torch.empty(B, L // 2, C1, dtype=torch.bfloat16, device=DEV)
    ops.upcat_bwd(dcat.to(DEV), zh.to(DEV), dzh)
    dc = _np(dcat)
    _close(_np(dzh), (dc[:, 0::2, :C1] + dc[:, 1::2, :C1]) * _dsilu(_np(zh)), True)
    # skip gradient: the pooled path and the concatenation's skip half meet at a SiLU output
    dpool = _bf16(rng.standard_normal((B, L // 2, C2)))
    z = _bf16(rng.standard_normal((B, L, C2)))
    dz = torch.empty(B, L, C2, dtype=torch.bfloat16, device=DEV)
    ops.skip_grad(z.to(DEV), dz, dpool=dpool.to(DEV), dcat=dcat.to(DEV), cat_off=C1)
    ref = (0.5 * np.repeat(_np(dpool), 2, axis=1) + dc[:, :, C1:]) * _dsilu(_np(z))
    _close(_np(dz), ref, True)


def test_bias_grad_mse_adam_transpose_and_input():
    rng = np.random.default_rng(41)
    dz = _bf16(rng.standard_normal((3, 77, 192)))
    db = torch.ones(192, dtype=torch.float32, device=DEV)
    ops.bias_grad(dz.to(DEV), db)
    _close(_np(db), 1 + _np(dz).reshape(-1, 192).sum(0), False)
    # MSE over 600 of 640 channels, gradient scale
    pred = torch.from_numpy(rng.standard_normal((2, 50, 600)).astype(np.float32)).to(DEV)
    tgt = torch.from_numpy(rng.standard_normal((2, 50, 600)).astype(np.float32)).to(DEV)
    loss = torch.zeros(1, dtype=torch.float64, device=DEV)
    dp = torch.full((2, 50, 640), 9.0, dtype=torch.bfloat16, device=DEV)
    ops.mse(pred, tgt, loss, dp=dp, scale=0.5)
    d = _np(pred) - _np(tgt)
    assert abs(loss.item() - (d ** 2).sum()) < 1e-6 * (d ** 2).sum()
    dpn = _np(dp)
    _close(dpn[:, :, :600], 0.5 * d, True)
    assert not dpn[:, :, 600:].any()
    # Adam
    n = 1000
    p = rng.standard_normal(n).astype(np.float32)
    g = rng.standard_normal(n).astype(np.float32)
    m = rng.standard_normal(n).astype(np.float32) * 0.1
    v = np.abs(rng.standard_normal(n).astype(np.float32)) * 0.01
    tp, tg, tm, tv = (torch.from_numpy(a.copy()).to(DEV) for a in (p, g, m, v))
    pb = torch.empty(n, dtype=torch.bfloat16, device=DEV)
    lr, b1, b2, eps, wd, step = 1e-3, 0.9, 0.999, 1e-8, 0.01, 3
    ops.adam(tp, tg, tm, tv, step, lr, b1, b2, eps, wd, gscale=2.0, p_bf16=pb)
    g2 = 2.0 * g.astype(np.float64)
    m2 = b1 * m + (1 - b1) * g2
    v2 = b2 * v + (1 - b2) * g2 * g2
    p2 = p * (1 - lr * wd) - lr * (m2 / (1 - b1 ** step)) / (np.sqrt(v2 / (1 - b2 ** step)) + eps)
    _close(_np(tp), p2, False)
    _close(_np(tm), m2, False)
    _close(_np(pb), p2, True)
    # network input
    track = rng.random((2, 4, 30)).astype(np.float32)
    params = rng.random((2, 4)).astype(np.float32)
    x = torch.empty(2, 30, 64, dtype=torch.bfloat16, device=DEV)
    ops.assemble_input(torch.from_numpy(track).to(DEV), torch.from_numpy(params).to(DEV), x)
    xn = _np(x)
    _close(xn[:, :, :4], np.transpose(track, (0, 2, 1)).astype(np.float64), True)
    _close(xn[:, :, 4:8], np.repeat(params[:, None, :], 30, axis=1).astype(np.float64), True)
    assert not xn[:, :, 8:].any()


def test_band_target_and_map_scores():
    rng = np.random.default_rng(51)
    ncols, nrows = 300, 600
    band = rng.poisson(3.0, size=(ncols, nrows)).astype(np.uint32)
    band[7] = 0  # a bin without contacts
    out = torch.empty(ncols, nrows, dtype=torch.float32, device=DEV)
    ops.band_target(torch.from_numpy(band.view(np.int32)).to(DEV), ncols, nrows, out)
    s = band.sum(1, keepdims=True).astype(np.float64)
    ref = np.log1p(band * np.divide(nrows, s, out=np.zeros_like(s), where=s > 0))
    assert np.allclose(_np(out), ref, rtol=1e-7, atol=1e-7)
    assert not _np(out)[7].any()
    # per-map sums for Pearson r / relative L2
    a = rng.standard_normal((3, 1000)).astype(np.float32)
    b = (a + 0.3 * rng.standard_normal((3, 1000))).astype(np.float32)
    sums = torch.zeros(3, 6, dtype=torch.float64, device=DEV)
    ops.map_sums(torch.from_numpy(a).to(DEV), torch.from_numpy(b).to(DEV), 1000, 3, sums)
    sn = sums.cpu().numpy()
    A, Bm = a.astype(np.float64), b.astype(np.float64)
    want = np.stack([A.sum(1), Bm.sum(1), (A * A).sum(1), (Bm * Bm).sum(1), (A * Bm).sum(1),
                     ((A - Bm) ** 2).sum(1)], 1)
    assert np.allclose(sn, want, rtol=1e-10, atol=1e-8)
    r, rel = ops.map_scores(torch.from_numpy(a).to(DEV), torch.from_numpy(b).to(DEV), 1000, 3)
    for m in range(3):
        assert abs(r[m] - np.corrcoef(A[m], Bm[m])[0, 1]) < 1e-12
        assert abs(rel[m] - np.linalg.norm(A[m] - Bm[m]) / np.linalg.norm(Bm[m])) < 1e-12
    # compacting the head's padded rows
    pad = torch.from_numpy(rng.standard_normal((2, 5, 640)).astype(np.float32)).to(DEV)
    dense = torch.empty(2, 5, 600, dtype=torch.float32, device=DEV)
    ops.compact_rows(pad, 600, dense)
    assert np.array_equal(_np(dense), _np(pad)[:, :, :600])
