"""Python binding of the surrogate's GPU kernels (libmgpu_surrogate.so, include/mgpu_surrogate.h).

Every function takes torch CUDA tensors (used here only as device memory) and enqueues the
library's own kernel on the current torch stream; there is no fallback: if the library is
missing, loading fails.  Activations are channels-last BF16 [B, L, C]; convolution weights are
BF16 [Cout, taps, Cin].
"""

import ctypes as C
import os

import numpy as np
import torch

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_lib", "libmgpu_surrogate.so")
ACT_NONE, ACT_SILU = 0, 1
_lib = None


class SurrogateKernelError(RuntimeError):
    pass


def load(path=LIB_PATH):
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: run modlefork_gb300.build.build() first")
    lib = C.CDLL(path)
    vp, i32, u64, f32 = C.c_void_p, C.c_int, C.c_uint64, C.c_float
    sigs = {
        "msur_last_error_string": (C.c_char_p, []),
        "msur_take_error": (i32, [C.POINTER(C.c_uint)]),
        "msur_conv_forward": (i32, [vp, i32, i32, i32, vp, i32, i32, vp, i32, vp, vp, vp, i32, i32, vp, vp]),
        "msur_conv_wgrad": (i32, [vp, vp, i32, i32, i32, i32, i32, vp, i32, vp]),
        "msur_pool2": (i32, [vp, i32, i32, i32, vp, vp]),
        "msur_skip_grad": (i32, [vp, i32, vp, i32, i32, vp, i32, i32, i32, vp, vp]),
        "msur_upcat": (i32, [vp, vp, i32, i32, i32, i32, vp, vp]),
        "msur_upcat_bwd": (i32, [vp, vp, i32, i32, i32, i32, vp, vp]),
        "msur_bias_grad": (i32, [vp, u64, i32, i32, vp, vp]),
        "msur_mse": (i32, [vp, i32, vp, i32, u64, i32, vp, i32, f32, vp, vp]),
        "msur_adam": (i32, [vp, vp, vp, vp, u64, f32, f32, f32, f32, f32, i32, f32, vp, vp]),
        "msur_weight_transpose": (i32, [vp, i32, i32, i32, vp, vp]),
        "msur_assemble_input": (i32, [vp, vp, i32, i32, i32, vp, vp]),
        "msur_band_target": (i32, [vp, u64, i32, vp, vp]),
        "msur_map_sums": (i32, [vp, u64, vp, u64, u64, i32, vp, vp, vp]),
        "msur_compact_rows": (i32, [vp, i32, u64, i32, vp, vp]),
        "msur_conv_set_stages": (i32, [i32, i32]),
        "msur_conv_get_stages": (i32, [i32]),
        "msur_conv_forward_fused": (i32, [C.c_void_p, i32, i32, i32, C.c_void_p, i32, i32, C.c_void_p, i32,
                                           C.c_void_p, i32, C.c_void_p, i32, C.c_void_p, i32, C.c_void_p, i32,
                                           i32, C.c_void_p]),
        "msur_conv_set_form": (i32, [i32, i32]),
        "msur_conv_get_form": (i32, [i32]),
        "msur_conv_set_persistent": (i32, [i32, i32]),
        "msur_conv_get_persistent": (i32, [i32]),
    }
    for name, (res, args) in sigs.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def _check(rc, what):
    if rc != 0:
        raise SurrogateKernelError(f"{what}: {load().msur_last_error_string().decode(errors='replace')}")


def _p(t):
    return None if t is None else t.data_ptr()


def _stream():
    return torch.cuda.current_stream().cuda_stream


def take_error():
    """Read and clear the tensor-core kernels' wait-timeout flag (0 = none)."""
    code = C.c_uint()
    _check(load().msur_take_error(C.byref(code)), "msur_take_error")
    return code.value


def conv_forward(x, w, bias=None, act=ACT_NONE, out_pre=None, out_post=None, out_f32=None, n_valid=None,
                 out_stride=None, gate=None):
    """v = conv(x, w) + bias over positions (zero padded), optionally times silu'(gate);
    writes v (out_pre, out_f32) and act(v) (out_post).  x [B, L, Cin], w [Cout, taps, Cin]."""
    B, L, Cin = x.shape
    Cout, taps, Cin_w = w.shape
    assert Cin_w == Cin and x.dtype == torch.bfloat16 and w.dtype == torch.bfloat16
    outs = [t for t in (out_pre, out_post, out_f32) if t is not None]
    if out_stride is None:
        out_stride = outs[0].shape[-1]
    if n_valid is None:
        n_valid = min(Cout, out_stride)
    _check(load().msur_conv_forward(_p(x), B, L, Cin, _p(w), Cout, taps, _p(bias), act, _p(out_pre), _p(out_post),
                                    _p(out_f32), out_stride, n_valid, _p(gate), _stream()), "msur_conv_forward")


def conv_forward_fused(x, w, bias=None, act=ACT_NONE, out_post=None, skip=None, dup=None, pool=None):
    """conv_forward's post-activation value written to out_post [B, L, Cout] (or None), to the
    row-strided view `skip` [B, L, Cout] (e.g. cat[:, :, C1:]), upsampled by two to the
    row-strided view `dup` [B, 2L, Cout] (e.g. cat[:, :, :C1]) and average-pooled by two to
    `pool` [B, L/2, Cout] (as pool2 computes it); needs the staged kernel form."""
    B, L, Cin = x.shape
    Cout, taps, _ = w.shape
    for t, rows in ((skip, L), (dup, 2 * L), (pool, L // 2)):
        if t is not None:
            assert t.shape == (B, rows, Cout) and t.stride(2) == 1 and t.stride(0) == rows * t.stride(1)
    out_stride = out_post.shape[-1] if out_post is not None else Cout
    stride = lambda t: t.stride(1) if t is not None else 0  # noqa: E731
    _check(load().msur_conv_forward_fused(
        _p(x), B, L, Cin, _p(w), Cout, taps, _p(bias), act, _p(out_post), out_stride, _p(skip), stride(skip),
        _p(dup), stride(dup), _p(pool), stride(pool), Cout, _stream()), "msur_conv_forward_fused")


def conv_wgrad(x, dz, dw, splits=0):
    """dw [Cout, taps, Cin] (FP32) += weight gradient of conv(x, w) for output gradient dz."""
    B, L, Cin = x.shape
    Cout, taps, _ = dw.shape
    assert dz.shape == (B, L, Cout) and dw.dtype == torch.float32
    _check(load().msur_conv_wgrad(_p(x), _p(dz), B, L, Cin, Cout, taps, _p(dw), splits, _stream()),
           "msur_conv_wgrad")


def pool2(x, y):
    B, Lout, C = y.shape
    _check(load().msur_pool2(_p(x), B, Lout, C, _p(y), _stream()), "msur_pool2")


def skip_grad(z, dz, dpool=None, dcat=None, cat_off=0):
    B, L, C = z.shape
    Lp = dpool.shape[1] if dpool is not None else 0
    cat_stride = dcat.shape[-1] if dcat is not None else 0
    _check(load().msur_skip_grad(_p(dpool), Lp, _p(dcat), cat_stride, cat_off, _p(z), B, L, C, _p(dz), _stream()),
           "msur_skip_grad")


def upcat(x, skip, out):
    B, L, C2 = skip.shape
    C1 = x.shape[-1]
    _check(load().msur_upcat(_p(x), _p(skip), B, L, C1, C2, _p(out), _stream()), "msur_upcat")


def upcat_bwd(dcat, z, dz):
    B, Lh, C1 = z.shape
    _check(load().msur_upcat_bwd(_p(dcat), _p(z), B, Lh, C1, dcat.shape[-1], _p(dz), _stream()), "msur_upcat_bwd")


def bias_grad(dz, db, n_valid=None):
    C = n_valid or db.shape[0]
    rows = dz.numel() // dz.shape[-1]
    _check(load().msur_bias_grad(_p(dz), rows, C, dz.shape[-1], _p(db), _stream()), "msur_bias_grad")


def mse(pred, target, loss, dp=None, scale=1.0, n_valid=None):
    n_valid = n_valid or target.shape[-1]
    rows = pred.numel() // pred.shape[-1]
    dstride = dp.shape[-1] if dp is not None else n_valid
    _check(load().msur_mse(_p(pred), pred.shape[-1], _p(target), target.shape[-1], rows, n_valid, _p(dp), dstride,
                           scale, _p(loss), _stream()), "msur_mse")


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0, gscale=1.0, p_bf16=None):
    _check(load().msur_adam(_p(p), _p(g), _p(m), _p(v), p.numel(), lr, b1, b2, eps, wd, step, gscale, _p(p_bf16),
                            _stream()), "msur_adam")


def weight_transpose(w, wt):
    N, taps, Cw = w.shape
    _check(load().msur_weight_transpose(_p(w), N, taps, Cw, _p(wt), _stream()), "msur_weight_transpose")


def assemble_input(track, params, x):
    B, L, C = x.shape
    _check(load().msur_assemble_input(_p(track), _p(params), B, L, C, _p(x), _stream()), "msur_assemble_input")


def band_target(band, ncols, nrows, out):
    _check(load().msur_band_target(_p(band), ncols, nrows, _p(out), _stream()), "msur_band_target")


def map_sums(pred, ref, n, nmaps, out, pstride=None, rstride=None, means=None):
    pstride = pstride if pstride is not None else n
    rstride = rstride if rstride is not None else n
    _check(load().msur_map_sums(_p(pred), pstride, _p(ref), rstride, n, nmaps, _p(means), _p(out), _stream()),
           "msur_map_sums")


def map_scores(pred, ref, n, nmaps, pstride=None, rstride=None):
    """Per-map Pearson r (two passes: means, then covariances of the deviations, clamped to
    [-1, 1], as src/stats/correlation_impl.hpp:66-87 computes it) and relative L2 error
    ||p - r|| / ||r||, both in FP64 on the device.  Returns two numpy arrays of nmaps values."""
    dev = pred.device
    s1 = torch.zeros(nmaps, 6, dtype=torch.float64, device=dev)
    map_sums(pred, ref, n, nmaps, s1, pstride, rstride)
    means = (s1[:, :2] / n).contiguous()
    s2 = torch.zeros(nmaps, 6, dtype=torch.float64, device=dev)
    map_sums(pred, ref, n, nmaps, s2, pstride, rstride, means=means)
    s2 = s2.cpu().numpy()
    raw = s1.cpu().numpy()
    r = np.clip(s2[:, 4] / np.sqrt(s2[:, 2] * s2[:, 3]), -1.0, 1.0)
    rel_l2 = np.sqrt(s2[:, 5] / raw[:, 3])
    return r, rel_l2


def compact_rows(inp, n_valid, out):
    rows = inp.numel() // inp.shape[-1]
    _check(load().msur_compact_rows(_p(inp), inp.shape[-1], rows, n_valid, _p(out), _stream()), "msur_compact_rows")


def conv_set_stages(bn, stages):
    """Pipeline depth (2-4 stages) of the convolution kernels with N tile bn (64, 128, 256)."""
    _check(load().msur_conv_set_stages(bn, stages), "msur_conv_set_stages")


def conv_get_stages(bn):
    return load().msur_conv_get_stages(bn)


FORM_PERSISTENT = 1  # bit 0: persistent kernel instead of one CTA per tile
FORM_STAGED = 2      # bit 1: outputs through shared memory and TMA stores


def conv_set_form(bn, form):
    """Kernel form (FORM_* bits, 0-3) of the convolution kernels with N tile bn (64, 128, 256)."""
    _check(load().msur_conv_set_form(bn, form), "msur_conv_set_form")


def conv_get_form(bn):
    return load().msur_conv_get_form(bn)


def conv_set_persistent(bn, on):
    """Persistent (1) or one-CTA-per-tile (0) convolution kernel for N tile bn (64, 128, 256)."""
    _check(load().msur_conv_set_persistent(bn, 1 if on else 0), "msur_conv_set_persistent")


def conv_get_persistent(bn):
    return load().msur_conv_get_persistent(bn)
