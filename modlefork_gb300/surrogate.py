"""The learned surrogate: a 1D U-Net neural operator from a window's barrier track and extrusion
parameters to the expected banded contact map the simulator converges to.

Every arithmetic step runs in the library's own kernels (libmgpu_surrogate.so): the
convolutions on the tensor cores (tcgen05, BF16 operands, FP32 accumulators), pooling,
upsampling, losses, gradients and Adam in hand-written CUDA.  torch only provides device memory
and the stream; there is no autograd: the backward pass is written out layer by layer below.

Architecture (``UNet(widths=(64, 128, 256, 384, 512), mid=512)``, about 8.9 M parameters):

* input: [B, 4000, 64] BF16, channels 0-3 the barrier track (summed occupancy, + motifs,
  - motifs, LEF density), 4-7 the parameter vector, the rest zero;
* encoder level i (length 4000 / 2^i): two 3-tap convolutions with SiLU, then average pooling
  by two; a bottleneck of two 3-tap convolutions at 125 positions;
* decoder level i: nearest upsampling by two concatenated with the encoder's level-i output,
  two 3-tap convolutions with SiLU;
* head: a 1-tap convolution to 640 channels of which the first 600 are the band's diagonals
  d = 0..599 of each bin, in FP32: the output is the band in its own column-major layout
  (ContactMatrixDense, contact_matrix_dense_impl.hpp:40-51), as the row-normalised log1p target.

Training minimises the mean squared error against simulated targets with Adam; evaluation
scores every map by Pearson r and relative L2 against fresh simulator runs, and a map whose r
falls below the gate (0.95) is answered by the simulator instead.
"""

import math
import time

import numpy as np
import torch

from . import surrogate_ops as ops

NROWS = 600     # diagonals of the band (3 Mbp at 5 kb)
HEAD_PAD = 640  # head channels: the 600 diagonals padded to the tile width
IN_CH = 64      # input channels (8 used, padded to the tensor cores' K step)
LOSS_SCALE = 1024.0
# Tuned kernel form (surrogate_ops.FORM_* bits) and pipeline depth per forward convolution,
# name -> (form, stages) (filled from the autotuner's table by autotune.apply_surrogate; results
# do not depend on it).
LAYER_CFG = {}


def tile_width(cout):
    """N tile width msur_conv_forward uses for a convolution with cout output channels."""
    return 64 if cout <= 64 else (256 if cout % 256 == 0 else 128)


def _align(n, a=64):
    return (n + a - 1) // a * a


class ConvSpec:
    def __init__(self, name, cout, taps, cin, act=True):
        self.name, self.cout, self.taps, self.cin, self.act = name, cout, taps, cin, act

    @property
    def wsize(self):
        return self.cout * self.taps * self.cin


def conv_specs(widths, mid):
    """The network's convolutions in order: two per encoder level, two in the bottleneck, two
    per decoder level (deepest first), then the head."""
    specs = []
    cin = IN_CH
    for i, w in enumerate(widths):
        specs += [ConvSpec(f"enc{i}a", w, 3, cin), ConvSpec(f"enc{i}b", w, 3, w)]
        cin = w
    specs += [ConvSpec("mid_a", mid, 3, cin), ConvSpec("mid_b", mid, 3, mid)]
    ch = mid
    for i in reversed(range(len(widths))):
        w = widths[i]
        specs += [ConvSpec(f"dec{i}a", w, 3, ch + w), ConvSpec(f"dec{i}b", w, 3, w)]
        ch = w
    specs.append(ConvSpec("head", HEAD_PAD, 1, widths[0], act=False))
    return specs


class UNet:
    """Parameters, optimiser state and per-batch-size workspaces of the surrogate network."""

    def __init__(self, widths=(64, 128, 256, 384, 512), mid=512, length=4000, device=0, seed=0, head_bias=None):
        self.widths = tuple(widths)
        self.mid = mid
        self.depth = len(widths)
        if length % (1 << self.depth):
            raise ValueError(f"length {length} must be divisible by 2^{self.depth}")
        self.length = length
        self.dev = torch.device("cuda", device)
        specs = conv_specs(self.widths, mid)
        self.specs = {s.name: s for s in specs}
        # one flat FP32 buffer of parameters (each weight and bias 64-element aligned, so every
        # BF16 view starts 16-byte aligned for TMA), its gradient, Adam moments and BF16 copy
        offs, n = {}, 0
        for s in specs:
            offs[s.name] = (n, n + _align(s.wsize))
            n = offs[s.name][1] + _align(s.cout)
        self.nparams_padded = n
        self.nparams = sum(s.wsize + s.cout for s in specs)
        kw = dict(device=self.dev)
        self.p = torch.zeros(n, dtype=torch.float32, **kw)
        self.g = torch.zeros(n, dtype=torch.float32, **kw)
        self.m = torch.zeros(n, dtype=torch.float32, **kw)
        self.v = torch.zeros(n, dtype=torch.float32, **kw)
        self.pb = torch.zeros(n, dtype=torch.bfloat16, **kw)
        self.w32, self.b32, self.wb, self.gw, self.gb, self.wt = {}, {}, {}, {}, {}, {}
        for s in specs:
            wo, bo = offs[s.name]
            shape = (s.cout, s.taps, s.cin)
            self.w32[s.name] = self.p[wo:wo + s.wsize].view(shape)
            self.b32[s.name] = self.p[bo:bo + s.cout]
            self.wb[s.name] = self.pb[wo:wo + s.wsize].view(shape)
            self.gw[s.name] = self.g[wo:wo + s.wsize].view(shape)
            self.gb[s.name] = self.g[bo:bo + s.cout]
            self.wt[s.name] = torch.empty(s.cin, s.taps, s.cout, dtype=torch.bfloat16, **kw)
        self.step_count = 0
        self._ws = {}
        self._init(seed, head_bias)

    # ---- parameters ----------------------------------------------------------------------
    def _init(self, seed, head_bias):
        rng = np.random.default_rng(seed)
        host = np.zeros(self.nparams_padded, dtype=np.float32)
        for name, s in self.specs.items():
            wo = self.w32[name].data_ptr() - self.p.data_ptr()
            wo //= 4
            fan_in = s.taps * s.cin
            gain = 1.6 if s.act else 0.02  # SiLU keeps about 0.36 of the variance; a quiet head
            host[wo:wo + s.wsize] = rng.standard_normal(s.wsize) * gain / math.sqrt(fan_in)
        self.p.copy_(torch.from_numpy(host))
        if head_bias is not None:
            hb = torch.zeros(HEAD_PAD, dtype=torch.float32)
            hb[:NROWS] = torch.as_tensor(np.asarray(head_bias, dtype=np.float32))
            self.b32["head"].copy_(hb)
        self.pb.copy_(self.p)
        self._refresh_transposes()

    def _refresh_transposes(self):
        for name in self.specs:
            ops.weight_transpose(self.wb[name], self.wt[name])

    def params_dict(self):
        """name -> (w [Cout, taps, Cin], b [Cout]) as numpy float32 copies."""
        return {k: (self.w32[k].cpu().numpy(), self.b32[k].cpu().numpy()) for k in self.specs}

    def state_dict(self):
        return {"widths": np.array(self.widths), "mid": np.array(self.mid), "length": np.array(self.length),
                "params": self.p.cpu().numpy()}

    def load_state(self, state):
        p = torch.as_tensor(np.asarray(state["params"], dtype=np.float32))
        if p.numel() != self.p.numel():
            raise ValueError("parameter count differs from this network's")
        self.p.copy_(p)
        self.pb.copy_(self.p)
        self._refresh_transposes()

    @classmethod
    def from_state(cls, state, device=0):
        net = cls(widths=tuple(int(w) for w in state["widths"]), mid=int(state["mid"]), length=int(state["length"]),
                  device=device)
        net.load_state(state)
        return net

    # ---- workspaces ----------------------------------------------------------------------
    def _workspace(self, B, train):
        key = (B, train)
        if key in self._ws:
            return self._ws[key]
        kw = dict(dtype=torch.bfloat16, device=self.dev)
        L, D = self.length, self.depth
        ws = {"x": torch.empty(B, L, IN_CH, **kw), "out": torch.empty(B, L, NROWS, dtype=torch.float32, device=self.dev)}
        lens = [L >> i for i in range(D + 1)]
        for i, w in enumerate(self.widths):
            for k in ("za", "ya", "zb", "yb"):
                if train or k in ("ya", "yb"):
                    ws[f"{k}{i}"] = torch.empty(B, lens[i], w, **kw)
            ws[f"p{i}"] = torch.empty(B, lens[i + 1], w, **kw)
            ch = self.mid if i == D - 1 else self.widths[i + 1]
            ws[f"cat{i}"] = torch.empty(B, lens[i], ch + w, **kw)
            for k in ("zda", "yda", "zdb", "ydb"):
                if train or k in ("yda", "ydb"):
                    ws[f"{k}{i}"] = torch.empty(B, lens[i], w, **kw)
        for k in ("zma", "yma", "zmb", "ymb"):
            if train or k in ("yma", "ymb"):
                ws[k] = torch.empty(B, lens[D], self.mid, **kw)
        if train:
            ws["dout"] = torch.empty(B, L, HEAD_PAD, **kw)
            ws["loss"] = torch.zeros(1, dtype=torch.float64, device=self.dev)
            for i, w in enumerate(self.widths):
                ch = self.mid if i == D - 1 else self.widths[i + 1]
                ws[f"dcat{i}"] = torch.empty(B, lens[i], ch + w, **kw)
                ws[f"dzb{i}"] = torch.empty(B, lens[i], w, **kw)   # encoder b, and the decoder's
                ws[f"dza{i}"] = torch.empty(B, lens[i], w, **kw)   # gradients reuse them per level
                ws[f"ddb{i}"] = torch.empty(B, lens[i], w, **kw)
                ws[f"dda{i}"] = torch.empty(B, lens[i], w, **kw)
                ws[f"dp{i}"] = torch.empty(B, lens[i + 1], w, **kw)
            ws["dmb"] = torch.empty(B, lens[D], self.mid, **kw)
            ws["dma"] = torch.empty(B, lens[D], self.mid, **kw)
        self._ws[key] = ws
        return ws

    # ---- forward -------------------------------------------------------------------------
    def _layer_form(self, name):
        """(form, stages) the convolution `name` runs with: its tuned entry, else the width's."""
        cfg = LAYER_CFG.get(name)
        if cfg is not None:
            return cfg
        bn = tile_width(self.specs[name].cout)
        return ops.conv_get_form(bn), ops.conv_get_stages(bn)

    def _set_layer(self, name):
        cfg = LAYER_CFG.get(name)
        if cfg is not None:
            bn = tile_width(self.specs[name].cout)
            ops.conv_set_form(bn, cfg[0])
            ops.conv_set_stages(bn, cfg[1])

    def _conv(self, name, x, pre=None, post=None, f32=None, **kw):
        s = self.specs[name]
        self._set_layer(name)
        ops.conv_forward(x, self.wb[name], bias=self.b32[name], act=ops.ACT_SILU if s.act else ops.ACT_NONE,
                         out_pre=pre, out_post=post, out_f32=f32, **kw)

    def _conv_fused(self, name, x, post=None, skip=None, dup=None, pool=None):
        s = self.specs[name]
        self._set_layer(name)
        ops.conv_forward_fused(x, self.wb[name], bias=self.b32[name], act=ops.ACT_SILU if s.act else ops.ACT_NONE,
                               out_post=post, skip=skip, dup=dup, pool=pool)

    def fusable(self):
        """Whether inference can fill the decoder's concatenation buffers from the convolutions
        that produce them: those convolutions (the encoders' second, the bottleneck's second and
        the decoders' second above level 0) must run the staged epilogue."""
        names = [f"enc{i}b" for i in range(self.depth)] + ["mid_b"] + [f"dec{i}b" for i in range(1, self.depth)]
        return all(self._layer_form(n)[0] & ops.FORM_STAGED for n in names)

    def forward(self, x, train=False, out=None, fuse=True):
        """x: [B, L, 64] BF16 input; returns the [B, L, 600] FP32 prediction: `out` when given
        (contiguous FP32 on the device), else a workspace view that the next call overwrites.

        In inference (and with fuse, when fusable()) the encoder's second convolution writes its
        output into the skip half of its level's concatenation buffer and, pooled, into the next
        level's input, and the convolution below a decoder level writes its output upsampled into
        the other half, so no separate pooling or upsample-and-concatenate step runs; the results
        are the same either way."""
        B = x.shape[0]
        ws = self._workspace(B, train)
        get = (lambda k: ws.get(k)) if train else (lambda k: None)
        fused = fuse and not train and self.fusable()
        h = x
        ws["h_in0"] = x
        for i in range(self.depth):
            self._conv(f"enc{i}a", h, pre=get(f"za{i}"), post=ws[f"ya{i}"])
            if fused:
                cat = ws[f"cat{i}"]
                self._conv_fused(f"enc{i}b", ws[f"ya{i}"], skip=cat[:, :, cat.shape[-1] - self.widths[i]:],
                                 pool=ws[f"p{i}"])
            else:
                self._conv(f"enc{i}b", ws[f"ya{i}"], pre=get(f"zb{i}"), post=ws[f"yb{i}"])
                ops.pool2(ws[f"yb{i}"], ws[f"p{i}"])
            h = ws[f"p{i}"]
        self._conv("mid_a", h, pre=get("zma"), post=ws["yma"])
        if fused:
            self._conv_fused("mid_b", ws["yma"], dup=ws[f"cat{self.depth - 1}"][:, :, :self.mid])
        else:
            self._conv("mid_b", ws["yma"], pre=get("zmb"), post=ws["ymb"])
            h = ws["ymb"]
        for i in reversed(range(self.depth)):
            if not fused:
                ops.upcat(h, ws[f"yb{i}"], ws[f"cat{i}"])
            self._conv(f"dec{i}a", ws[f"cat{i}"], pre=get(f"zda{i}"), post=ws[f"yda{i}"])
            if fused and i > 0:
                self._conv_fused(f"dec{i}b", ws[f"yda{i}"], dup=ws[f"cat{i - 1}"][:, :, :self.widths[i]])
            else:
                self._conv(f"dec{i}b", ws[f"yda{i}"], pre=get(f"zdb{i}"), post=ws[f"ydb{i}"])
                h = ws[f"ydb{i}"]
        dst = ws["out"] if out is None else out
        self._conv("head", h, f32=dst, n_valid=NROWS, out_stride=NROWS)
        return dst

    # ---- backward ------------------------------------------------------------------------
    def _grads(self, name, x, dz):
        """Weight and bias gradients of convolution `name` with input x and output gradient dz."""
        ops.conv_wgrad(x, dz, self.gw[name])
        ops.bias_grad(dz, self.gb[name])

    def _dgrad(self, name, dz, out, gate=None):
        ops.conv_forward(dz, self.wt[name], out_post=out, gate=gate)

    def backward(self, B):
        """Gradients of the last training forward pass into self.g (after ws['dout'] is set)."""
        ws = self._ws[(B, True)]
        D = self.depth
        self._grads("head", ws["ydb0"], ws["dout"])
        self._dgrad("head", ws["dout"], ws["ddb0"], gate=ws["zdb0"])
        for i in range(D):
            self._grads(f"dec{i}b", ws[f"yda{i}"], ws[f"ddb{i}"])
            self._dgrad(f"dec{i}b", ws[f"ddb{i}"], ws[f"dda{i}"], gate=ws[f"zda{i}"])
            self._grads(f"dec{i}a", ws[f"cat{i}"], ws[f"dda{i}"])
            self._dgrad(f"dec{i}a", ws[f"dda{i}"], ws[f"dcat{i}"])
            if i + 1 < D:
                ops.upcat_bwd(ws[f"dcat{i}"], ws[f"zdb{i + 1}"], ws[f"ddb{i + 1}"])
            else:
                ops.upcat_bwd(ws[f"dcat{i}"], ws["zmb"], ws["dmb"])
        self._grads("mid_b", ws["yma"], ws["dmb"])
        self._dgrad("mid_b", ws["dmb"], ws["dma"], gate=ws["zma"])
        self._grads("mid_a", ws[f"p{D - 1}"], ws["dma"])
        self._dgrad("mid_a", ws["dma"], ws[f"dp{D - 1}"])
        for i in reversed(range(D)):
            ch = self.mid if i == D - 1 else self.widths[i + 1]
            ops.skip_grad(ws[f"zb{i}"], ws[f"dzb{i}"], dpool=ws[f"dp{i}"], dcat=ws[f"dcat{i}"], cat_off=ch)
            self._grads(f"enc{i}b", ws[f"ya{i}"], ws[f"dzb{i}"])
            self._dgrad(f"enc{i}b", ws[f"dzb{i}"], ws[f"dza{i}"], gate=ws[f"za{i}"])
            x_in = ws["h_in0"] if i == 0 else ws[f"p{i - 1}"]
            self._grads(f"enc{i}a", x_in, ws[f"dza{i}"])
            if i > 0:
                self._dgrad(f"enc{i}a", ws[f"dza{i}"], ws[f"dp{i - 1}"])

    def loss_and_grad(self, x, target):
        """Forward, MSE loss against target [B, L, 600] and gradients in self.g (scaled by
        LOSS_SCALE); returns the loss as a device scalar (FP64 sum of squares / count)."""
        B = x.shape[0]
        ws = self._workspace(B, True)
        out = self.forward(x, train=True)
        n = B * self.length * NROWS
        ws["loss"].zero_()
        self.g.zero_()
        ops.mse(out, target, ws["loss"], dp=ws["dout"], scale=2.0 * LOSS_SCALE / n)
        self.backward(B)
        return ws["loss"] / n

    def adam_step(self, lr, b1=0.9, b2=0.999, eps=1e-8, wd=0.0):
        self.step_count += 1
        ops.adam(self.p, self.g, self.m, self.v, self.step_count, lr, b1, b2, eps, wd, gscale=1.0 / LOSS_SCALE,
                 p_bf16=self.pb)
        self._refresh_transposes()

    def flops_per_map(self, backward=False):
        """Multiply-adds x 2 of one map's forward pass (x 3 with the backward pass)."""
        f = 0
        for name, s in self.specs.items():
            level = 0
            if name.startswith(("enc", "dec")):
                level = int(name[3])
            elif name.startswith("mid"):
                level = self.depth
            f += 2 * (self.length >> level) * s.cout * s.taps * s.cin
        return f * (3 if backward else 1)


# ---------------------------------------------------------------------------------------------
class Dataset:
    """Inputs and targets resident on the device: x [N, L, 64] BF16, target [N, L, 600] FP32."""

    def __init__(self, track, params, target, device=0):
        dev = device if isinstance(device, torch.device) else torch.device("cuda", device)
        self.track = torch.as_tensor(track).to(dev, torch.float32).contiguous()
        self.params = torch.as_tensor(params).to(dev, torch.float32).contiguous()
        self.target = torch.as_tensor(target).to(dev, torch.float32).contiguous()
        N, _, L = self.track.shape
        self.x = torch.empty(N, L, IN_CH, dtype=torch.bfloat16, device=dev)
        ops.assemble_input(self.track, self.params, self.x)

    def __len__(self):
        return self.x.shape[0]

    def diagonal_mean(self):
        """Mean target per diagonal over all maps and bins: the distance-decay baseline."""
        return self.target.double().mean(dim=(0, 1)).float().cpu().numpy()


def train(net, data, steps, batch=16, lr=2e-3, lr_min=2e-5, warmup=100, seed=0, log=None, log_every=200):
    """Adam on the MSE with a linear warm-up and cosine decay; returns per-step losses."""
    rng = np.random.default_rng(seed)
    N = len(data)
    xb = torch.empty(batch, net.length, IN_CH, dtype=torch.bfloat16, device=net.dev)
    tb = torch.empty(batch, net.length, NROWS, dtype=torch.float32, device=net.dev)
    losses = []
    t0 = time.perf_counter()
    for step in range(steps):
        idx = torch.from_numpy(rng.choice(N, size=batch, replace=N < batch)).to(net.dev)
        torch.index_select(data.x, 0, idx, out=xb)
        torch.index_select(data.target, 0, idx, out=tb)
        loss = net.loss_and_grad(xb, tb)
        if step < warmup:
            cur = lr * (step + 1) / warmup
        else:
            cur = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * (step - warmup) / max(1, steps - warmup)))
        net.adam_step(cur)
        losses.append(loss)
        if log and (step % log_every == 0 or step == steps - 1):
            log(f"step {step}: loss {loss.item():.5f} lr {cur:.2e} ({time.perf_counter() - t0:.1f} s)")
    return torch.stack(losses).cpu().numpy().ravel()


def predict(net, x, batch=256):
    """Predictions [N, L, 600] FP32 for inputs x [N, L, 64] in batches."""
    out = torch.empty(x.shape[0], net.length, NROWS, dtype=torch.float32, device=net.dev)
    for i in range(0, x.shape[0], batch):
        j = min(x.shape[0], i + batch)
        out[i:j].copy_(net.forward(x[i:j], train=False))
    return out


def predict_host(net, track, params, out, batch=256):
    """Host inputs in, host predictions out: track [N, 4, L] and params [N, 4] FP32 host tensors,
    out [N, L, 600] FP32 host tensor (pinned memory, so that the copies run asynchronously).
    Batches alternate between two device input/output slots: batch i's forward runs on the
    current stream while batch i-1's predictions are copied back on a second stream, so the
    device-to-host copy of the maps (9.6 MB each) overlaps the next batch's compute."""
    N = track.shape[0]
    dev = net.dev
    compute = torch.cuda.current_stream(dev)
    copier = torch.cuda.Stream(device=dev)
    nb = min(batch, N)
    slots = []
    for _ in range(2):
        slots.append({"track": torch.empty((nb,) + tuple(track.shape[1:]), dtype=torch.float32, device=dev),
                      "params": torch.empty((nb,) + tuple(params.shape[1:]), dtype=torch.float32, device=dev),
                      "x": torch.empty(nb, net.length, IN_CH, dtype=torch.bfloat16, device=dev),
                      "out": torch.empty(nb, net.length, NROWS, dtype=torch.float32, device=dev),
                      "copied": None})
    for k, i in enumerate(range(0, N, batch)):
        j = min(N, i + batch)
        sl = slots[k % 2]
        if sl["copied"] is not None:
            compute.wait_event(sl["copied"])  # the slot's previous maps have left the device
        n = j - i
        sl["track"][:n].copy_(track[i:j], non_blocking=True)
        sl["params"][:n].copy_(params[i:j], non_blocking=True)
        ops.assemble_input(sl["track"][:n], sl["params"][:n], sl["x"][:n])
        net.forward(sl["x"][:n], out=sl["out"][:n])
        done = torch.cuda.Event()
        done.record(compute)
        copier.wait_event(done)
        with torch.cuda.stream(copier):
            out[i:j].copy_(sl["out"][:n], non_blocking=True)
            sl["out"].record_stream(copier)
            sl["copied"] = torch.cuda.Event()
            sl["copied"].record(copier)
    compute.wait_stream(copier)
    return out


def evaluate(pred, target):
    """Per-map Pearson r and relative L2 error of predictions against targets (both [N, L, 600])."""
    n = pred.shape[1] * pred.shape[2]
    return ops.map_scores(pred, target, n, pred.shape[0])


def baseline_prediction(diag_mean, n, length, device):
    """The method without the network: every bin predicted by the training set's mean target
    per diagonal (the distance-decay curve)."""
    row = torch.as_tensor(np.asarray(diag_mean, dtype=np.float32), device=device)
    return row.view(1, 1, NROWS).expand(n, length, NROWS).contiguous()
