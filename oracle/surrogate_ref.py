"""FP64 numpy restatement of the surrogate network: test infrastructure, not the product.

The same U-Net as modlefork_gb300.surrogate.UNet (layer order, parameter layout, zero padding,
average pooling, nearest upsampling with skip concatenation, SiLU, the 600-of-640-channel
head and the mean-squared-error loss), written with numpy in float64, forward and backward.
Its backward pass is checked against central finite differences (tests/test_surrogate_cpu.py);
the GPU's gradients are then checked against it (tests/test_surrogate_gpu.py).
"""

import numpy as np

NROWS, HEAD_PAD, IN_CH = 600, 640, 64


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def conv(x, w, b):
    """y[b, l, n] = b[n] + sum_t sum_c x[b, l + t - pad, c] w[n, t, c], zero padded."""
    B, L, _ = x.shape
    taps = w.shape[1]
    pad = (taps - 1) // 2
    xp = np.zeros((B, L + 2 * pad, x.shape[2]))
    xp[:, pad:pad + L] = x
    y = np.zeros((B, L, w.shape[0])) + b
    for t in range(taps):
        y += xp[:, t:t + L] @ w[:, t].T
    return y


def conv_backward(x, w, dz):
    """(dx, dw, db) of conv for output gradient dz."""
    B, L, C = x.shape
    taps = w.shape[1]
    pad = (taps - 1) // 2
    xp = np.zeros((B, L + 2 * pad, C))
    xp[:, pad:pad + L] = x
    dw = np.stack([np.einsum("bln,blc->nc", dz, xp[:, t:t + L]) for t in range(taps)], axis=1)
    db = dz.sum(axis=(0, 1))
    dxp = np.zeros_like(xp)
    for t in range(taps):
        dxp[:, t:t + L] += dz @ w[:, t]
    return dxp[:, pad:pad + L], dw, db


class RefUNet:
    """Parameters as a dict name -> (w [Cout, taps, Cin], b [Cout]) in float64."""

    def __init__(self, widths, mid, length):
        self.widths, self.mid, self.length, self.depth = tuple(widths), mid, length, len(widths)
        specs = []
        cin = IN_CH
        for i, w in enumerate(widths):
            specs += [(f"enc{i}a", w, 3, cin, True), (f"enc{i}b", w, 3, w, True)]
            cin = w
        specs += [("mid_a", mid, 3, cin, True), ("mid_b", mid, 3, mid, True)]
        ch = mid
        for i in reversed(range(self.depth)):
            w = widths[i]
            specs += [(f"dec{i}a", w, 3, ch + w, True), (f"dec{i}b", w, 3, w, True)]
            ch = w
        specs.append(("head", HEAD_PAD, 1, widths[0], False))
        self.specs = specs
        self.params = {}

    def set_params(self, params):
        self.params = {k: (np.asarray(w, np.float64), np.asarray(b, np.float64)) for k, (w, b) in params.items()}

    def forward(self, x):
        P, D = self.params, self.depth
        c = {"x": x}
        h = x
        for i in range(D):
            c[f"za{i}"] = conv(h, *P[f"enc{i}a"])
            c[f"ya{i}"] = silu(c[f"za{i}"])
            c[f"zb{i}"] = conv(c[f"ya{i}"], *P[f"enc{i}b"])
            c[f"yb{i}"] = silu(c[f"zb{i}"])
            y = c[f"yb{i}"]
            c[f"p{i}"] = 0.5 * (y[:, 0::2] + y[:, 1::2])
            h = c[f"p{i}"]
        c["zma"] = conv(h, *P["mid_a"])
        c["yma"] = silu(c["zma"])
        c["zmb"] = conv(c["yma"], *P["mid_b"])
        h = silu(c["zmb"])
        for i in reversed(range(D)):
            c[f"cat{i}"] = np.concatenate([np.repeat(h, 2, axis=1), c[f"yb{i}"]], axis=2)
            c[f"zda{i}"] = conv(c[f"cat{i}"], *P[f"dec{i}a"])
            c[f"yda{i}"] = silu(c[f"zda{i}"])
            c[f"zdb{i}"] = conv(c[f"yda{i}"], *P[f"dec{i}b"])
            h = silu(c[f"zdb{i}"])
        c["ydb0"] = h
        c["out"] = conv(h, *P["head"])[:, :, :NROWS]
        self.cache = c
        return c["out"]

    def loss(self, x, target):
        out = self.forward(x)
        return float(np.mean((out - target) ** 2))

    def gradients(self, x, target):
        """(loss, dict name -> (dw, db)) of the mean squared error."""
        out = self.forward(x)
        c, P, D = self.cache, self.params, self.depth
        n = out.size
        loss = float(np.mean((out - target) ** 2))
        dout = np.zeros(out.shape[:2] + (HEAD_PAD,))
        dout[:, :, :NROWS] = 2.0 * (out - target) / n
        g = {}
        dh, g["head"] = self._back("head", c["ydb0"], dout)
        dz = dh * dsilu(c["zdb0"])
        for i in range(D):
            dy, g[f"dec{i}b"] = self._back(f"dec{i}b", c[f"yda{i}"], dz)
            dz = dy * dsilu(c[f"zda{i}"])
            dcat, g[f"dec{i}a"] = self._back(f"dec{i}a", c[f"cat{i}"], dz)
            ch = dcat.shape[2] - self.widths[i]
            c[f"dskip{i}"] = dcat[:, :, ch:]
            dup = dcat[:, :, :ch]
            dprev = dup[:, 0::2] + dup[:, 1::2]
            zprev = c[f"zdb{i + 1}"] if i + 1 < D else c["zmb"]
            dz = dprev * dsilu(zprev)
        dy, g["mid_b"] = self._back("mid_b", c["yma"], dz)
        dz = dy * dsilu(c["zma"])
        dp, g["mid_a"] = self._back("mid_a", c[f"p{D - 1}"], dz)
        for i in reversed(range(D)):
            dyb = np.repeat(0.5 * dp, 2, axis=1) + c[f"dskip{i}"]
            dz = dyb * dsilu(c[f"zb{i}"])
            dy, g[f"enc{i}b"] = self._back(f"enc{i}b", c[f"ya{i}"], dz)
            dz = dy * dsilu(c[f"za{i}"])
            x_in = c["x"] if i == 0 else c[f"p{i - 1}"]
            dp, g[f"enc{i}a"] = self._back(f"enc{i}a", x_in, dz)
        return loss, g

    def _back(self, name, x, dz):
        w, _ = self.params[name]
        dx, dw, db = conv_backward(x, w, dz)
        return dx, (dw, db)
