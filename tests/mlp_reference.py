"""CPU reference of the learned proposal's network (test infrastructure):
forward pass, pinball loss and its gradient, with optional emulation of
the device's BF16 operands (round to nearest even) so that tensor-core
results can be compared closely.  Parameter layout as the device's:
W0 [64][16] (inputs 0..5 used), W1, W2 [64][64], W3 [16][64], b0, b1, b2
[64], b3 [16]."""

import numpy as np

H, OUT, IN, IN_PAD = 64, 16, 6, 16
OFF = {}
_o = 0
for _name, _size in (("W0", H * IN_PAD), ("W1", H * H), ("W2", H * H), ("W3", OUT * H),
                     ("b0", H), ("b1", H), ("b2", H), ("b3", OUT)):
    OFF[_name] = (_o, _size)
    _o += _size
TOTAL = _o


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32)


def unpack(p):
    def get(name, shape):
        o, n = OFF[name]
        return np.asarray(p[o:o + n], dtype=np.float64).reshape(shape)
    return (get("W0", (H, IN_PAD)), get("W1", (H, H)), get("W2", (H, H)), get("W3", (OUT, H)),
            get("b0", (H,)), get("b1", (H,)), get("b2", (H,)), get("b3", (OUT,)))


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def _q(x, emulate):
    return bf16(x).astype(np.float64) if emulate else np.asarray(x, dtype=np.float64)


def forward(p, x, emulate=True):
    W0, W1, W2, W3, b0, b1, b2, b3 = unpack(p)
    x16 = np.zeros((len(x), IN_PAD))
    x16[:, :IN] = x
    z0 = _q(x16, emulate) @ _q(W0, emulate).T + b0
    z1 = _q(silu(z0), emulate) @ _q(W1, emulate).T + b1
    z2 = _q(silu(z1), emulate) @ _q(W2, emulate).T + b2
    o = _q(silu(z2), emulate) @ _q(W3, emulate).T + b3
    return o, (x16, z0, z1, z2)


def loss_and_grad(p, samples, tau, emulate=True):
    """Mean pinball loss on the sampled bin and its gradient (flat vector)."""
    samples = np.asarray(samples, dtype=np.float64)
    n = len(samples)
    x, bins, t = samples[:, :IN], samples[:, IN].astype(int), samples[:, IN + 1]
    ok = (bins >= 0) & np.isfinite(t)
    o, (x16, z0, z1, z2) = forward(p, x, emulate)
    W0, W1, W2, W3, *_ = unpack(p)
    idx = np.arange(n)
    res = np.where(ok, t - o[idx, np.clip(bins, 0, OUT - 1)], 0.0)
    loss = np.where(ok, np.where(res > 0, tau * res, (tau - 1.0) * res), 0.0).sum() / n
    d_o = np.zeros_like(o)
    d_o[idx[ok], bins[ok]] = np.where(res[ok] > 0, -tau, 1.0 - tau) / n
    q = lambda a: _q(a, emulate)  # noqa: E731
    h0, h1, h2 = silu(z0), silu(z1), silu(z2)
    g = {"W3": q(d_o).T @ q(h2), "b3": d_o.sum(0)}
    dz2 = (q(d_o) @ q(W3)) * dsilu(z2)
    g["W2"], g["b2"] = q(dz2).T @ q(h1), dz2.sum(0)
    dz1 = (q(dz2) @ q(W2)) * dsilu(z1)
    g["W1"], g["b1"] = q(dz1).T @ q(h0), dz1.sum(0)
    dz0 = (q(dz1) @ q(W1)) * dsilu(z0)
    g["W0"], g["b0"] = q(dz0).T @ q(x16), dz0.sum(0)
    g["W0"][:, IN:] = 0.0
    flat = np.zeros(TOTAL)
    for name, (off, size) in OFF.items():
        flat[off:off + size] = np.asarray(g[name]).ravel()
    return loss, flat


def init(seed):
    """He-uniform initial parameters (the device uses its own generator)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(TOTAL, dtype=np.float32)
    for name, fan_in, shape in (("W0", IN, (H, IN_PAD)), ("W1", H, (H, H)), ("W2", H, (H, H)),
                                ("W3", H, (OUT, H))):
        o, n = OFF[name]
        w = rng.uniform(-1, 1, shape) * np.sqrt(6.0 / fan_in)
        if name == "W0":
            w[:, IN:] = 0.0
        p[o:o + n] = w.ravel()
    for name in ("b0", "b1", "b2", "b3"):
        o, n = OFF[name]
        p[o:o + n] = rng.normal(0.0, 0.1, n)
    return p
