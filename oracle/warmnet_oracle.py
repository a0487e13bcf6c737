"""CPU restatement of the learned SOR warm-start network (numpy).

TEST INFRASTRUCTURE ONLY: loaded by tests/ as the checker of the CUDA
forward and backward kernels (fargo_thorin_gb300/csrc/warmnet.cu); the
product never imports it.  The network has no counterpart in the reference,
which starts every SOR solve from the previous temperature
(src_main/EnergySources.c:406-511).

``bf16=True`` rounds to bfloat16 (round to nearest even) at the same points
as the CUDA kernels: network input, weights, every stored activation, the
output gradient and the masked gradients fed to the tensor cores; sums run
in float64 and are rounded to float32 where the kernels keep FP32.  With
``bf16=False`` everything stays float64, which is what the finite-difference
check of the backward pass uses.
"""
from __future__ import annotations

import numpy as np

C = 32
NIN = 7
INPUTS = 16
# (cin, cout) per layer: e0 e1 e2 e3 d2 d1 d0 out
LAYERS = [(NIN, C)] + [(C, C)] * 6 + [(C, 1)]


def layer_offsets():
    off, o = [], 0
    for cin, cout in LAYERS:
        off.append(o)
        o += cout * 9 * cin + cout
    return off, o


OFFSETS, NPARAMS = layer_offsets()


def bf16(x):
    """Round float32 values to the nearest bfloat16 (ties to even)."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).reshape(a.shape)


def bf16_bits(x):
    return (bf16(x).view(np.uint32) >> 16).astype(np.uint16)


def from_bits(b):
    return (b.astype(np.uint32) << 16).view(np.float32)


def unpack(params):
    out = []
    for (cin, cout), o in zip(LAYERS, OFFSETS):
        w = params[o:o + cout * 9 * cin].reshape(cout, 9, cin)
        b = params[o + cout * 9 * cin:o + cout * 9 * cin + cout]
        out.append((w, b))
    return out


def _shift(x, dr, dc):
    """x[b, i + dr, (j + dc) mod W, c], zero outside rings 0..H-1."""
    y = np.roll(x, -dc, axis=2)
    out = np.zeros_like(y)
    H = x.shape[1]
    if dr == 0:
        out[:] = y
    elif dr > 0:
        out[:, :H - dr] = y[:, dr:]
    else:
        out[:, -dr:] = y[:, :H + dr]
    return out


TAPS = [(t // 3 - 1, t % 3 - 1) for t in range(9)]


def conv(x, w):
    """3x3 convolution, periodic in azimuth, zero-padded in radius:
    out[p][co] = sum_t sum_ci x[p + tap_t][ci] * w[co][t][ci] (float64)."""
    out = 0.0
    for t, (dr, dc) in enumerate(TAPS):
        out = out + np.einsum("bhwc,oc->bhwo", _shift(x, dr, dc).astype(np.float64), w[:, t, :].astype(np.float64))
    return out


def conv_input_grad(g, w):
    """Gradient of conv with respect to its input: conv of g with the
    flipped, transposed kernel."""
    wt = np.transpose(w[:, ::-1, :], (2, 1, 0))     # [ci][t'][co] = w[co][8 - t'][ci]
    return conv(g, wt)


def weight_grad(x, g):
    """dW[co][t][ci] = sum_p g[p][co] * x[p + tap_t][ci]; db[co] = sum_p g[p][co]."""
    dw = np.stack([np.einsum("bhwo,bhwc->oc", g.astype(np.float64), _shift(x, dr, dc).astype(np.float64))
                   for dr, dc in TAPS], axis=1)
    return dw, g.astype(np.float64).sum(axis=(0, 1, 2))


def pool(a):
    return 0.25 * ((a[:, 0::2, 0::2] + a[:, 0::2, 1::2]) + (a[:, 1::2, 0::2] + a[:, 1::2, 1::2]))


def up(a):
    return np.repeat(np.repeat(a, 2, axis=1), 2, axis=2)


def forward(params, x, bf=True):
    """x: [B][H][W][16] float (bf16 values when bf).  Returns y [B][H][W] and
    the stored activations."""
    R = bf16 if bf else (lambda v: np.asarray(v, dtype=np.float64))
    F = (lambda v: np.asarray(v, dtype=np.float32)) if bf else (lambda v: np.asarray(v, dtype=np.float64))
    L = [(R(w), F(b)) for w, b in unpack(np.asarray(params, dtype=np.float32 if bf else np.float64))]
    x6 = R(x)[..., :NIN]
    act = {}

    def layer(k, inp):
        w, b = L[k]
        return R(np.maximum(F(conv(inp, w)) + b, 0.0))

    act["x"] = x6
    act["a0"] = layer(0, x6)
    act["p1"] = R(pool(F(act["a0"])))
    act["a1"] = layer(1, act["p1"])
    act["p2"] = R(pool(F(act["a1"])))
    act["a2"] = layer(2, act["p2"])
    act["p3"] = R(pool(F(act["a2"])))
    act["a3"] = layer(3, act["p3"])
    act["u2"] = R(F(up(act["a3"])) + F(act["a2"]))
    act["b2"] = layer(4, act["u2"])
    act["u1"] = R(F(up(act["b2"])) + F(act["a1"]))
    act["b1"] = layer(5, act["u1"])
    act["u0"] = R(F(up(act["b1"])) + F(act["a0"]))
    act["b0"] = layer(6, act["u0"])
    w, b = L[7]
    y = F(conv(act["b0"], w))[..., 0] + b[0]
    return y, act


def loss_and_grad(params, x, target, bf=True):
    """Loss mean over rings 1..H-2 of (y - target)^2 and its gradient."""
    R = bf16 if bf else (lambda v: np.asarray(v, dtype=np.float64))
    F = (lambda v: np.asarray(v, dtype=np.float32)) if bf else (lambda v: np.asarray(v, dtype=np.float64))
    y, act = forward(params, x, bf)
    B, H, W = y.shape
    inv_n = 1.0 / (B * (H - 2) * W)
    if bf:
        inv_n = np.float32(inv_n)
    mask = np.zeros((B, H, W), bool)
    mask[:, 1:H - 1] = True
    d = np.where(mask, F(y) - F(target), 0.0)
    loss = float((d.astype(np.float64) ** 2).sum() * float(inv_n))
    gy = R(F(2.0 * d * inv_n))[..., None]
    Lw = [R(w) for w, _ in unpack(np.asarray(params, dtype=np.float32 if bf else np.float64))]
    grads = [None] * 8

    def wg(k, inp, g):
        grads[k] = weight_grad(inp, g)

    def relu_mask(g, a):
        return R(np.where(a > 0, F(g), 0.0))

    wg(7, act["b0"], gy)
    g = relu_mask(F(conv_input_grad(gy, Lw[7])), act["b0"])
    wg(6, act["u0"], g)
    ga0 = F(conv_input_grad(g, Lw[6]))
    g = relu_mask(pool(ga0) * 4.0, act["b1"])
    wg(5, act["u1"], g)
    ga1 = F(conv_input_grad(g, Lw[5]))
    g = relu_mask(pool(ga1) * 4.0, act["b2"])
    wg(4, act["u2"], g)
    ga2 = F(conv_input_grad(g, Lw[4]))
    g = relu_mask(pool(ga2) * 4.0, act["a3"])
    wg(3, act["p3"], g)
    gp3 = F(conv_input_grad(g, Lw[3]))
    g = relu_mask(ga2 + 0.25 * up(gp3), act["a2"])
    wg(2, act["p2"], g)
    gp2 = F(conv_input_grad(g, Lw[2]))
    g = relu_mask(ga1 + 0.25 * up(gp2), act["a1"])
    wg(1, act["p1"], g)
    gp1 = F(conv_input_grad(g, Lw[1]))
    g = relu_mask(ga0 + 0.25 * up(gp1), act["a0"])
    wg(0, act["x"], g)
    flat = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])
    return loss, flat, y
