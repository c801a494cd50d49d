"""TEST INFRASTRUCTURE ONLY -- the CPU checker of the learned accelerator's network.

A numpy (FP64) restatement of the U-Net that the library runs and trains
with its own BF16 kernels (doma_gb300/csrc/unet.cu, conv.cu): the same layer
table, parameter layout, forward pass, mean-square loss and hand-derived
backward pass.  With ``bf16=True`` every tensor the GPU stores in BF16
(weights, activations, activation gradients) is rounded to BF16
(round-to-nearest-even) at the same point, so the GPU's results differ from
this only by FP32-vs-FP64 accumulation and the odd rounding-boundary flip.
With ``bf16=False`` it is plain FP64 calculus, which ``finite_difference``
checks.  DOMA itself has no learned accelerator, so nothing here restates a
DOMA file; the product never imports this module.
"""
from __future__ import annotations

import numpy as np

IN_CH = 16
WIDTH = (32, 64, 128, 256)
# (cin, cout, relu) of the 14 convolutions, in parameter order
LAYERS = [
    (IN_CH, 32, True), (32, 32, True),
    (32, 64, True), (64, 64, True),
    (64, 128, True), (128, 128, True),
    (128, 256, True), (256, 256, True),
    (256, 128, False), (128, 128, True),
    (128, 64, False), (64, 64, True),
    (64, 32, False), (32, 32, True),
]


def layout():
    """Offsets (w_off, b_off) per layer, head (w_off, b_off), total count."""
    offs, o = [], 0
    for cin, cout, _ in LAYERS:
        w = o
        o += 27 * cin * cout
        offs.append((w, o))
        o += cout
    head = (o, o + 32)
    return offs, head, o + 33


def round_bf16(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    out = ((u + r) & 0xFFFF0000).astype(np.uint32)
    return out.view(np.float32).astype(np.float64)


class Params:
    def __init__(self, flat: np.ndarray, bf16: bool):
        offs, head, n = layout()
        assert flat.size == n
        self.w, self.b = [], []
        for (cin, cout, _), (wo, bo) in zip(LAYERS, offs):
            w = flat[wo:wo + 27 * cin * cout].reshape(27, cout, cin).astype(np.float64)
            self.w.append(round_bf16(w) if bf16 else w)
            self.b.append(flat[bo:bo + cout].astype(np.float64))
        self.hw = flat[head[0]:head[0] + 32].astype(np.float64)
        self.hb = float(flat[head[1]])


def taps():
    for t in range(27):
        yield t, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1


def shifted(x, dz, dy, dx):
    """x[b, z+dz, y+dy, x+dx, :] with zeros outside."""
    B, Z, Y, X, C = x.shape
    xp = np.zeros((B, Z + 2, Y + 2, X + 2, C))
    xp[:, 1:-1, 1:-1, 1:-1] = x
    return xp[:, 1 + dz:1 + dz + Z, 1 + dy:1 + dy + Y, 1 + dx:1 + dx + X]


def conv(x, w, b=None):
    out = 0.0
    for t, dz, dy, dx in taps():
        out = out + shifted(x, dz, dy, dx) @ w[t].T
    return out + (0.0 if b is None else b)


def conv_dgrad(g, w):
    """Gradient of conv's input: sum_t shift(g, -t) @ w[t]."""
    out = 0.0
    for t, dz, dy, dx in taps():
        out = out + shifted(g, -dz, -dy, -dx) @ w[t]
    return out


def conv_wgrad(x, g):
    """dw[t][co][ci] = sum_m g[m][co] * x[m + off(t)][ci]."""
    cin, cout = x.shape[-1], g.shape[-1]
    dw = np.zeros((27, cout, cin))
    gm = g.reshape(-1, cout)
    for t, dz, dy, dx in taps():
        dw[t] = gm.T @ shifted(x, dz, dy, dx).reshape(-1, cin)
    return dw


def pool(x):
    B, Z, Y, X, C = x.shape
    return x.reshape(B, Z // 2, 2, Y // 2, 2, X // 2, 2, C).mean(axis=(2, 4, 6))


def sumpool(x):
    B, Z, Y, X, C = x.shape
    return x.reshape(B, Z // 2, 2, Y // 2, 2, X // 2, 2, C).sum(axis=(2, 4, 6))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def forward(flat, x, bf16=True):
    """-> (out [B,Z,Y,X], cache)"""
    P = Params(flat, bf16)
    R = round_bf16 if bf16 else (lambda a: a)
    relu = lambda a: np.maximum(a, 0.0)
    c = {"x": R(x)}
    e = [None] * 4
    ea = [None] * 4
    p = [None] * 4
    ea[0] = R(relu(conv(c["x"], P.w[0], P.b[0])))
    e[0] = R(relu(conv(ea[0], P.w[1], P.b[1])))
    for l in range(1, 4):
        p[l] = R(pool(e[l - 1]))
        ea[l] = R(relu(conv(p[l], P.w[2 * l], P.b[2 * l])))
        e[l] = R(relu(conv(ea[l], P.w[2 * l + 1], P.b[2 * l + 1])))
    cc, u, d = [None] * 4, [None] * 4, [None] * 4
    deep = e[3]
    for l in (2, 1, 0):
        upl = 8 + 2 * (2 - l)
        cc[l + 1] = R(conv(deep, P.w[upl], P.b[upl]))
        u[l] = R(relu(up(cc[l + 1]) + e[l]))
        d[l] = R(relu(conv(u[l], P.w[upl + 1], P.b[upl + 1])))
        deep = d[l]
    out = d[0] @ P.hw + P.hb
    c.update(e=e, ea=ea, p=p, cc=cc, u=u, d=d, P=P)
    return out, c


def loss_and_grads(flat, x, target, bf16=True):
    """Mean-square loss and the gradient of every parameter (flat, float64)."""
    out, c = forward(flat, x, bf16)
    P = c["P"]
    R = round_bf16 if bf16 else (lambda a: a)
    offs, head, n = layout()
    g = np.zeros(n)
    V = out.size
    r = out - target
    loss = float(np.sum(r * r) / V)
    gs_out = 2.0 * r / V
    if bf16:
        gs_out = gs_out.astype(np.float32).astype(np.float64)
    d, u, e, ea, p, cc = c["d"], c["u"], c["e"], c["ea"], c["p"], c["cc"]
    g[head[0]:head[0] + 32] = np.tensordot(gs_out, d[0], axes=(range(4), range(4)))
    g[head[1]] = gs_out.sum()
    gz = R(gs_out[..., None] * P.hw * (d[0] > 0))

    def put(layer, x_in, gz_):
        wo, bo = offs[layer]
        cin, cout, _ = LAYERS[layer]
        g[wo:wo + 27 * cin * cout] = conv_wgrad(x_in, gz_).reshape(-1)
        g[bo:bo + cout] = gz_.reshape(-1, cout).sum(axis=0)

    gs = [None] * 3
    for l in (0, 1, 2):
        upl = 8 + 2 * (2 - l)
        put(upl + 1, u[l], gz)
        gs[l] = R(conv_dgrad(gz, P.w[upl + 1])) * (u[l] > 0)
        gc = R(sumpool(gs[l]))
        deep_in = e[3] if l == 2 else d[l + 1]
        put(upl, deep_in, gc)
        gz = R(conv_dgrad(gc, P.w[upl])) * (deep_in > 0)
    # bottom (gz = gradient of e3's pre-activation)
    put(7, ea[3], gz)
    gz = R(conv_dgrad(gz, P.w[7])) * (ea[3] > 0)
    put(6, p[3], gz)
    gp = R(conv_dgrad(gz, P.w[6]))
    for l in (2, 1, 0):
        gz = R((up(gp) * 0.125 + gs[l]) * (e[l] > 0))
        put(2 * l + 1, ea[l], gz)
        gz = R(conv_dgrad(gz, P.w[2 * l + 1])) * (ea[l] > 0)
        put(2 * l, c["x"] if l == 0 else p[l], gz)
        if l > 0:
            gp = R(conv_dgrad(gz, P.w[2 * l]))
    return loss, g, out


def finite_difference(flat, x, target, direction, eps=1e-6):
    """Central difference of the FP64 loss along `direction`."""
    lp, _, _ = loss_and_grads(flat + eps * direction, x, target, bf16=False)
    lm, _, _ = loss_and_grads(flat - eps * direction, x, target, bf16=False)
    return (lp - lm) / (2 * eps)
