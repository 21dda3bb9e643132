"""CPU oracle of the pose-proposal network (test infrastructure only: the
parity tests compare libgbrelion's gbr_posenet_* kernels with it; nothing in
the product imports it).

No counterpart in the reference: its coarse search is exhaustive
(src/acc/acc_ml_optimiser_impl.h:1016-1414).  This file restates, in float64
numpy, the network that relion_gb300/csrc/k_posenet.cu defines:

  features  polar bins of the whitened coarse power |X_j|^2 * 2 minv_j over the
            active coarse pixels: ring = ROUND(sqrt(x^2 + y^2)) in 1..H (ROUND as
            src/macros.h, half away from zero), angle bin floor((atan2(y, x) +
            pi/2) / pi * W) with W -> 0; value log(1 + mean) - log 2, 0 in
            empty bins
  conv      out[b,o,y,x] = bias[o] + sum_{c,ky,kx} K[o,c,ky,kx] in[b,c,y+ky-1,(x+kx-2) mod W]
            (zero outside the rings), ReLU; two layers 1 -> C1 -> C2, 3 x 5
  pool      mean over the angle axis
  linear    logits = h W3 + b3
  loss      mean over samples of sum_n t_n (logsumexp(l) - l_n)

and its exact gradient (checked against central differences in
tests/test_oracle_posenet.py).
"""
import numpy as np

KH, KW = 3, 5


def layout(H, W, C1, C2, ND):
    """Offsets of W1, b1, W2, b2, W3, b3 in the flat parameter array."""
    F = C2 * H
    o = {}
    o["w1"] = 0
    o["b1"] = o["w1"] + C1 * KH * KW
    o["w2"] = o["b1"] + C1
    o["b2"] = o["w2"] + C2 * C1 * KH * KW
    o["w3"] = o["b2"] + C2
    o["b3"] = o["w3"] + F * ND
    o["n"] = o["b3"] + ND
    return o


def unpack(p, H, W, C1, C2, ND):
    o = layout(H, W, C1, C2, ND)
    return dict(w1=p[o["w1"]:o["b1"]].reshape(C1, 1, KH, KW), b1=p[o["b1"]:o["w2"]],
                w2=p[o["w2"]:o["b2"]].reshape(C2, C1, KH, KW), b2=p[o["b2"]:o["w3"]],
                w3=p[o["w3"]:o["b3"]].reshape(C2 * H, ND), b3=p[o["b3"]:o["n"]])


def pixel_bins(xy, H, W):
    x = xy[:, 0].astype(np.float64)
    y = xy[:, 1].astype(np.float64)
    ring = np.floor(np.sqrt(x * x + y * y) + 0.5).astype(np.int64)
    a = np.arctan2(y, x) + 0.5 * np.pi
    t = np.floor(a / np.pi * W).astype(np.int64)
    t[t >= W] -= W
    t[t < 0] = 0
    b = (ring - 1) * W + t
    b[(ring < 1) | (ring > H)] = -1
    return b


def features(fimg, xy, minv, H, W):
    """fimg [B][cur][cur/2+1] complex -> features [B][H*W]."""
    fimg = np.asarray(fimg)
    cur = fimg.shape[1]
    rows = np.where(xy[:, 1] < 0, xy[:, 1] + cur, xy[:, 1])
    X = fimg[:, rows, xy[:, 0]].astype(np.complex128)
    v = (X.real ** 2 + X.imag ** 2) * 2.0 * minv.astype(np.float64)[None, :]
    bins = pixel_bins(xy, H, W)
    ok = bins >= 0
    nb = H * W
    cnt = np.bincount(bins[ok], minlength=nb).astype(np.float64)
    out = np.zeros((len(fimg), nb))
    for i in range(len(fimg)):
        s = np.bincount(bins[ok], weights=v[i, ok], minlength=nb)
        m = np.where(cnt > 0, s / np.maximum(cnt, 1), 0.0)
        out[i] = np.where(cnt > 0, np.log1p(m) - np.log(2.0), 0.0)
    return out


def _shift(a, dy, dx):
    """s[..., y, x] = a[..., y+dy, (x+dx) mod W], zero where y+dy is outside."""
    H = a.shape[-2]
    r = np.roll(a, -dx, axis=-1)
    s = np.zeros_like(r)
    if dy >= 0:
        s[..., :H - dy, :] = r[..., dy:, :]
    else:
        s[..., -dy:, :] = r[..., :H + dy, :]
    return s


def _unshift(g, dy, dx):
    """Adjoint of _shift."""
    H = g.shape[-2]
    s = np.zeros_like(g)
    if dy >= 0:
        s[..., dy:, :] = g[..., :H - dy, :]
    else:
        s[..., :H + dy, :] = g[..., -dy:, :]
    return np.roll(s, dx, axis=-1)


def conv(a, k, bias):
    out = np.zeros((a.shape[0], k.shape[0]) + a.shape[2:])
    for ky in range(KH):
        for kx in range(KW):
            out += np.einsum("oc,bcyx->boyx", k[:, :, ky, kx], _shift(a, ky - 1, kx - 2))
    return out + bias[None, :, None, None]


def forward(p, feat, H, W, C1, C2, ND):
    q = unpack(np.asarray(p, np.float64), H, W, C1, C2, ND)
    f = np.asarray(feat, np.float64).reshape(-1, 1, H, W)
    a1 = np.maximum(conv(f, q["w1"], q["b1"]), 0.0)
    a2 = np.maximum(conv(a1, q["w2"], q["b2"]), 0.0)
    h = a2.mean(axis=3).reshape(len(f), C2 * H)
    logits = h @ q["w3"] + q["b3"][None, :]
    return dict(q=q, f=f, a1=a1, a2=a2, h=h, logits=logits)


def loss_grad(p, feat, target, H, W, C1, C2, ND):
    """Mean loss and its gradient with respect to the flat parameters."""
    c = forward(p, feat, H, W, C1, C2, ND)
    q, B = c["q"], len(c["f"])
    t = np.asarray(target, np.float64)
    l = c["logits"]
    m = l.max(axis=1, keepdims=True)
    lse = m[:, 0] + np.log(np.exp(l - m).sum(axis=1))
    loss = float(np.mean((t * (lse[:, None] - l)).sum(axis=1)))
    pr = np.exp(l - lse[:, None])
    dl = (pr * t.sum(axis=1, keepdims=True) - t) / B
    g = {}
    g["w3"] = c["h"].T @ dl
    g["b3"] = dl.sum(axis=0)
    dh = (dl @ q["w3"].T).reshape(B, C2, H, 1)
    d2 = np.broadcast_to(dh / W, c["a2"].shape) * (c["a2"] > 0)
    g["w2"], g["b2"], da1 = _conv_grads(c["a1"], q["w2"], d2)
    d1 = da1 * (c["a1"] > 0)
    g["w1"], g["b1"], _ = _conv_grads(c["f"], q["w1"], d1)
    o = layout(H, W, C1, C2, ND)
    flat = np.zeros(o["n"])
    order = ["w1", "b1", "w2", "b2", "w3", "b3", "n"]
    for k, nxt in zip(order[:-1], order[1:]):
        flat[o[k]:o[nxt]] = g[k].ravel()
    return loss, flat


def _conv_grads(a, k, d):
    gk = np.zeros_like(k)
    da = np.zeros_like(a)
    for ky in range(KH):
        for kx in range(KW):
            s = _shift(a, ky - 1, kx - 2)
            gk[:, :, ky, kx] = np.einsum("boyx,bcyx->oc", d, s)
            da += _unshift(np.einsum("oc,boyx->bcyx", k[:, :, ky, kx], d), ky - 1, kx - 2)
    return gk, d.sum(axis=(0, 2, 3)), da
