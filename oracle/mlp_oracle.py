"""CPU oracle of the surrogate network (TEST INFRASTRUCTURE ONLY).

FP64 numpy forward and backward of the network that meshlib_gb300/csrc/mlp_net.cu trains, with
the same rounding points as the GPU: features, weights of the four hidden layers, hidden
activations and the activation gradients fed to the tensor-core GEMMs are rounded to bf16
(round to nearest even); everything else is FP64.  Parameter layout: W1[128x192] b1 W2 b2 W3 b3
W4 b4 w5[128] b5; metadata: centre xyz, scale, 32 frequencies, target clamp, margin, band.
"""
from __future__ import annotations

import numpy as np

F, H = 192, 128
SIZES = [("W1", (H, F)), ("b1", (H,)), ("W2", (H, H)), ("b2", (H,)), ("W3", (H, H)), ("b3", (H,)),
         ("W4", (H, H)), ("b4", (H,)), ("w5", (H,)), ("b5", (1,))]


def unpack(params):
    out, o = {}, 0
    for name, shp in SIZES:
        n = int(np.prod(shp))
        out[name] = np.asarray(params[o:o + n], np.float64).reshape(shp)
        o += n
    assert o == len(params)
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], np.float64).ravel() for name, _ in SIZES])


def bf16(x):
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    b = a.view(np.uint32).astype(np.uint64)
    b = ((b + 0x7FFF + ((b >> 16) & 1)) >> 16) << 16
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def features(pts, meta):
    c = np.asarray(meta[:3], np.float32)
    s = np.float32(meta[3])
    freq = np.asarray(meta[4:36], np.float32)
    u = ((np.asarray(pts, np.float32) - c) * s).astype(np.float32)
    out = np.zeros((len(pts), F))
    for a in range(3):
        arg = (freq[None, :] * u[:, a:a + 1]).astype(np.float32).astype(np.float64)
        out[:, 64 * a + 0:64 * a + 64:2] = np.sin(arg)
        out[:, 64 * a + 1:64 * a + 64:2] = np.cos(arg)
    return bf16(out)


def silu(z):
    return z / (1 + np.exp(-z))


def silu_grad(z):
    s = 1 / (1 + np.exp(-z))
    return s * (1 + z * (1 - s))


def loss_and_grads(params, meta, pts, targets):
    """Mean squared error against targets clamped to +-meta[36] and its parameter gradients."""
    P = unpack(params)
    n = len(pts)
    f = features(pts, meta)
    Ws = [bf16(P["W1"]), bf16(P["W2"]), bf16(P["W3"]), bf16(P["W4"])]
    bs = [P["b1"], P["b2"], P["b3"], P["b4"]]
    acts, zs = [f], []
    for W, b in zip(Ws, bs):
        z = acts[-1] @ W.T + b
        zs.append(z)
        acts.append(bf16(silu(z)))
    y = acts[-1] @ P["w5"] + P["b5"][0]
    t = np.clip(np.asarray(targets, np.float64), -meta[36], meta[36])
    r = y - t
    loss = float((r * r).mean())
    g = 2 * r / n
    G = {"w5": acts[-1].T @ g, "b5": np.array([g.sum()])}
    gz = np.outer(g, P["w5"]) * silu_grad(zs[3])
    G["b4"] = gz.sum(0)
    dz = bf16(gz)
    for l in range(3, -1, -1):
        G["W" + str(l + 1)] = dz.T @ acts[l]
        if l == 0:
            break
        gz = (dz @ Ws[l]) * silu_grad(zs[l - 1])
        G["b" + str(l)] = gz.sum(0)
        dz = bf16(gz)
    return loss, pack(G)


def predict(params, meta, pts):
    P = unpack(params)
    h = features(pts, meta)
    for W, b in [(P["W1"], P["b1"]), (P["W2"], P["b2"]), (P["W3"], P["b3"]), (P["W4"], P["b4"])]:
        h = bf16(silu(h @ bf16(W).T + b))
    return h @ P["w5"] + P["b5"][0]
