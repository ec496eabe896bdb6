"""CPU FP64 restatement of the learned emission proposal: network, loss, gradient, lobe table and
mixture density.

TEST INFRASTRUCTURE ONLY: imported by the test suite as the checker of the tensor-core kernels and the
device sampler; the product never imports this module.

No reference counterpart exists (the reference emits uniformly, Classes_Sources.cs:256-265,
390-403); the definitions follow include/pach_proposal.h:

* input x = cond * 0.1 (cond: source xyz, receiver xyz, bounds min xyz, bounds max xyz, metres);
* z_l = h_{l-1} W_l^T + b_l, h_l = GELU(z_l) = z Phi(z) for l = 1..3, out = z_4 (160 = 32 x 5);
* lobe k: mu = u / max(|u|, 1e-6), kappa = exp(clamp(s, -3, 6)), pi = softmax(a);
  vMF density on the 2-sphere f(d) = kappa / (2 pi (1 - e^(-2 kappa))) exp(kappa (mu.d - 1));
* loss of a row = -sum_b p_b log q(d_b) over the 1536 cube-map bin centres d_b, mean over rows.

``emulate_bf16=True`` rounds where the GPU kernels store BF16 (input, weights, hidden activations,
output gradient and hidden-layer gradients as GEMM operands) so that the comparison isolates the
kernels' arithmetic from the intended reduced precision; bias gradients stay unrounded as on the GPU.
"""
from __future__ import annotations

import math

import numpy as np
from scipy.special import erf

N_IN, N_HID, N_OUT, N_LOBES, N_BINS = 12, 256, 160, 32, 1536
LOGK_MIN, LOGK_MAX = -3.0, 6.0
IN_SCALE = 0.1
LAYERS = [(256, 12), (256, 256), (256, 256), (160, 256)]  # (out, in)


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def param_count() -> int:
    return sum(n * k + n for n, k in LAYERS)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    out, i = [], 0
    for n, k in LAYERS:
        W = p[i:i + n * k].reshape(n, k)
        i += n * k
        b = p[i:i + n]
        i += n
        out.append((W, b))
    return out


def pack(layers):
    return np.concatenate([np.concatenate([W.reshape(-1), b]) for W, b in layers])


def gelu(z):
    return 0.5 * z * (1.0 + erf(z / math.sqrt(2.0)))


def gelu_d(z):
    return 0.5 * (1.0 + erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2.0 * math.pi)


def direction_bins():
    """Cube-map bin centres [1536][3] and exact solid angles [1536]: faces +x -x +y -y +z -z, 16 x 16
    cells over the face's other two axes (u, v) in x, y, z order."""
    dirs = np.zeros((N_BINS, 3))
    om = np.zeros(N_BINS)
    F = lambda u, v: math.atan2(u * v, math.sqrt(1.0 + u * u + v * v))
    for f in range(6):
        sg = -1.0 if f & 1 else 1.0
        for j in range(16):
            for i in range(16):
                u0, u1, v0, v1 = i / 8 - 1, (i + 1) / 8 - 1, j / 8 - 1, (j + 1) / 8 - 1
                uc, vc = 0.5 * (u0 + u1), 0.5 * (v0 + v1)
                d = [(sg, uc, vc), (uc, sg, vc), (uc, vc, sg)][f // 2]
                b = f * 256 + j * 16 + i
                dirs[b] = np.asarray(d) / np.linalg.norm(d)
                om[b] = F(u1, v1) - F(u0, v1) - F(u1, v0) + F(u0, v0)
    return dirs, om


def direction_bin(d) -> int:
    x, y, z = (float(c) for c in d)
    ax, ay, az = abs(x), abs(y), abs(z)
    if ax >= ay and ax >= az:
        f, u, v = (0 if x > 0 else 1), y / ax, z / ax
    elif ay >= az:
        f, u, v = (2 if y > 0 else 3), x / ay, z / ay
    else:
        f, u, v = (4 if z > 0 else 5), x / az, y / az
    i = min(15, max(0, int((u + 1) * 8)))
    j = min(15, max(0, int((v + 1) * 8)))
    return f * 256 + j * 16 + i


def lobes(out):
    """Raw outputs [..., 160] -> mu [..., 32, 3], kappa, log pi, log vMF normaliser, |u|, free mask."""
    o = np.asarray(out, dtype=np.float64).reshape(*np.shape(out)[:-1], N_LOBES, 5)
    u = o[..., :3]
    n = np.maximum(np.linalg.norm(u, axis=-1), 1e-6)
    mu = u / n[..., None]
    s = np.clip(o[..., 3], LOGK_MIN, LOGK_MAX)
    kap = np.exp(s)
    a = o[..., 4]
    lpi = a - a.max(axis=-1, keepdims=True)
    lpi = lpi - np.log(np.exp(lpi).sum(axis=-1, keepdims=True))
    lnorm = s - math.log(2 * math.pi) - np.log(-np.expm1(-2 * kap))
    free = ((o[..., 3] > LOGK_MIN) & (o[..., 3] < LOGK_MAX)).astype(float)
    return mu, kap, lpi, lnorm, n, free


def forward(p, cond, emulate_bf16=True):
    rnd = bf16 if emulate_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    L = unpack(p)
    h = rnd(np.asarray(cond, dtype=np.float64) * IN_SCALE)
    cache = {"h": [h], "z": []}
    for l, (W, b) in enumerate(L):
        z = h @ rnd(W).T + b
        if l < 3:
            cache["z"].append(z)
            h = rnd(gelu(z))
            cache["h"].append(h)
        else:
            out = z
    return out, cache


def row_loss_grad(out_row, target_row, bins):
    """Loss of one row and d loss / d out (160)."""
    mu, kap, lpi, lnorm, n, free = lobes(out_row)
    cm = bins @ mu.T - 1.0                          # [B][32]
    x = lpi + lnorm + kap * cm
    mx = x.max(axis=1, keepdims=True)
    e = np.exp(x - mx)
    q = e.sum(axis=1, keepdims=True)
    logq = (mx + np.log(q))[:, 0]
    p = np.asarray(target_row, dtype=np.float64)
    loss = -np.sum(p * logq)
    r = p[:, None] * e / q                          # p_b * responsibility
    R = r.sum(axis=0)
    S = (r * cm).sum(axis=0)
    G = r.T @ bins                                  # [32][3]
    P = p.sum()
    pi = np.exp(lpi)
    dA = pi * P - R
    dK = -(R * (1.0 / kap - 2.0 / np.expm1(2.0 * kap)) + S)
    dS = dK * kap * free
    g = -kap[:, None] * G
    gm = (g * mu).sum(axis=1, keepdims=True)
    dU = (g - gm * mu) / n[:, None]
    d = np.concatenate([dU, dS[:, None], dA[:, None]], axis=1).reshape(-1)
    return loss, d


def loss_grad(p, cond, target, bins=None, emulate_bf16=True):
    """Mean loss and gradient (public parameter order) over the rows."""
    rnd = bf16 if emulate_bf16 else (lambda v: np.asarray(v, dtype=np.float64))
    if bins is None:
        bins = direction_bins()[0]
    bins = np.asarray(bins, dtype=np.float64)
    cond = np.asarray(cond, dtype=np.float64)
    M = cond.shape[0]
    out, cache = forward(p, cond, emulate_bf16)
    loss = 0.0
    dout = np.zeros_like(out)
    for m in range(M):
        l, d = row_loss_grad(out[m], target[m], bins)
        loss += l
        dout[m] = d / M
    L = unpack(p)
    grads = [None] * 4
    dz = dout
    for l in range(3, -1, -1):
        W, b = L[l]
        h_prev = cache["h"][l]
        dzr = rnd(dz)
        grads[l] = (dzr.T @ h_prev, dz.sum(axis=0))
        if l > 0:
            dz = (dzr @ rnd(W)) * gelu_d(cache["z"][l - 1])
    return loss / M, pack(grads)


def lobe_table(out):
    """The tracer's lobe table: per lobe (mu xyz, kappa, log pi + log norm, cumulative pi)."""
    mu, kap, lpi, lnorm, _, _ = lobes(out)
    cdf = np.cumsum(np.exp(lpi), axis=-1)
    cdf[..., -1] = 1.0
    return mu, kap, lpi + lnorm, cdf


def mixture_density(out, d, mix):
    """q(d) of the defensive mixture over the rows of out [n][160] at directions d [m][3]."""
    mu, kap, lw, _ = lobe_table(np.asarray(out).reshape(-1, N_OUT))
    d = np.asarray(d, dtype=np.float64)
    qs = np.zeros(d.shape[0])
    for j in range(mu.shape[0]):
        qs += np.exp(lw[j][None, :] + kap[j][None, :] * (d @ mu[j].T - 1.0)).sum(axis=1)
    return mix / (4 * math.pi) + (1 - mix) * qs / mu.shape[0]
