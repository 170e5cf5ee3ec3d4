"""CPU restatement (numpy, FP64) of the learned-warm-start network.

TEST INFRASTRUCTURE ONLY: imported by ``tests/`` as the checker of the GPU
network's forward pass and gradients -- never by the product package.

The network and its parameter layout are this project's own definition (the
reference has no learned component); the formulas below restate it:

    f_i  = [p1_i/s, p2_i/s, b_i/sb, 2x_i-1, 2y_i-1, 2z_i-1, 0 x 10]
    h0   = relu(We f + be)
    h_l  = h_{l-1} + relu(Wl [h_{l-1} ; mean_{j in N(i), j != i} h_{l-1,j}] + bl)
    pred = 2 p1 - p2 + s (wd . h_3 + bd)
    loss = mean over active nodes of ((pred - target) / s)^2, or, given the
           matrix K, e^T K e / (number of active nodes) with e the normalised
           error on the active nodes (zero elsewhere)

``rounded=True`` reproduces the GPU's storage precision: weights, features,
activations (h, a, z) and the layer gradients fed to the tensor cores (dz) are
rounded to bfloat16 (round to nearest even) at the same points, everything
else is exact FP64.  ``rounded=False`` is the plain FP64 network, whose
gradient is pinned against central finite differences in the CPU tests.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

W = 64
F = 16
LAYERS = 3
OFF_WE = 0
OFF_BE = OFF_WE + W * F
OFF_L = OFF_BE + W
LAYER_SIZE = W * 2 * W + W
OFF_WD = OFF_L + LAYERS * LAYER_SIZE
OFF_BD = OFF_WD + W
NPARAMS = OFF_BD + 1


def bf16(x):
    """Round to bfloat16 (nearest even) through float32; returned as float64."""
    f = np.ascontiguousarray(np.asarray(x, dtype=np.float64).astype(np.float32))
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + np.uint64(0x7FFF) + ((u >> np.uint64(16)) & np.uint64(1))) >> np.uint64(16)) << np.uint64(16)
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params):
    p = np.asarray(params, dtype=np.float64)
    out = {"We": p[OFF_WE:OFF_BE].reshape(W, F), "be": p[OFF_BE:OFF_L]}
    for l in range(LAYERS):
        o = OFF_L + l * LAYER_SIZE
        out[f"W{l + 1}"] = p[o:o + 2 * W * W].reshape(W, 2 * W)
        out[f"b{l + 1}"] = p[o + 2 * W * W:o + LAYER_SIZE]
    out["wd"] = p[OFF_WD:OFF_BD]
    out["bd"] = p[OFF_BD:OFF_BD + 1]
    return out


def pack(d):
    p = np.zeros(NPARAMS)
    p[OFF_WE:OFF_BE] = d["We"].reshape(-1)
    p[OFF_BE:OFF_L] = d["be"]
    for l in range(LAYERS):
        o = OFF_L + l * LAYER_SIZE
        p[o:o + 2 * W * W] = d[f"W{l + 1}"].reshape(-1)
        p[o + 2 * W * W:o + LAYER_SIZE] = d[f"b{l + 1}"]
    p[OFF_WD:OFF_BD] = d["wd"]
    p[OFF_BD] = d["bd"][0]
    return p


def graph(findrm, colm):
    """Neighbour-mean operator P (P[i, j] = 1/deg_i for j in row i, j != i)."""
    n = len(findrm) - 1
    rows = np.repeat(np.arange(n), np.diff(findrm))
    keep = colm != rows
    deg = np.diff(findrm) - 1
    inv = np.where(deg > 0, (1.0 / np.maximum(deg, 1).astype(np.float32)).astype(np.float32), 0.0)
    P = sp.csr_matrix((inv[rows[keep]].astype(np.float64), (rows[keep], colm[keep])), shape=(n, n))
    return P


def forward(params, p1, p2, b, X, P, target=None, mask=None, rounded=True, K=None):
    R = bf16 if rounded else (lambda v: np.asarray(v, dtype=np.float64))
    q = unpack(params)
    n = p1.size
    feat = np.zeros((n, F))
    if rounded:
        # FP32: the values rounded to float times the float reciprocal of the scale
        s = float(np.float32(np.max(np.abs(p1)))) or 1.0
        sb = float(np.float32(np.max(np.abs(b)))) or 1.0
        f32 = lambda v: np.asarray(v, dtype=np.float32).astype(np.float64)
        i_s, i_sb = np.float32(1.0) / np.float32(s), np.float32(1.0) / np.float32(sb)
        feat[:, 0] = (np.asarray(p1, np.float32) * i_s).astype(np.float64)
        feat[:, 1] = (np.asarray(p2, np.float32) * i_s).astype(np.float64)
        feat[:, 2] = (np.asarray(b, np.float32) * i_sb).astype(np.float64)
    else:
        s = float(np.max(np.abs(p1))) or 1.0
        sb = float(np.max(np.abs(b))) or 1.0
        f32 = lambda v: np.asarray(v, dtype=np.float64)
        feat[:, 0] = p1 / s
        feat[:, 1] = p2 / s
        feat[:, 2] = b / sb
    feat[:, 3:6] = f32(2.0 * X - 1.0)
    Fm = R(feat)
    c = {"s": s, "F": Fm, "H": [], "Z": [], "A": [], "X": []}
    z = Fm @ R(q["We"]).T + q["be"]
    c["Z"].append(R(z))
    H = R(np.maximum(z, 0.0))
    c["H"].append(H)
    for l in range(1, LAYERS + 1):
        A = R(P @ H)
        Xl = np.hstack([H, A])
        z = Xl @ R(q[f"W{l}"]).T + q[f"b{l}"]
        c["A"].append(A)
        c["X"].append(Xl)
        c["Z"].append(R(z))
        H = R(H + np.maximum(z, 0.0))
        c["H"].append(H)
    o = H @ R(q["wd"]) + q["bd"][0]
    ext = 2.0 * p1 - p2
    c["o"] = o
    c["pred"] = ext + s * o
    if target is not None:
        act = np.ones(n, bool) if mask is None else mask.astype(bool)
        e = np.where(act, (ext - target) / s + o, 0.0)
        c["e"] = e
        c["nact"] = int(act.sum())
        if K is None:
            c["ge"] = 2.0 * e
            c["loss"] = float(np.sum(e * e) / c["nact"])
        else:
            Ke = np.where(act, K @ e, 0.0)
            c["ge"] = 2.0 * Ke
            c["loss"] = float(e @ Ke / c["nact"])
    return c


def gradients(params, p1, p2, b, X, P, target, mask=None, rounded=True, K=None):
    """(loss, flat gradient) of the loss with respect to the FP32 parameters."""
    R = bf16 if rounded else (lambda v: np.asarray(v, dtype=np.float64))
    q = unpack(params)
    c = forward(params, p1, p2, b, X, P, target, mask, rounded, K)
    g = {}
    go = c["ge"] / c["nact"]
    H3 = c["H"][LAYERS]
    wd = R(q["wd"])
    g["wd"] = H3.T @ go
    g["bd"] = np.array([go.sum()])
    dH = go[:, None] * wd[None, :]
    for l in range(LAYERS, 0, -1):
        dZ = R(dH * (c["Z"][l] > 0))
        Wl = R(q[f"W{l}"])
        dX = dZ @ Wl
        g[f"W{l}"] = dZ.T @ c["X"][l - 1]
        g[f"b{l}"] = dZ.sum(axis=0)
        dH = dH + dX[:, :W] + P.T @ dX[:, W:]
    dZ0 = R(dH * (c["Z"][0] > 0))
    g["We"] = dZ0.T @ c["F"]
    g["be"] = dZ0.sum(axis=0)
    return c["loss"], pack(g)
