"""The CPU restatement of the warm-start network: its analytic gradient
against central finite differences (plain FP64 mode), and its BF16 storage
mode against the FP64 mode."""
import numpy as np
import pytest

from fluidity_gb300 import meshgen as M
from fluidity_gb300.warmstart import init_weights, rotating_source
from oracle import gnn_oracle as G


def _case(n=3, seed=5):
    import scipy.sparse as sp
    nd, X = M.cube_mesh(n)
    N = X.shape[0]
    # first-order pattern of the mesh (node pairs sharing an element)
    r = np.repeat(nd, 4, axis=1).reshape(-1)
    c = np.tile(nd, (1, 4)).reshape(-1)
    A = sp.csr_matrix((np.ones(r.size), (r, c)), shape=(N, N))
    A.sum_duplicates()
    A.sort_indices()
    P = G.graph(A.indptr.astype(np.int64), A.indices.astype(np.int64))
    rng = np.random.default_rng(seed)
    p1 = 1e-3 * rotating_source(X, 3)
    p2 = 1e-3 * rotating_source(X, 2)
    b = rotating_source(X, 4)
    target = 1e-3 * rotating_source(X, 4) + 1e-5 * rng.standard_normal(N)
    mask = (rng.random(N) > 0.2).astype(np.uint8)
    w = init_weights(11).astype(np.float64)
    w[G.OFF_WD:G.OFF_BD] *= 100.0  # a decoder large enough that every layer matters
    w[G.OFF_BE:G.OFF_L] = 0.05 * rng.standard_normal(G.W)
    return w, p1, p2, b, X, P, target, mask


def _laplacian(n):
    """A symmetric positive definite matrix on the mesh graph (graph Laplacian
    plus identity) standing in for the assembled stiffness matrix."""
    import scipy.sparse as sp
    nd, X = M.cube_mesh(n)
    N = X.shape[0]
    r = np.repeat(nd, 4, axis=1).reshape(-1)
    c = np.tile(nd, (1, 4)).reshape(-1)
    A = sp.csr_matrix((np.ones(r.size), (r, c)), shape=(N, N))
    A.data[:] = -1.0
    A = A + sp.diags(-np.asarray(A.sum(axis=1)).ravel() + 1.0)
    return A.tocsr()


@pytest.mark.parametrize("energy", [False, True])
def test_gradient_matches_finite_differences(energy):
    w, p1, p2, b, X, P, target, mask = _case()
    K = _laplacian(3) if energy else None
    loss, g = G.gradients(w, p1, p2, b, X, P, target, mask, rounded=False, K=K)
    rng = np.random.default_rng(3)
    blocks = [(G.OFF_WE, G.OFF_BE), (G.OFF_BE, G.OFF_L), (G.OFF_L, G.OFF_L + 8192),
              (G.OFF_L + G.LAYER_SIZE - 64, G.OFF_L + G.LAYER_SIZE),
              (G.OFF_L + 2 * G.LAYER_SIZE, G.OFF_L + 2 * G.LAYER_SIZE + 8192),
              (G.OFF_WD, G.OFF_BD), (G.OFF_BD, G.NPARAMS)]
    for lo, hi in blocks:
        cand = np.arange(lo, hi)
        cand = cand[np.abs(g[cand]) > 1e-3 * np.abs(g[lo:hi]).max()]
        for k in rng.choice(cand, size=min(4, cand.size), replace=False):
            h = 1e-6 * max(1.0, abs(w[k]))
            wp, wm = w.copy(), w.copy()
            wp[k] += h
            wm[k] -= h
            lp = G.forward(wp, p1, p2, b, X, P, target, mask, rounded=False, K=K)["loss"]
            lm = G.forward(wm, p1, p2, b, X, P, target, mask, rounded=False, K=K)["loss"]
            fd = (lp - lm) / (2 * h)
            assert abs(fd - g[k]) <= 1e-5 * abs(g[k]) + 1e-9 * np.abs(g).max(), (k, fd, g[k])


def test_bf16_storage_stays_close_to_fp64():
    w, p1, p2, b, X, P, target, mask = _case()
    l64, g64 = G.gradients(w, p1, p2, b, X, P, target, mask, rounded=False)
    l16, g16 = G.gradients(w, p1, p2, b, X, P, target, mask, rounded=True)
    assert abs(l16 - l64) <= 2e-2 * l64
    cos = g16 @ g64 / np.linalg.norm(g16) / np.linalg.norm(g64)
    assert cos > 0.99


def test_bf16_rounding_is_nearest_even():
    # bf16 keeps 8 significant bits: ulp(1) = 2^-7; ties go to the even mantissa
    x = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5, 0.0])
    r = G.bf16(x)
    assert list(r) == [1.0, 1.0, 1.0 + 2 ** -6, 1.0 + 2 ** -7, 1.0, -2.5, 0.0]
