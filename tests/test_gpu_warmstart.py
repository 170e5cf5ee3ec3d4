"""The learned warm start on the GPU: forward pass and gradients of the BF16
tensor-core kernels against the CPU restatement of the network, deterministic
training, and the iterations the trained network saves the pressure solve."""
import numpy as np
import pytest

from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M
from fluidity_gb300 import warmstart as WS
from oracle import gnn_oracle as G

pytestmark = pytest.mark.gpu


def _setup(n=6, seed=5):
    import torch
    nd, X = M.cube_mesh(n)
    m = ft.Mesh(nd, X)
    s = m.sparsity()
    P = G.graph(s.findrm.astype(np.int64), s.colm.astype(np.int64))
    rng = np.random.default_rng(seed)
    N = X.shape[0]
    p1 = 1e-3 * WS.rotating_source(X, 3)
    p2 = 1e-3 * WS.rotating_source(X, 2)
    b = WS.rotating_source(X, 4)
    target = 1e-3 * WS.rotating_source(X, 4) + 1e-5 * rng.standard_normal(N)
    mask = (rng.random(N) > 0.2).astype(np.uint8)
    w = WS.init_weights(11)
    w[G.OFF_WD:G.OFF_BD] *= 100.0
    w[G.OFF_BE:G.OFF_L] = (0.05 * rng.standard_normal(G.W)).astype(np.float32)
    net = WS.PressureGuessNet(m)
    net.set_weights(w)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    return m, X, P, net, w.astype(np.float64), (p1, p2, b, target, mask), \
        (d(p1), d(p2), d(b), d(target), d(mask))


def test_forward_matches_oracle():
    m, X, P, net, w, (p1, p2, b, t, mk), (dp1, dp2, db, dt, dm) = _setup()
    pred = net.predict(dp1, dp2, db).cpu().numpy()
    c = G.forward(w, p1, p2, b, X, P, rounded=True)
    ext = 2 * p1 - p2
    # the network's part of the prediction, relative to its own size
    err = np.abs((pred - ext) - (c["pred"] - ext)).max() / np.abs(c["pred"] - ext).max()
    assert err < 1e-2, err


@pytest.mark.parametrize("energy", [False, True])
def test_gradients_match_oracle(energy):
    import scipy.sparse as sp
    import torch
    m, X, P, net, w, (p1, p2, b, t, mk), (dp1, dp2, db, dt, dm) = _setup()
    K = None
    if energy:
        # the loss in the energy norm of the assembled Poisson matrix
        src = torch.from_numpy(M.poisson_source(X)).cuda()
        val, _ = ft.assemble_advection_diffusion_cg(
            m, ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2), source=src)
        net.set_loss(val)
        s = m.sparsity()
        K = sp.csr_matrix((val.cpu().numpy(), s.colm, s.findrm), shape=(m.N, m.N))
    loss, g = net.gradients(dp1, dp2, db, dt, dm)
    lo, go = G.gradients(w, p1, p2, b, X, P, t, mk, rounded=True, K=K)
    assert abs(loss - lo) <= 1e-3 * lo
    blocks = {"We": (G.OFF_WE, G.OFF_BE), "be": (G.OFF_BE, G.OFF_L), "wd": (G.OFF_WD, G.OFF_BD),
              "bd": (G.OFF_BD, G.NPARAMS)}
    for l in range(3):
        o = G.OFF_L + l * G.LAYER_SIZE
        blocks[f"W{l + 1}"] = (o, o + 8192)
        blocks[f"b{l + 1}"] = (o + 8192, o + G.LAYER_SIZE)
    for name, (a, z) in blocks.items():
        rel = np.linalg.norm(g[a:z] - go[a:z]) / np.linalg.norm(go[a:z])
        assert rel < 2e-2, (name, rel)
    # deterministic: the same call gives the same bits
    loss2, g2 = net.gradients(dp1, dp2, db, dt, dm)
    assert loss2 == loss and np.array_equal(g, g2)


def test_training_step_descends_and_is_deterministic():
    import torch
    m, X, P, net, w, host, (dp1, dp2, db, dt, dm) = _setup()
    nact = int(host[4].sum())
    l0, _ = net.gradients(dp1, dp2, db, dt, dm)
    for _ in range(20):
        net.train_step(dp1, dp2, db, dt, dm, nact, lr=1e-3)
    l1, _ = net.gradients(dp1, dp2, db, dt, dm)
    assert l1 < 0.8 * l0
    w1 = net.weights()
    net.set_weights(w.astype(np.float32))
    for _ in range(20):
        net.train_step(dp1, dp2, db, dt, dm, nact, lr=1e-3)
    torch.cuda.synchronize()
    assert np.array_equal(net.weights(), w1)


def test_learned_guess_saves_iterations():
    """Rotating-source sequence on a 12^3 mesh: train on steps 2..79, then CG
    (rtol 1e-10) on the held-out steps 80..99 from the zero, previous-step and
    learned guesses; all reach the same tolerance, the learned guess in the
    fewest iterations."""
    import torch
    nd, X = M.cube_mesh(12)
    m = ft.Mesh(nd, X)
    seq = WS.PoissonSequence(m, X, M.boundary_nodes(X))
    ps, bs = WS.pressure_sequence(seq, 100)
    net = WS.PressureGuessNet(m)
    losses = WS.train(net, ps, bs, seq.mask, seq.nact, range(2, 80), epochs=30, lr=2e-3)
    assert losses[-1] < 0.5 * losses[0]
    opts = ft.solver_options(ksp="cg", rtol=1e-10, max_its=20000)
    its = {"zero": [], "previous": [], "learned": []}
    for t in range(80, 100):
        guesses = {"zero": torch.zeros_like(ps[t]), "previous": ps[t - 1].clone(),
                   "learned": net.predict(ps[t - 1], ps[t - 2], bs[t])}
        for k, x in guesses.items():
            rep = seq.solve(t, x, opts)
            assert rep["reason"] == 2
            assert rep["true_rel_residual"] < 1e-9
            assert torch.allclose(x, ps[t], rtol=0, atol=1e-8 * ps[t].abs().max().item())
            its[k].append(rep["iterations"])
    mean = {k: float(np.mean(v)) for k, v in its.items()}
    assert mean["learned"] < mean["previous"] < mean["zero"], mean
