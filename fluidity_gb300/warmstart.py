"""Learned initial guess for sequences of pressure (Poisson) solves.

``PressureGuessNet`` wraps the fl_gnn_* entry points: a three-layer
message-passing network over the mesh's sparsity graph that predicts the next
pressure from the previous two, the right-hand side and the coordinates, with
its own BF16 tensor-core forward and backward kernels and an Adam step on the
GPU.  ``rotating_source`` and ``pressure_sequence`` generate the training
sequence: Poisson solves whose source is a Gaussian blob circling the centre
of the cube.  The solver always runs to its tolerance from the network's
guess, so the network only changes how many iterations that takes.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from . import femtools as ft
from . import meshgen as M
from ._lib import check

SEED_NET = 20261207


def _ptr(a):
    return None if a is None else a.data_ptr()


class PressureGuessNet:
    """The network of one P1 mesh; parameters live on the GPU (FP32 masters)."""

    def __init__(self, mesh: ft.Mesh, seed: int = SEED_NET):
        self.lib = _lib.load()
        self.mesh = mesh
        self.nparams = int(self.lib.fl_gnn_num_params())
        h = C.c_void_p()
        check(self.lib.fl_gnn_create(mesh.handle, C.byref(h)), "fl_gnn_create")
        self.handle = h.value
        self.set_weights(init_weights(seed, self.nparams))

    # parameters ------------------------------------------------------------
    def set_weights(self, w):
        w = np.ascontiguousarray(w, dtype=np.float32)
        assert w.size == self.nparams
        check(self.lib.fl_gnn_set_weights(self.handle, w.ctypes.data, self.nparams), "fl_gnn_set_weights")

    def weights(self) -> np.ndarray:
        w = np.empty(self.nparams, dtype=np.float32)
        check(self.lib.fl_gnn_get_weights(self.handle, w.ctypes.data, self.nparams), "fl_gnn_get_weights")
        return w

    def set_loss(self, val=None):
        """None: mean squared error; a device tensor of matrix values: the
        energy norm of the error in that matrix (kept referenced)."""
        self._kval = val
        check(self.lib.fl_gnn_set_loss(self.handle, _ptr(val)), "fl_gnn_set_loss")

    # compute ---------------------------------------------------------------
    def predict(self, p1, p2, b, out=None, stream=None):
        import torch
        if out is None:
            out = torch.empty_like(p1)
        check(self.lib.fl_gnn_predict(self.handle, _ptr(p1), _ptr(p2), _ptr(b), _ptr(out),
                                      ft._stream_ptr(stream)), "fl_gnn_predict")
        return out

    def gradients(self, p1, p2, b, target, mask=None, stream=None):
        g = np.empty(self.nparams, dtype=np.float32)
        loss = C.c_float()
        nact = int(mask.sum().item()) if mask is not None else 0
        check(self.lib.fl_gnn_gradients(self.handle, _ptr(p1), _ptr(p2), _ptr(b), _ptr(target),
                                        _ptr(mask), nact, g.ctypes.data, C.byref(loss),
                                        ft._stream_ptr(stream)), "fl_gnn_gradients")
        return float(loss.value), g

    def train_step(self, p1, p2, b, target, mask=None, nact=None, lr=1e-3, loss_out=None,
                   stream=None):
        if mask is not None and nact is None:
            nact = int(mask.sum().item())
        check(self.lib.fl_gnn_train_step(self.handle, _ptr(p1), _ptr(p2), _ptr(b), _ptr(target),
                                         _ptr(mask), int(nact or 0), C.c_float(lr), _ptr(loss_out),
                                         ft._stream_ptr(stream)), "fl_gnn_train_step")

    def close(self):
        if self.handle:
            self.lib.fl_gnn_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def init_weights(seed: int = SEED_NET, nparams: int | None = None) -> np.ndarray:
    """Seeded initial parameters: uniform(-a, a) weights with a = sqrt(6 / fan_in)
    (encoder fan-in 6: the padding columns are zero), residual branches scaled
    by 1/2, decoder weights 1e-2 / 8, zero biases."""
    W, F, L = 64, 16, 3
    n = nparams or (W * F + W + L * (2 * W * W + W) + W + 1)
    u = 2.0 * M.uniform01(seed, n) - 1.0
    w = np.zeros(n)
    o = 0
    we = u[o:o + W * F].reshape(W, F) * np.sqrt(6.0 / 6.0)
    we[:, 6:] = 0.0
    w[o:o + W * F] = we.reshape(-1)
    o += W * F + W
    for _ in range(L):
        w[o:o + 2 * W * W] = 0.5 * np.sqrt(6.0 / (2 * W)) * u[o:o + 2 * W * W]
        o += 2 * W * W + W
    w[o:o + W] = 1e-2 / 8.0 * u[o:o + W]
    return w.astype(np.float32)


# ------------------------------------------------------------- the sequence --
def rotating_source(X, step, period=60, radius=0.25, width=0.02):
    """b = exp(-|x - c(t)|^2 / width), c(t) on a circle of the given radius in
    the plane z = 1/2 about the cube's centre, one revolution per period steps."""
    a = 2.0 * np.pi * step / period
    c = np.array([0.5 + radius * np.cos(a), 0.5 + radius * np.sin(a), 0.5])
    d = X - c[None, :]
    return np.exp(-np.sum(d * d, axis=1) / width)


class PoissonSequence:
    """P1 Poisson systems K p = M b (Dirichlet 0) for the rotating source on one
    mesh: the matrix is assembled once, the right-hand side per step."""

    def __init__(self, mesh: ft.Mesh, X, bnodes, stream=None):
        import torch
        self.mesh, self.X, self.stream = mesh, X, stream
        dev = torch.device("cuda")
        self.dev = dev
        self.params = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
        self.bn = torch.as_tensor(bnodes, dtype=torch.int32, device=dev)
        self.g = torch.zeros(len(bnodes), dtype=torch.float64, device=dev)
        self.mask = torch.ones(mesh.N, dtype=torch.uint8, device=dev)
        self.mask[self.bn.long()] = 0
        self.nact = int(mesh.N - len(bnodes))
        self.val = torch.empty(mesh.nnz, dtype=torch.float64, device=dev)
        self.rhs = torch.empty(mesh.N, dtype=torch.float64, device=dev)
        self.ina = torch.zeros(mesh.N, dtype=torch.uint8, device=dev)

    def source(self, step):
        import torch
        return torch.from_numpy(rotating_source(self.X, step)).to(self.dev)

    def system(self, step, src=None):
        """Assembled matrix and rhs of the step (the matrix does not change)."""
        src = self.source(step) if src is None else src
        ft.assemble_advection_diffusion_cg(self.mesh, self.params, source=src, val=self.val,
                                           rhs=self.rhs, stream=self.stream)
        self.ina.zero_()
        ft.apply_dirichlet_conditions(self.mesh, self.rhs, self.ina, self.bn, self.g, dt=1.0,
                                      stream=self.stream)
        return self.val, self.rhs, self.ina

    def solve(self, step, x, options, src=None):
        val, rhs, ina = self.system(step, src)
        rep = ft.petsc_solve(self.mesh, x, val, rhs, options, inactive=ina, stream=self.stream)
        return rep


def pressure_sequence(seq: PoissonSequence, nsteps: int, rtol=1e-10):
    """Solves of steps 0..nsteps-1 (each from the previous solution) and their
    right-hand sides b = M f: lists of device tensors."""
    import torch
    opts = ft.solver_options(ksp="cg", rtol=rtol, max_its=20000)
    ps, bs = [], []
    x = torch.zeros(seq.mesh.N, dtype=torch.float64, device=seq.dev)
    for t in range(nsteps):
        seq.solve(t, x, opts)
        ps.append(x.clone())
        bs.append(seq.rhs.clone())
    return ps, bs


def train(net: PressureGuessNet, ps, bs, mask, nact, steps, *, epochs=20, lr=2e-3,
          lr_final=1e-4, stream=None, seed=SEED_NET, kval=None):
    """Adam over the samples (p[t-1], p[t-2], b[t]) -> p[t] for t in `steps`,
    in a seeded shuffled order per epoch, cosine learning-rate decay; the loss
    is the energy norm of the error in the matrix `kval` when given, else the
    mean squared error.  Returns the mean loss of each epoch."""
    import torch
    net.set_loss(kval)
    steps = list(steps)
    total = epochs * len(steps)
    loss_dev = torch.zeros(total, dtype=torch.float32, device=ps[0].device)
    k = 0
    for ep in range(epochs):
        order = np.argsort(M.uniform01(seed + ep, len(steps)))
        for j in order:
            t = steps[j]
            a = k / max(1, total - 1)
            rate = lr_final + 0.5 * (lr - lr_final) * (1.0 + np.cos(np.pi * a))
            net.train_step(ps[t - 1], ps[t - 2], bs[t], ps[t], mask, nact, rate,
                           loss_out=loss_dev[k:k + 1], stream=stream)
            k += 1
    per = (loss_dev.view(epochs, len(steps)).double() / nact).mean(dim=1)
    return per.cpu().numpy()
