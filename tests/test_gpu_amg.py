"""The smoothed-aggregation AMG preconditioner: CG with it reaches the same
tolerance as Jacobi CG on the Dirichlet Poisson systems, agrees with a
direct solve, is deterministic, and needs far fewer iterations."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu


def _system(n, degree=1, kappa=1.0):
    import torch
    nd, X = M.cube_mesh(n)
    if degree == 2:
        nd2, n2 = ft.make_global_numbering_p2(nd)
        Xf = M.p2_coordinates(nd, nd2, X, M.P2_COUNTS)
        m = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
        q = 4
    else:
        Xf, m, q = X, ft.Mesh(nd, X), 2
    p = ft.advdif_params(diffusivity=kappa, have_source=True, quad_degree=q)
    src = torch.from_numpy(M.poisson_source(Xf)).cuda()
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, source=src)
    bn = M.boundary_nodes(Xf)
    ina = torch.zeros(m.N, dtype=torch.uint8, device="cuda")
    g = torch.from_numpy(np.linspace(0.0, 0.1, bn.size)).cuda()
    ft.apply_dirichlet_conditions(m, rhs, ina, torch.from_numpy(bn).cuda(), g, dt=1.0)
    return m, val, rhs, ina


def _direct(m, val, rhs, ina):
    s = m.sparsity()
    v, b, g = val.cpu().numpy(), rhs.cpu().numpy(), ina.cpu().numpy()
    A = sp.csr_matrix((v, s.colm, s.findrm), shape=(m.N, m.N))
    act, gh = np.nonzero(g == 0)[0], np.nonzero(g)[0]
    x = b.copy()
    x[act] = spla.spsolve(A[act][:, act].tocsc(), b[act] - A[act][:, gh] @ b[gh])
    return x


@pytest.mark.parametrize("degree,n,kappa", [(1, 16, 1.0), (1, 12, np.diag([1.0, 1.0, 1e-3])), (2, 6, 1.0)])
def test_amg_cg_matches_direct_and_jacobi(degree, n, kappa):
    import torch
    m, val, rhs, ina = _system(n, degree, kappa)
    opts = ft.solver_options(ksp="cg", rtol=1e-10)
    xj = torch.zeros(m.N, dtype=torch.float64, device="cuda")
    rj = ft.petsc_solve(m, xj, val, rhs, opts, inactive=ina)
    amg = ft.AmgPreconditioner(m, val, ina)
    lv = amg.levels()
    assert lv[0][0] == m.N and len(lv) >= 2 and all(a[0] > b[0] for a, b in zip(lv, lv[1:]))
    x = torch.zeros(m.N, dtype=torch.float64, device="cuda")
    r = amg.solve(x, rhs, opts)
    assert r["reason"] == 2 and rj["reason"] == 2
    assert r["true_rel_residual"] < 1e-9
    assert r["iterations"] * 3 < rj["iterations"], (r["iterations"], rj["iterations"])
    xd = _direct(m, val, rhs, ina)
    xh = x.cpu().numpy()
    assert np.abs(xh - xd).max() <= 1e-7 * np.abs(xd).max()
    g = ina.cpu().numpy() == 1
    assert np.array_equal(xh[g], rhs.cpu().numpy()[g])
    amg.close()


def test_amg_is_deterministic_and_reusable():
    import torch
    m, val, rhs, ina = _system(10)
    opts = ft.solver_options(ksp="cg", rtol=1e-10)
    a1, a2 = ft.AmgPreconditioner(m, val, ina), ft.AmgPreconditioner(m, val, ina)
    assert a1.levels() == a2.levels()
    x1 = torch.zeros(m.N, dtype=torch.float64, device="cuda")
    x2 = torch.zeros_like(x1)
    r1, r2 = a1.solve(x1, rhs, opts), a2.solve(x2, rhs, opts)
    assert r1["iterations"] == r2["iterations"] and torch.equal(x1, x2)
    # a second rhs on the same hierarchy, from a nonzero guess
    rhs2 = rhs * 2.0
    x3 = x1 * 2.0 + 1e-3
    r3 = a1.solve(x3, rhs2, opts)
    assert r3["reason"] == 2 and r3["true_rel_residual"] < 1e-9
    assert torch.allclose(x3, 2.0 * x1, rtol=0, atol=1e-7 * x1.abs().max().item())
    # iteration limit
    x4 = torch.zeros_like(x1)
    r4 = a1.solve(x4, rhs, ft.solver_options(ksp="cg", rtol=1e-15, max_its=3))
    assert r4["reason"] == -3 and r4["iterations"] == 3
    a1.close()
    a2.close()


def test_amg_unpreconditioned_norm_bounds_the_true_residual():
    import torch
    m, val, rhs, ina = _system(14)
    amg = ft.AmgPreconditioner(m, val, ina, unpreconditioned_norm=True)
    for guess in ("zero", "nonzero"):
        x = torch.zeros(m.N, dtype=torch.float64, device="cuda")
        if guess == "nonzero":
            x += 0.01
        r = amg.solve(x, rhs, ft.solver_options(ksp="cg", rtol=1e-10))
        assert r["reason"] == 2
        assert r["true_rel_residual"] <= 1.5e-10, r
    amg.close()


def test_amg_fp32_cycle():
    """A single-precision V-cycle inside the FP64 CG reaches the same FP64
    tolerance and solution."""
    import torch
    m, val, rhs, ina = _system(14)
    opts = ft.solver_options(ksp="cg", rtol=1e-10)
    amg = ft.AmgPreconditioner(m, val, ina, unpreconditioned_norm=True)
    x64 = torch.zeros(m.N, dtype=torch.float64, device="cuda")
    r64 = amg.solve(x64, rhs, opts)
    amg.set_precision(True)
    x32 = torch.zeros_like(x64)
    r32 = amg.solve(x32, rhs, opts)
    assert r32["reason"] == 2 and r32["true_rel_residual"] <= 1.5e-10
    assert r32["iterations"] <= 1.3 * r64["iterations"] + 2
    assert torch.allclose(x32, x64, rtol=0, atol=1e-8 * x64.abs().max().item())
    # and back to FP64: the same bits as before
    amg.set_precision(False)
    x = torch.zeros_like(x64)
    amg.solve(x, rhs, opts)
    assert torch.equal(x, x64)
    amg.close()
