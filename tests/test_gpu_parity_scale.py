"""Parity with the oracle at the benchmark sizes, not only on small meshes.

* the 128^3 six-tet cube (12,582,912 P1 tets): first-order sparsity and CG1
  colouring bit-exact; the P1 Poisson system (isotropic, and the anisotropic
  diffusivity diag(1, 1, 1e-3)) within 1e-12 row-scaled;
* the 64^3 P2 Poisson system (1,572,864 tets, 2,146,689 nodes): P2 numbering
  and sparsity bit-exact, entries within 1e-12 row-scaled;
* the advection-diffusion workload at its configured 16^3, ten steps of
  GMRES(30) + Jacobi, against the oracle after every step;
* members of a batch (a tracer on the shared 64^3 mesh, a Poisson member on
  the smallest uneven mesh) against the oracle's assembly and solve.

Tolerances: assembled entries |a - a_ref| <= 1e-12 max_j |a_ref(i, j)|,
rhs within 1e-12 of max |rhs_ref|; solutions at rtol 1e-10 within 1e-7 of
max |x_ref| (both solves stop at the same relative residual, not at the same
vector); integer arrays equal.
"""
import numpy as np
import pytest

from conftest import row_scaled_error
from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def cube128(O):
    nd, X = M.cube_mesh(128)
    m = ft.Mesh(nd, X)
    f, c, ce = O.make_sparsity(nd)
    ocol, ncol = O.colour_cg1(nd)
    yield nd, X, m, (f, c, ce), (ocol, ncol)
    m.close()


def test_sparsity_and_colouring_bit_exact_128(cube128, O):
    nd, X, m, (f, c, ce), (ocol, ncol) = cube128
    sp = m.sparsity()
    assert sp.nnz == 31_802_497 and m.E == 12_582_912 and m.N == 2_146_689
    assert np.array_equal(sp.findrm, f)
    assert np.array_equal(sp.colm, c)
    assert np.array_equal(sp.centrm, ce)
    col, ptr, el = m.colouring()
    assert m.ncolours == ncol
    assert np.array_equal(col, ocol)
    optr, oel = O.colour_sets(ocol, ncol)
    assert np.array_equal(ptr, optr) and np.array_equal(el, oel)


@pytest.mark.parametrize("kappa", ["isotropic", "anisotropic"])
def test_p1_poisson_assembly_128_matches_oracle(cube128, O, kappa):
    import torch
    nd, X, m, (f, c, _), (ocol, ncol) = cube128
    K = 1.0 if kappa == "isotropic" else np.diag([1.0, 1.0, 1e-3])
    src = M.poisson_source(X)
    oval, orhs, st = O.assemble_advdif(ndglno_t=nd, nt=X.shape[0], ndglno_x=nd, coords=X, findrm=f,
                                       colm=c, diffusivity=K, source=src,
                                       colours=O.colour_sets(ocol, ncol))
    assert st == 0
    p = ft.advdif_params(diffusivity=K, have_source=True, quad_degree=2)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, source=torch.from_numpy(src).cuda())
    torch.cuda.synchronize()
    val, rhs = val.cpu().numpy(), rhs.cpu().numpy()
    assert row_scaled_error(val, oval, f) <= TOL
    assert np.abs(rhs - orhs).max() <= TOL * np.abs(orhs).max()


def test_p2_poisson_64_matches_oracle(O):
    import torch
    nd, X = M.cube_mesh(64)
    nd2, n2 = ft.make_global_numbering_p2(nd)
    ond2, on2 = O.make_global_numbering_p2(nd)
    assert n2 == on2 == 2_146_689 and np.array_equal(nd2, ond2)
    X2 = M.p2_coordinates(nd, nd2, X, M.P2_COUNTS)
    m = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    sp = m.sparsity()
    f, c, ce = O.make_sparsity(nd2, n2)
    assert sp.nnz == 60_859_905
    assert np.array_equal(sp.findrm, f) and np.array_equal(sp.colm, c) and np.array_equal(sp.centrm, ce)
    ocol, ncol = O.colour_cg1(nd)
    src = M.poisson_source(X2)
    oval, orhs, st = O.assemble_advdif(ndglno_t=nd2, nt=n2, ndglno_x=nd, coords=X, findrm=f, colm=c,
                                       diffusivity=1.0, source=src, colours=O.colour_sets(ocol, ncol),
                                       quad_degree=4, t_degree=2)
    assert st == 0
    p = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=4)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, source=torch.from_numpy(src).cuda())
    torch.cuda.synchronize()
    val, rhs = val.cpu().numpy(), rhs.cpu().numpy()
    assert row_scaled_error(val, oval, f) <= TOL
    assert np.abs(rhs - orhs).max() <= TOL * np.abs(orhs).max()
    m.close()


def test_advdif_ten_steps_16_matches_oracle(O):
    """The CPU-runnable workload at its configured size: 16^3, theta 0.5,
    dt 0.01, ten steps of GMRES(30) + Jacobi to 1e-10; the GPU driver and the
    oracle agree after every step, with the same iteration counts (+-1)."""
    nd, X = M.cube_mesh(16)
    m = ft.Mesh(nd, X)
    s = m.sparsity()
    u = M.advdif_velocity(X)
    bn = M.boundary_nodes(X)
    T = M.gaussian_tracer(X)
    To = T.copy()
    p = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True, diffusivity=1e-3)
    opts = ft.solver_options(ksp="gmres", restart=30, rtol=1e-10, start_from_zero=True)
    ocol, ncol = O.colour_cg1(nd)
    cs = O.colour_sets(ocol, ncol)
    for step in range(10):
        T, rep = ft.solve_field_equation_cg(m, T, p, opts, bc_nodes=bn, bc_values=np.zeros(bn.size),
                                            velocity=u)
        assert rep["reason"] == 2
        val, rhs, st = O.assemble_advdif(ndglno_t=nd, nt=m.N, ndglno_x=nd, coords=X,
                                         findrm=s.findrm, colm=s.colm, theta=0.5, dt=0.01,
                                         have_mass=True, velocity=u, T=To, diffusivity=1e-3,
                                         colours=cs)
        assert st == 0
        ina = np.zeros(m.N, dtype=np.uint8)
        O.apply_dirichlet(bn, np.zeros(bn.size), To, 0.01, rhs, ina)
        dx, its, reason, _ = O.petsc_solve(s.findrm.astype(np.int64), s.colm, val, ina, rhs,
                                           ksp="gmres", restart=30, rtol=1e-10)
        assert reason == 2 and abs(its - rep["iterations"]) <= 1, (step, its, rep["iterations"])
        To = To + 0.01 * dx
        assert np.abs(T - To).max() <= 1e-9 * np.abs(To).max(), step
    m.close()


def test_batch_members_match_oracle(O):
    """A batch of the benchmark's first tracer on the shared 64^3 mesh and the
    Poisson member on the n=24 uneven mesh: each member's assembled system and
    solution against the oracle's assembly, Dirichlet rows and solve."""
    import torch
    kap, sc = M.batch_tracer_params(1)
    nd, X = M.cube_mesh(64)
    shared = ft.Mesh(nd, X)
    T0 = M.gaussian_tracer(X)
    u = sc[0] * M.advdif_velocity(X)
    pt = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True, diffusivity=float(kap[0]))
    ndi, Xi = M.batch_mesh(0)
    mi = ft.Mesh(ndi, Xi)
    pp = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
    b = ft.Batch()
    bn, bni = M.boundary_nodes(X), M.boundary_nodes(Xi)
    r_t = b.add(shared, pt, ft.solver_options(ksp="gmres", restart=30, rtol=1e-10, max_its=10000),
                bc_nodes=bn, bc_values=np.zeros(bn.size), t=torch.from_numpy(T0).cuda(),
                velocity=torch.from_numpy(u).cuda())
    r_p = b.add(mi, pp, ft.solver_options(ksp="cg", rtol=1e-10, max_its=20000), bc_nodes=bni,
                bc_values=np.zeros(bni.size), source=torch.from_numpy(M.poisson_source(Xi)).cuda())
    reps = b.run()
    torch.cuda.synchronize()
    assert all(r["reason"] == 2 for r in reps), reps
    cases = ((shared, nd, X, bn, r_t, reps[0], "gmres",
              dict(theta=0.5, dt=0.01, have_mass=True, velocity=u, T=T0, diffusivity=float(kap[0]))),
             (mi, ndi, Xi, bni, r_p, reps[1], "cg",
              dict(diffusivity=1.0, source=M.poisson_source(Xi))))
    for m, ndm, Xm, bnm, reg, rep, ksp, kw in cases:
        f, c, _ = O.make_sparsity(ndm)
        ocol, ncol = O.colour_cg1(ndm)
        oval, orhs, st = O.assemble_advdif(ndglno_t=ndm, nt=Xm.shape[0], ndglno_x=ndm, coords=Xm, findrm=f,
                                           colm=c, colours=O.colour_sets(ocol, ncol), **kw)
        assert st == 0
        ina = np.zeros(Xm.shape[0], dtype=np.uint8)
        O.apply_dirichlet(bnm, np.zeros(bnm.size), kw.get("T"), kw.get("dt", 1.0), orhs, ina)
        assert row_scaled_error(reg["val"].cpu().numpy(), oval, f) <= TOL
        assert np.abs(reg["rhs"].cpu().numpy() - orhs).max() <= TOL * np.abs(orhs).max()
        assert np.array_equal(reg["inactive"].cpu().numpy(), ina)
        ox, its, reason, _ = O.petsc_solve(f, c, oval, ina, orhs, ksp=ksp, restart=30, rtol=1e-10,
                                           max_its=20000)
        assert reason == 2 and abs(its - rep["iterations"]) <= 1, (ksp, its, rep["iterations"])
        x = reg["x"].cpu().numpy()
        assert np.abs(x - ox).max() <= 1e-7 * np.abs(ox).max()
    b.close()
    shared.close()
    mi.close()
