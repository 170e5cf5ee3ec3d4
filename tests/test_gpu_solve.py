"""Device CG / GMRES / mixed-precision solves against the oracle's restatement
of petsc_solve (ghost rows, rhs lifting, PETSc KSP + Jacobi, default
convergence test) and against direct solves."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu


def poisson(O, n, degree=1, kappa=1.0):
    nd, X = M.cube_mesh(n)
    if degree == 2:
        nd2, n2 = O.make_global_numbering_p2(nd)
        Xf = M.p2_coordinates(nd, nd2, X, O.tet_counts(2))
        m = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
        q = 4
    else:
        Xf, m, q = X, ft.Mesh(nd, X), 2
    p = ft.advdif_params(diffusivity=kappa, have_source=True, quad_degree=q)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, source=M.poisson_source(Xf))
    ina = np.zeros(m.N, dtype=np.uint8)
    bn = M.boundary_nodes(Xf)
    ft.apply_dirichlet_conditions(m, rhs, ina, bn, np.zeros(bn.size), dt=1.0)
    return m, Xf, val, rhs, ina


def direct(m, val, rhs, ina):
    s = m.sparsity()
    A = sp.csr_matrix((val, s.colm, s.findrm), shape=(m.N, m.N))
    act, gh = np.nonzero(ina == 0)[0], np.nonzero(ina)[0]
    x = rhs.copy()
    x[act] = spla.spsolve(A[act][:, act].tocsc(), rhs[act] - A[act][:, gh] @ rhs[gh])
    return x


def oracle_solve(O, m, val, rhs, ina, **kw):
    s = m.sparsity()
    return O.petsc_solve(s.findrm.astype(np.int64), s.colm, val, ina, rhs, **kw)


@pytest.mark.parametrize("degree,n", [(1, 8), (2, 3)])
def test_cg_matches_oracle_and_direct(O, degree, n):
    m, X, val, rhs, ina = poisson(O, n, degree)
    x = np.zeros(m.N)
    rep = ft.petsc_solve(m, x, val, rhs, ft.solver_options(ksp="cg", rtol=1e-10), inactive=ina)
    ox, oits, oreason, orn = oracle_solve(O, m, val, rhs, ina, ksp="cg", rtol=1e-10)
    assert rep["reason"] == 2 and oreason == 2
    assert abs(rep["iterations"] - oits) <= 1
    xd = direct(m, val, rhs, ina)
    scale = np.abs(xd).max()
    assert np.abs(x - xd).max() <= 1e-7 * scale
    assert np.abs(x - ox).max() <= 1e-7 * scale
    # ghost nodes take their rhs value
    assert np.array_equal(x[ina == 1], rhs[ina == 1])


def test_gmres_advdif_matches_oracle(O):
    nd, X = M.cube_mesh(8)
    m = ft.Mesh(nd, X)
    T0 = M.gaussian_tracer(X)
    p = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True, diffusivity=1e-3)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, t=T0, velocity=M.advdif_velocity(X))
    ina = np.zeros(m.N, dtype=np.uint8)
    bn = M.boundary_nodes(X)
    ft.apply_dirichlet_conditions(m, rhs, ina, bn, np.zeros(bn.size), t=T0, dt=0.01)
    for restart in (30, 4):
        x = np.zeros(m.N)
        rep = ft.petsc_solve(m, x, val, rhs, ft.solver_options(ksp="gmres", restart=restart,
                                                               rtol=1e-10), inactive=ina)
        ox, oits, oreason, _ = oracle_solve(O, m, val, rhs, ina, ksp="gmres", restart=restart,
                                            rtol=1e-10)
        assert rep["reason"] == oreason == 2
        assert abs(rep["iterations"] - oits) <= 1
        xd = direct(m, val, rhs, ina)
        assert np.abs(x - xd).max() <= 1e-7 * np.abs(xd).max()


def test_nonzero_initial_guess(O):
    m, X, val, rhs, ina = poisson(O, 6)
    x0 = np.random.default_rng(0).standard_normal(m.N) * 1e-3
    x = x0.copy()
    rep = ft.petsc_solve(m, x, val, rhs, ft.solver_options(rtol=1e-10, start_from_zero=False),
                         inactive=ina)
    ox, oits, oreason, _ = oracle_solve(O, m, val, rhs, ina, x0=x0, rtol=1e-10,
                                        start_from_zero=False)
    assert rep["reason"] == oreason == 2
    assert abs(rep["iterations"] - oits) <= 1
    assert abs(rep["rnorm0"] - 0) > 0


def test_failure_reasons(O):
    m, X, val, rhs, ina = poisson(O, 6)
    x = np.zeros(m.N)
    rep = ft.petsc_solve(m, x, val, rhs, ft.solver_options(rtol=1e-12, max_its=2), inactive=ina)
    assert rep["reason"] == -3 and rep["iterations"] == 2
    bad = rhs.copy()
    bad[np.nonzero(ina == 0)[0][0]] = np.nan
    x = np.zeros(m.N)
    rep = ft.petsc_solve(m, x, val, bad, ft.solver_options(rtol=1e-12), inactive=ina)
    assert rep["reason"] == -9
    x = np.zeros(m.N)
    rep = ft.petsc_solve(m, x, val, rhs, ft.solver_options(ksp="gmres", rtol=1e-12, max_its=3),
                         inactive=ina)
    assert rep["reason"] == -3 and rep["iterations"] == 3


@pytest.mark.parametrize("precision", ["mixed", "reliable"])
@pytest.mark.parametrize("kappa", [1.0, np.diag([1.0, 1.0, 1e-3])])
def test_mixed_precision_reaches_fp64_tolerance(O, kappa, precision):
    m, X, val, rhs, ina = poisson(O, 16, kappa=kappa)
    x64 = np.zeros(m.N)
    r64 = ft.petsc_solve(m, x64, val, rhs, ft.solver_options(rtol=1e-10), inactive=ina)
    xm = np.zeros(m.N)
    rm = ft.petsc_solve(m, xm, val, rhs, ft.solver_options(rtol=1e-10, precision=precision),
                        inactive=ina)
    assert r64["reason"] == 2 and rm["reason"] == 2
    assert rm["outer_iterations"] >= 2
    # the convergence test ran on the fp64 residual, against the fp64 solve's scale
    assert rm["rnorm0"] == pytest.approx(r64["rnorm0"], rel=1e-12)
    assert rm["final_rnorm"] <= 1e-10 * r64["rnorm0"] * (1 + 1e-12)
    assert rm["true_rel_residual"] <= 2 * r64["true_rel_residual"] + 1e-11
    assert np.abs(xm - x64).max() <= 1e-7 * np.abs(x64).max()
    if precision == "reliable":
        # no restarts of the Krylov space: close to the fp64 iteration count
        assert rm["iterations"] <= 1.25 * r64["iterations"] + 5


@pytest.mark.parametrize("start_from_zero", [True, False])
def test_unpreconditioned_norm_cg_matches_oracle(O, start_from_zero):
    """KSP_NORM_UNPRECONDITIONED: the test on ||r|| against the oracle's CG
    with the same norm (iterations +-1, same solution), and the true relative
    residual at the tolerance (the recurrence residual of FP64 CG drifts from
    the true one only by rounding)."""
    m, X, val, rhs, ina = poisson(O, 10, kappa=np.diag([1.0, 1.0, 1e-3]))
    x0 = np.zeros(m.N) if start_from_zero else 1e-3 * np.cos(3 * X[:, 1])
    x = x0.copy()
    opts = ft.solver_options(rtol=1e-10, norm="unpreconditioned", start_from_zero=start_from_zero)
    rep = ft.petsc_solve(m, x, val, rhs, opts, inactive=ina)
    ox, oits, oreason, orn = oracle_solve(O, m, val, rhs, ina, x0=x0, rtol=1e-10, norm="unpreconditioned",
                                          start_from_zero=start_from_zero)
    assert rep["reason"] == oreason == 2
    assert abs(rep["iterations"] - oits) <= 1
    assert np.abs(x - ox).max() <= 1e-7 * np.abs(ox).max()
    # the convergence is confirmed on the recomputed residual: rtol bounds it
    assert rep["true_rel_residual"] <= 1e-10 * (1 + 1e-9)
    assert abs(rep["final_rnorm"] / rep["rnorm0"] - rep["true_rel_residual"]) <= 1e-12


@pytest.mark.parametrize("precision", ["mixed", "reliable"])
def test_unpreconditioned_norm_mixed_meets_true_tolerance(O, precision):
    """Mixed precision with the unpreconditioned test: the outer test runs on
    the FP64 residual ||b - A x||, so the reported true relative residual is at
    most rtol."""
    m, X, val, rhs, ina = poisson(O, 14, kappa=np.diag([1.0, 1.0, 1e-3]))
    xm = np.zeros(m.N)
    rm = ft.petsc_solve(m, xm, val, rhs, ft.solver_options(rtol=1e-10, precision=precision,
                                                           norm="unpreconditioned"), inactive=ina)
    assert rm["reason"] == 2 and rm["outer_iterations"] >= 2
    assert rm["true_rel_residual"] <= 1e-10 * (1 + 1e-9)
    xd = direct(m, val, rhs, ina)
    assert np.abs(xm - xd).max() <= 1e-7 * np.abs(xd).max()


def test_unpreconditioned_norm_needs_cg(O):
    m, X, val, rhs, ina = poisson(O, 3)
    with pytest.raises(RuntimeError, match="unpreconditioned"):
        ft.petsc_solve(m, np.zeros(m.N), val, rhs,
                       ft.solver_options(ksp="gmres", norm="unpreconditioned"), inactive=ina)


def test_reliable_updates_from_a_guess_and_iteration_limit(O):
    m, X, val, rhs, ina = poisson(O, 12)
    xd = direct(m, val, rhs, ina)
    x = xd * (1 + 1e-3 * np.sin(7 * X[:, 0]))
    r = ft.petsc_solve(m, x, val, rhs, ft.solver_options(rtol=1e-10, precision="reliable"),
                       inactive=ina)
    x0 = np.zeros(m.N)
    r0 = ft.petsc_solve(m, x0, val, rhs, ft.solver_options(rtol=1e-10, precision="reliable"),
                        inactive=ina)
    assert r["reason"] == r0["reason"] == 2 and r["iterations"] < r0["iterations"]
    assert np.abs(x - xd).max() <= 1e-7 * np.abs(xd).max()
    xl = np.zeros(m.N)
    rl = ft.petsc_solve(m, xl, val, rhs, ft.solver_options(rtol=1e-14, max_its=9,
                                                           precision="reliable"), inactive=ina)
    assert rl["reason"] == -3 and rl["iterations"] == 9


def test_device_resident_solve(O):
    import torch
    m, X, val, rhs, ina = poisson(O, 8)
    x = np.zeros(m.N)
    rep = ft.petsc_solve(m, x, val, rhs, ft.solver_options(rtol=1e-10), inactive=ina)
    dx = torch.zeros(m.N, dtype=torch.float64, device="cuda")
    drep = ft.petsc_solve(m, dx, torch.from_numpy(val).cuda(), torch.from_numpy(rhs).cuda(),
                          ft.solver_options(rtol=1e-10), inactive=torch.from_numpy(ina).cuda())
    torch.cuda.synchronize()
    assert drep["iterations"] == rep["iterations"]
    assert dx.cpu().numpy().tobytes() == x.tobytes()  # deterministic reductions


def test_advdif_ten_steps_matches_oracle(O):
    """The CPU workload (advection-diffusion, theta=0.5, dt=0.01, GMRES+Jacobi, 10
    steps) at 8^3: the GPU driver and the oracle agree after every step."""
    nd, X = M.cube_mesh(8)
    m = ft.Mesh(nd, X)
    s = m.sparsity()
    u = M.advdif_velocity(X)
    bn = M.boundary_nodes(X)
    T = M.gaussian_tracer(X)
    T[bn] = 0.0
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
        ina = np.zeros(m.N, dtype=np.uint8)
        O.apply_dirichlet(bn, np.zeros(bn.size), To, 0.01, rhs, ina)
        dx, its, reason, _ = O.petsc_solve(s.findrm.astype(np.int64), s.colm, val, ina, rhs,
                                           ksp="gmres", restart=30, rtol=1e-10)
        To = To + 0.01 * dx
        assert np.abs(T - To).max() <= 1e-9 * np.abs(To).max()


def test_readnsolve_of_a_dump_matches_petsc_solve(O, tmp_path):
    """A matrixdump of the Dirichlet Poisson system, solved through a
    pattern-only handle, gives the solve of the original csr_matrix."""
    from fluidity_gb300 import petsc_io as P
    m, X, val, rhs, ina = poisson(O, 8)
    s = m.sparsity()
    x = np.zeros(m.N)
    opts = ft.solver_options(ksp="cg", rtol=1e-10)
    rep = ft.petsc_solve(m, x, val, rhs, opts, inactive=ina)
    nf, nc, nv, b, x0 = P.petsc_matrix(s.findrm, s.colm, val, ina, rhs)
    f = tmp_path / "matrixdump"
    P.write_matrixdump(f, nf, nc, nv, b, x0)
    y, drep = P.petsc_readnsolve(f, opts)
    act = ina == 0
    assert drep["reason"] == 2 and abs(drep["iterations"] - rep["iterations"]) <= 1
    assert np.abs(y[act] - x[act]).max() <= 1e-8 * np.abs(x).max()
    assert np.abs(y[~act]).max() == 0.0


def test_every_row_dirichlet(O):
    """All rows inactive: the solution is the rhs on every row (ghost
    semantics) after no iteration, for CG and GMRES, as in the oracle."""
    m, Xf, val, rhs, ina = poisson(O, 3)
    ina[:] = 1
    g = np.linspace(-1.0, 1.0, m.N)
    rhs = g.copy()
    for ksp in ("cg", "gmres"):
        x = np.full(m.N, 7.0)
        rep = ft.petsc_solve(m, x, val, rhs, ft.solver_options(ksp=ksp, rtol=1e-10), inactive=ina)
        assert np.array_equal(x, g)
        ox, its, reason, _ = oracle_solve(O, m, val, rhs, ina, ksp=ksp)
        assert np.array_equal(ox, g)
        assert rep["iterations"] == its == 0


def test_projected_guess_is_the_a_norm_minimiser(O):
    """fl_dev_projected_guess against a dense restatement of the projection
    method on the ghost-reduced system, and the minimising property: the
    guess's A-norm error is below each basis vector's."""
    import torch
    m, X, val, rhs, ina = poisson(O, 7)
    xd = direct(m, val, rhs, ina)
    rng = np.random.default_rng(5)
    basis = [xd * (1 + 0.1 * rng.standard_normal(m.N)), np.sin(3 * X[:, 0]) * xd, rng.standard_normal(m.N),
             xd * (1 + 0.1 * rng.standard_normal(m.N))]
    dev = [torch.from_numpy(b).cuda() for b in basis]
    x0, a = ft.projected_guess(m, torch.from_numpy(val).cuda(), torch.from_numpy(rhs).cuda(), dev,
                               inactive=torch.from_numpy(ina).cuda())
    x0 = x0.cpu().numpy()
    s = m.sparsity()
    A = sp.csr_matrix((val, s.colm, s.findrm), shape=(m.N, m.N))
    act, gh = np.nonzero(ina == 0)[0], np.nonzero(ina)[0]
    Aa = A[act][:, act]
    b = rhs[act] - A[act][:, gh] @ rhs[gh]
    V = np.stack([v[act] for v in basis], axis=1)
    ad = np.linalg.solve(V.T @ (Aa @ V), V.T @ b)
    assert np.abs(a - ad).max() <= 1e-8 * np.abs(ad).max()
    assert np.abs(x0[act] - V @ ad).max() <= 1e-10 * np.abs(xd).max()
    assert np.array_equal(x0[gh], rhs[gh])

    def anorm(v):
        e = v[act] - xd[act]
        return float(np.sqrt(e @ (Aa @ e)))
    assert all(anorm(x0) <= anorm(v) for v in basis)
    # a vector in the span of earlier ones is dropped, the result unchanged
    x1, a1 = ft.projected_guess(m, torch.from_numpy(val).cuda(), torch.from_numpy(rhs).cuda(),
                                dev + [dev[0] * 2.0], inactive=torch.from_numpy(ina).cuda())
    assert a1[-1] == 0.0
    assert np.abs(x1.cpu().numpy() - x0).max() <= 1e-12 * np.abs(xd).max()


def _advdif_system(n):
    nd, X = M.cube_mesh(n)
    m = ft.Mesh(nd, X)
    T0 = M.gaussian_tracer(X)
    p = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True, diffusivity=1e-3)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, t=T0, velocity=M.advdif_velocity(X))
    ina = np.zeros(m.N, dtype=np.uint8)
    bn = M.boundary_nodes(X)
    ft.apply_dirichlet_conditions(m, rhs, ina, bn, np.zeros(bn.size), t=T0, dt=0.01)
    return m, val, rhs, ina


@pytest.mark.parametrize("n,restart", [(8, 30), (8, 4), (32, 30), (32, 7)])
def test_gmres_schedules_agree(O, n, restart):
    """The cooperative single-launch GMRES and the graph-replayed one run the
    same algorithm (same Krylov space, reductions in another order): same
    reason, iterations within one, solutions within the solve tolerance; the
    32^3 case (35,937 rows) takes several row passes per block."""
    m, val, rhs, ina = _advdif_system(n)
    x0 = np.random.default_rng(1).standard_normal(m.N) * 1e-2
    res = {}
    for sched in ("graph", "persistent"):
        for guess in (False, True):
            x = x0.copy() if guess else np.zeros(m.N)
            o = ft.solver_options(ksp="gmres", restart=restart, rtol=1e-10, schedule=sched,
                                  start_from_zero=not guess)
            rep = ft.petsc_solve(m, x, val, rhs, o, inactive=ina)
            res[sched, guess] = (x, rep)
    for guess in (False, True):
        (xg, rg), (xp, rp) = res["graph", guess], res["persistent", guess]
        assert rg["reason"] == rp["reason"] == 2
        assert abs(rg["iterations"] - rp["iterations"]) <= 1
        scale = np.abs(xg).max()
        assert np.abs(xg - xp).max() <= 1e-8 * scale
        assert rp["true_rel_residual"] <= 1e-8
    if n == 8:
        ox, oits, oreason, _ = oracle_solve(O, m, val, rhs, ina, ksp="gmres", restart=restart, rtol=1e-10)
        x, rep = res["persistent", False]
        assert rep["reason"] == oreason and abs(rep["iterations"] - oits) <= 1
        assert np.abs(x - ox).max() <= 1e-8 * np.abs(ox).max()


@pytest.mark.parametrize("sched", ["graph", "persistent"])
def test_gmres_schedule_edge_cases(O, sched):
    """Iteration limit inside and at the end of a cycle, a NaN right-hand
    side, a zero right-hand side (converged at the first test) and every row
    inactive, through both launch schedules."""
    m, val, rhs, ina = _advdif_system(6)
    for max_its in (3, 4, 8):
        x = np.zeros(m.N)
        rep = ft.petsc_solve(m, x, val, rhs, ft.solver_options(ksp="gmres", restart=4, rtol=1e-14,
                                                               max_its=max_its, schedule=sched),
                             inactive=ina)
        assert rep["reason"] == -3 and rep["iterations"] == max_its
    bad = rhs.copy()
    bad[np.nonzero(ina == 0)[0][0]] = np.nan
    x = np.zeros(m.N)
    rep = ft.petsc_solve(m, x, val, bad, ft.solver_options(ksp="gmres", schedule=sched), inactive=ina)
    assert rep["reason"] == -9
    x = np.zeros(m.N)
    zero = np.zeros(m.N)
    rep = ft.petsc_solve(m, x, val, zero, ft.solver_options(ksp="gmres", schedule=sched, start_from_zero=True),
                         inactive=ina)
    ox, its, reason, _ = oracle_solve(O, m, val, zero, ina, ksp="gmres")
    assert rep["reason"] == reason and rep["iterations"] == its == 0
    assert np.array_equal(x, ox)
    ina2 = np.ones(m.N, dtype=np.uint8)
    g = np.linspace(-1.0, 1.0, m.N)
    x = np.full(m.N, 7.0)
    rep = ft.petsc_solve(m, x, val, g, ft.solver_options(ksp="gmres", schedule=sched), inactive=ina2)
    assert np.array_equal(x, g) and rep["iterations"] == 0


@pytest.mark.parametrize("sched", ["graph", "persistent"])
def test_gmres_long_restart_matches_oracle(O, sched):
    """GMRES(60) on a Poisson system that needs more than 32 iterations in its
    first cycle: the Hessenberg update's second chunk of 32 rotations and the
    cooperative kernel's second lane of dot products run; reason, iterations
    (within two: the sums run in another order than the oracle's) and the
    solution match the oracle, and a restart inside the solve (restart 40)
    as well."""
    m, X, val, rhs, ina = poisson(O, 14)
    for restart in (60, 40):
        x = np.zeros(m.N)
        rep = ft.petsc_solve(m, x, val, rhs, ft.solver_options(ksp="gmres", restart=restart, rtol=1e-10,
                                                               schedule=sched), inactive=ina)
        ox, oits, oreason, _ = oracle_solve(O, m, val, rhs, ina, ksp="gmres", restart=restart, rtol=1e-10)
        assert oits > 32
        assert rep["reason"] == oreason == 2
        assert abs(rep["iterations"] - oits) <= 2
        assert np.abs(x - ox).max() <= 1e-7 * np.abs(ox).max()


def test_fused_field_step_matches_the_three_calls(O):
    """fl_dev_solve_field_equation_cg (assembly, rate-of-change Dirichlet
    conditions, solve from zero change, t + dt delta in one call) gives the
    bits of the three separate calls, step after step; a boundary node out of
    range is reported after the step and the next step still works."""
    import torch
    from fluidity_gb300 import _lib
    nd, X = M.cube_mesh(8)
    m = ft.Mesh(nd, X)
    p = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True, diffusivity=1e-3)
    u = torch.tensor(M.advdif_velocity(X), device="cuda")
    bn = torch.tensor(M.boundary_nodes(X), device="cuda")
    g = torch.zeros(bn.numel(), dtype=torch.float64, device="cuda")
    opts = ft.solver_options(ksp="gmres", restart=30, rtol=1e-10)
    t0 = torch.tensor(M.gaussian_tracer(X), device="cuda")
    ta, tb = t0.clone(), t0.clone()
    val = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(m.N, dtype=torch.float64, device="cuda")
    ina = torch.zeros(m.N, dtype=torch.uint8, device="cuda")
    for _ in range(3):
        ft.assemble_advection_diffusion_cg(m, p, t=ta, velocity=u, val=val, rhs=rhs)
        ina.zero_()
        ft.apply_dirichlet_conditions(m, rhs, ina, bn, g, t=ta, dt=p.dt)
        d = torch.zeros(m.N, dtype=torch.float64, device="cuda")
        rep_a = ft.petsc_solve(m, d, val, rhs, opts, inactive=ina)
        ta = ta + p.dt * d
        tb, rep_b = ft.solve_field_equation_cg_device(m, tb, p, opts, bc_nodes=bn, bc_values=g, velocity=u)
        assert rep_a["iterations"] == rep_b["iterations"] and rep_b["reason"] == 2
        assert torch.equal(ta, tb)
    bad = bn.clone()
    bad[0] = m.N + 5
    with pytest.raises(_lib.FlError):
        ft.solve_field_equation_cg_device(m, tb, p, opts, bc_nodes=bad, bc_values=g, velocity=u)
    tc, rep = ft.solve_field_equation_cg_device(m, tb, p, opts, bc_nodes=bn, bc_values=g, velocity=u)
    assert rep["reason"] == 2 and torch.isfinite(tc).all()
