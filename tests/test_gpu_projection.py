"""GPU pressure-projection matrices (P1 pressure, P1 velocity) against the
oracle's restatements of assemble_divergence_matrix_cg, compute_lumped_mass,
make_sparsity_transpose, mult_div_vector_div_T / mult_div_invscalar_div_T,
assemble_kmk_matrix and the mass-lumped projection vectors.

Integer work (the second-order pattern) is bit-exact.  Floating point:
|a - a_ref| <= 1e-12 * max_j |a_ref(i, j)| per row (matrices) and
1e-12 * max |v_ref| (vectors).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from conftest import row_scaled_error
from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M
from fluidity_gb300 import projection as PR

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


@pytest.fixture(scope="module", params=[4, 7])
def case(request, O):
    n = request.param
    nd, X = M.cube_mesh(n)
    mesh = ft.Mesh(nd, X)
    s = mesh.sparsity()
    f = s.findrm.astype(np.int64)
    sf, sc = O.sparsity_secondorder(f, s.colm)
    yield dict(n=n, nd=nd, X=X, mesh=mesh, f=f, c=s.colm, sf=sf, sc=sc)
    mesh.close()


def _np(t):
    return t.detach().cpu().numpy()


def _vec_ok(a, b, tol=TOL):
    return np.abs(a - b).max() <= tol * max(np.abs(b).max(), 1e-300)


def test_secondorder_pattern_bit_exact(case):
    so = PR.get_csr_sparsity_secondorder(case["mesh"])
    sp_ = so.sparsity()
    assert np.array_equal(sp_.findrm, case["sf"])
    assert np.array_equal(sp_.colm, case["sc"])
    rows = np.repeat(np.arange(len(case["sf"]) - 1), np.diff(case["sf"]))
    diag = np.nonzero(case["sc"] == rows)[0]
    assert np.array_equal(sp_.centrm, diag)


@pytest.mark.parametrize("by_parts", [False, True])
def test_divergence_matches_oracle(case, O, by_parts):
    nd, X, f, c = case["nd"], case["X"], case["f"], case["c"]
    faces, fe = M.boundary_faces(nd)
    out = PR.assemble_divergence_matrix_cg(case["mesh"], integrate_by_parts=by_parts, faces=faces, face_ele=fe)
    ct, rhs, dml, gml = O.assemble_divergence_p1(nd, X, f, c, by_parts=by_parts, faces=faces, face_ele=fe)
    got = _np(out["ct"])
    for d in range(3):
        assert row_scaled_error(got[d], ct[d], f) <= TOL
    assert _vec_ok(_np(out["div_mass_lumped"]), dml)
    assert _vec_ok(_np(out["grad_mass_lumped"]), gml)
    assert not _np(out["ct_rhs"]).any()


def test_divergence_surface_types(case, O):
    nd, X, f, c = case["nd"], case["X"], case["f"], case["c"]
    faces, fe = M.boundary_faces(nd)
    nf = len(faces)
    rng = np.random.default_rng(11)
    ty = np.zeros((nf, 3), np.int32)
    ty[::5, 0] = 1          # weak Dirichlet in x
    ty[1::5, 1] = 1         # weak Dirichlet in y
    ty[2::7, 2] = 2         # no_normal_flow: face skipped
    ty[3::11, 0] = 5        # prescribed normal flow
    ty[4::13, 1] = 4        # free_surface: skipped
    g = rng.random((nf, 3, 3))
    out = PR.assemble_divergence_matrix_cg(case["mesh"], integrate_by_parts=True, faces=faces, face_ele=fe,
                                           bc_type=ty, bc_val=g)
    ct, rhs, _, _ = O.assemble_divergence_p1(nd, X, f, c, by_parts=True, faces=faces, face_ele=fe, bc_type=ty,
                                             bc_val=g)
    got = _np(out["ct"])
    for d in range(3):
        assert row_scaled_error(got[d], ct[d], f) <= TOL
    assert _vec_ok(_np(out["ct_rhs"]), rhs)


def test_lumped_mass(case, O):
    ml = _np(PR.compute_lumped_mass(case["mesh"]))
    ref = O.lumped_mass(case["nd"], case["nd"], case["X"], len(case["X"]))
    assert _vec_ok(ml, ref)
    assert abs(ml.sum() - 1.0) < 1e-13


def test_cmc_matches_oracle(case, O, torch):
    nd, X, f, c = case["nd"], case["X"], case["f"], case["c"]
    mesh = case["mesh"]
    so = PR.get_csr_sparsity_secondorder(mesh)
    out = PR.assemble_divergence_matrix_cg(mesh)
    ct = out["ct"]
    ml = out["grad_mass_lumped"]
    inv = PR.inverse_lumped_mass(ml, M.boundary_nodes(X))
    cmc = PR.assemble_masslumped_cmc(so, ct, inv, ct)
    ref = O.mult_div_vector_div_T(f, c, _np(ct), _np(inv), _np(ct), case["sf"], case["sc"])
    assert row_scaled_error(_np(cmc), ref, case["sf"]) <= TOL
    # one and two blocks (ndim < 3)
    for ndim in (1, 2):
        w = inv[:, :ndim].contiguous()
        got = PR.mult_div_vector_div_T(so, ct[:ndim], w, ct[:ndim])
        ref = O.mult_div_vector_div_T(f, c, _np(ct)[:ndim], _np(w), _np(ct)[:ndim], case["sf"], case["sc"])
        assert row_scaled_error(_np(got), ref, case["sf"]) <= TOL
    # deterministic: a second evaluation is bitwise identical
    again = PR.assemble_masslumped_cmc(so, ct, inv, ct)
    assert torch.equal(again, cmc)


@pytest.mark.parametrize("theta", [1.0, 0.7])
def test_kmk_matches_oracle(case, O, theta):
    nd, X, f, c = case["nd"], case["X"], case["f"], case["c"]
    mesh = case["mesh"]
    so = PR.get_csr_sparsity_secondorder(mesh)
    ml = PR.compute_lumped_mass(mesh)
    kmk, kt = PR.assemble_kmk_matrix(mesh, so, ml, theta_pg=theta)
    okt, okmk = O.assemble_kmk(nd, X, f, c, _np(ml), case["sf"], case["sc"], theta_pg=theta)
    assert row_scaled_error(_np(kt), okt, f) <= TOL
    assert row_scaled_error(_np(kmk), okmk, case["sf"]) <= TOL
    # mult_div_invscalar_div_T on its own, on the oracle's kt
    import torch
    ktd = torch.as_tensor(okt, device="cuda")
    s = ml * theta if theta != 1.0 else ml
    got = PR.mult_div_invscalar_div_T(so, ktd, s, ktd)
    ref = O.mult_div_invscalar_div_T(f, c, okt, _np(s), okt, case["sf"], case["sc"])
    assert row_scaled_error(_np(got), ref, case["sf"]) <= TOL


def test_projection_vectors_match_oracle(case, O, torch):
    mesh, X, f, c = case["mesh"], case["X"], case["f"], case["c"]
    out = PR.assemble_divergence_matrix_cg(mesh)
    ct = out["ct"]
    inv = PR.inverse_lumped_mass(out["grad_mass_lumped"], M.boundary_nodes(X))
    rng = np.random.default_rng(5)
    N = len(X)
    u = torch.as_tensor(M.advdif_velocity(X), device="cuda").contiguous()
    mom = torch.as_tensor(rng.random((N, 3)), device="cuda").contiguous()
    ctr = torch.as_tensor(rng.random(N), device="cuda")
    rhs = PR.assemble_masslumped_poisson_rhs(mesh, ct, mom, ctr, inv, u, dt=0.1, theta_pg=0.5)
    ref = O.masslumped_poisson_rhs(f, c, _np(ct), _np(mom), _np(ctr), _np(inv), _np(u), 0.1, 0.5)
    assert _vec_ok(_np(rhs), ref)
    dp = torch.as_tensor(rng.random(N), device="cuda")
    u2 = u.clone()
    PR.correct_masslumped_velocity(mesh, ct, inv, dp, u2)
    ref = O.correct_masslumped_velocity(f, c, _np(ct), _np(inv), _np(dp), _np(u))
    assert _vec_ok(_np(u2), ref)


def test_projection_makes_velocity_discretely_divergence_free(case, torch):
    """CMC dp = -C u*, u = u* + M_l^-1 C^T dp gives C u = 0 on the pressure rows
    that the solve holds (all but one reference node), to the solver tolerance;
    CMC + KMK assembles and solves on the same pattern."""
    mesh, X = case["mesh"], case["X"]
    N = len(X)
    so = PR.get_csr_sparsity_secondorder(mesh)
    out = PR.assemble_divergence_matrix_cg(mesh)
    ct = out["ct"]
    inv = PR.inverse_lumped_mass(out["grad_mass_lumped"], M.boundary_nodes(X))
    cmc = PR.assemble_masslumped_cmc(so, ct, inv, ct)
    # a velocity that vanishes on the no-slip boundary keeps the (P1-P1,
    # unstabilised, possibly singular) system consistent
    bubble = 64.0 * np.prod(X * (1.0 - X), axis=1)
    u = torch.as_tensor(M.advdif_velocity(X) * bubble[:, None], device="cuda").contiguous()
    rhs = PR.assemble_masslumped_poisson_rhs(mesh, ct, None, None, None, u, dt=1.0, theta_pg=1.0)
    ina = torch.zeros(N, dtype=torch.uint8, device="cuda")
    ref_node = N // 2
    ina[ref_node] = 1
    rhs[ref_node] = 0.0
    dp = torch.zeros(N, dtype=torch.float64, device="cuda")
    rep = ft.petsc_solve(so, dp, cmc, rhs, ft.solver_options(ksp="cg", rtol=1e-12, max_its=5000), inactive=ina)
    assert rep["reason"] > 0
    before = sum(sp.csr_matrix((_np(ct[d]), case["c"], case["f"]), shape=(N, N)) @ _np(u)[:, d] for d in range(3))
    PR.correct_masslumped_velocity(mesh, ct, inv, dp, u)
    after = sum(sp.csr_matrix((_np(ct[d]), case["c"], case["f"]), shape=(N, N)) @ _np(u)[:, d] for d in range(3))
    keep = np.arange(N) != ref_node
    assert np.abs(after[keep]).max() < 1e-8 * np.abs(before).max()
    # the stabilised matrix of the P1-P1 pair solves on the same pattern
    kmk, _ = PR.assemble_kmk_matrix(mesh, so, PR.compute_lumped_mass(mesh), theta_pg=1.0)
    PR.add_kmk_matrix(so, cmc, kmk)
    dp.zero_()
    rep = ft.petsc_solve(so, dp, cmc, rhs, ft.solver_options(ksp="cg", rtol=1e-10, max_its=5000), inactive=ina)
    assert rep["reason"] > 0


def test_cmc_symmetry_at_size(torch):
    """Size-independent properties at 32^3: C M_l^-1 C^T is symmetric to
    rounding and is the same on a second evaluation."""
    nd, X = M.cube_mesh(32)
    mesh = ft.Mesh(nd, X)
    so = PR.get_csr_sparsity_secondorder(mesh)
    out = PR.assemble_divergence_matrix_cg(mesh)
    inv = PR.inverse_lumped_mass(out["grad_mass_lumped"], M.boundary_nodes(X))
    cmc = PR.assemble_masslumped_cmc(so, out["ct"], inv, out["ct"])
    s = so.sparsity()
    A = sp.csr_matrix((_np(cmc), s.colm, s.findrm), shape=(len(X),) * 2)
    assert abs(A - A.T).max() <= 1e-14 * abs(A).max()
    assert torch.equal(cmc, PR.assemble_masslumped_cmc(so, out["ct"], inv, out["ct"]))
    so.close()
    mesh.close()


@pytest.mark.parametrize("which", ["cube3", "cube6", "aniso"])
def test_taylor_hood_divergence_matches_oracle(O, torch, aniso_mesh, which):
    """P2 velocity / P1 pressure: the rectangular pattern bit-exact with the
    oracle's two-mesh make_sparsity, and C^T in both forms within 1e-12
    row-scaled of orc_assemble_divergence_p2p1, on the cube and on the
    reference's unstructured mesh."""
    nd, X = {"cube3": M.cube_mesh(3), "cube6": M.cube_mesh(6)}.get(which, aniso_mesh)
    nd2, n2 = O.make_global_numbering_p2(nd)
    mesh = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    pat = PR.TaylorHoodPattern(mesh)
    s = pat.sparsity()
    f, c = O.make_sparsity_rect(nd, nd2, X.shape[0])
    assert pat.N == X.shape[0] and pat.nnz == c.size
    assert np.array_equal(s.findrm, f) and np.array_equal(s.colm, c)
    for bp in (False, True):
        ct = PR.assemble_divergence_matrix_p2p1(mesh, pat, integrate_by_parts=bp)
        torch.cuda.synchronize()
        oct_ = O.assemble_divergence_p2p1(nd, nd2, X, f, c, by_parts=bp)
        got = ct.cpu().numpy()
        for d in range(3):
            assert row_scaled_error(got[d], oct_[d], f) <= TOL, (bp, d)
        again = PR.assemble_divergence_matrix_p2p1(mesh, pat, integrate_by_parts=bp)
        assert torch.equal(again, ct)  # deterministic
    pat.close()
    mesh.close()


@pytest.mark.parametrize("which", ["cube4", "unstructured"])
def test_taylor_hood_surface_terms_match_oracle(O, torch, aniso_mesh, which):
    """The by-parts surface loop of the Taylor-Hood divergence
    (fl_dev_assemble_divergence_p2p1_faces) against
    orc_assemble_divergence_p2p1_faces, with a mix of face types (none, weak
    Dirichlet, prescribed normal flow, no-normal-flow), 1-based faces too;
    and by parts with every face's terms equals not by parts.
    Tolerance: 1e-12 row-scaled on ct, 1e-12 of max |ct_rhs|."""
    nd, X = M.cube_mesh(4) if which == "cube4" else aniso_mesh
    nd2, n2 = O.make_global_numbering_p2(nd)
    mesh = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    pat = PR.TaylorHoodPattern(mesh)
    f, c = O.make_sparsity_rect(nd, nd2, X.shape[0])
    N = X.shape[0]
    faces6, xf, fe = M.boundary_faces_p2(nd, nd2)
    nf = xf.shape[0]
    rng = np.random.default_rng(23)
    ty = np.zeros((nf, 3), np.int32)
    kind = rng.integers(0, 4, nf)
    ty[kind == 1] = 1
    ty[kind == 2, 0] = 5
    ty[kind == 3, 1] = 2
    bv = rng.standard_normal((nf, 6, 3))
    kw = dict(pfaces=xf, ufaces=faces6, face_ele=fe, ndglno_x=nd, coords=X, findrm=f, colm=c)
    octb = O.assemble_divergence_p2p1(nd, nd2, X, f, c, by_parts=True)
    orhs = np.zeros(N)
    assert O.assemble_divergence_p2p1_faces(octb, orhs, bc_type=ty, bc_val=bv, **kw) == 0
    for base in (0, 1):
        ct = PR.assemble_divergence_matrix_p2p1(mesh, pat, integrate_by_parts=True)
        rhs = torch.zeros(N, dtype=torch.float64, device="cuda")
        PR.assemble_divergence_faces_p2p1(mesh, pat, ct, faces=xf + base, vfaces=faces6 + base, face_ele=fe + base,
                                          bc_type=ty, bc_val=bv, ct_rhs=rhs, index_base=base)
        torch.cuda.synchronize()
        got = ct.cpu().numpy()
        for d in range(3):
            assert row_scaled_error(got[d], octb[d], f) <= TOL, (base, d)
        assert np.abs(rhs.cpu().numpy() - orhs).max() <= TOL * np.abs(orhs).max()
    # every face type 0: the by-parts matrix equals the direct one
    ct = PR.assemble_divergence_matrix_p2p1(mesh, pat, integrate_by_parts=True)
    PR.assemble_divergence_faces_p2p1(mesh, pat, ct, faces=xf, vfaces=faces6, face_ele=fe)
    direct = PR.assemble_divergence_matrix_p2p1(mesh, pat, integrate_by_parts=False)
    torch.cuda.synchronize()
    got, want = ct.cpu().numpy(), direct.cpu().numpy()
    for d in range(3):
        assert row_scaled_error(got[d], want[d], f) <= 1e-12
    pat.close()
    mesh.close()


@pytest.mark.parametrize("which", ["cube4", "unstructured"])
def test_taylor_hood_cmc_matches_scipy(O, torch, aniso_mesh, which):
    """cmc_m of the Taylor-Hood pair (fl_gpu_rect_secondorder_register and
    fl_dev_mult_div_vector_div_T): the pattern equals the structure of C C^T
    through the velocity nodes, bit for bit, and C^T diag(w) C with a weight
    per velocity node and dimension agrees with scipy's FP64 triple product
    within 1e-12 row-scaled; symmetric and deterministic."""
    nd, X = M.cube_mesh(4) if which == "cube4" else aniso_mesh
    N = X.shape[0]
    nd2, n2 = O.make_global_numbering_p2(nd)
    mesh = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    pat = PR.TaylorHoodPattern(mesh)
    prod = PR.TaylorHoodProductPattern(pat)
    f, c = O.make_sparsity_rect(nd, nd2, N)
    S = sp.csr_matrix((np.ones(c.size), c, f), shape=(N, n2))
    P = (S @ S.T).tocsr()
    P.sort_indices()
    s = prod.sparsity()
    assert prod.N == N and prod.nnz == P.nnz
    assert np.array_equal(s.findrm, P.indptr) and np.array_equal(s.colm, P.indices)
    ct = PR.assemble_divergence_matrix_p2p1(mesh, pat)
    w = torch.tensor(np.random.default_rng(4).random((n2, 3)) + 0.5, device="cuda")
    cmc = PR.mult_div_vector_div_T(prod, ct, w.reshape(-1), ct)
    torch.cuda.synchronize()
    cth, wh = ct.cpu().numpy(), w.cpu().numpy()
    ref = sum(sp.csr_matrix((cth[d], c, f), shape=(N, n2)) @ sp.diags(wh[:, d])
              @ sp.csr_matrix((cth[d], c, f), shape=(N, n2)).T for d in range(3)).toarray()
    rows = np.repeat(np.arange(N), np.diff(P.indptr))
    want = ref[rows, P.indices]
    got = cmc.cpu().numpy()
    assert row_scaled_error(got, want, P.indptr) <= TOL
    A = sp.csr_matrix((got, P.indices, P.indptr), shape=(N, N))
    assert abs(A - A.T).max() <= 1e-14 * abs(A).max()
    assert torch.equal(cmc, PR.mult_div_vector_div_T(prod, ct, w.reshape(-1), ct))
    prod.close()
    pat.close()
    mesh.close()


@pytest.mark.parametrize("which", ["cube4", "unstructured"])
def test_p2_lumped_mass_matches_oracle(O, torch, aniso_mesh, which):
    """compute_lumped_mass of the P2 velocity mesh (the weights of the
    Taylor-Hood cmc_m): within 1e-13 of orc_lumped_mass (degree 2, the
    degree-4 rule), -V/20 at the vertices and V/5 at the edges of every
    element, summing to the domain's volume."""
    nd, X = M.cube_mesh(4) if which == "cube4" else aniso_mesh
    nd2, n2 = O.make_global_numbering_p2(nd)
    mesh = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    ml = PR.compute_lumped_mass(mesh)
    torch.cuda.synchronize()
    got = ml.cpu().numpy()
    want = O.lumped_mass(nd2, nd, X, n2, degree=2, quad_degree=4)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
    J = np.stack([X[nd[:, k]] - X[nd[:, 3]] for k in range(3)], axis=1)
    vol = np.abs(np.linalg.det(J)) / 6.0
    assert abs(got.sum() - vol.sum()) <= 1e-13 * vol.sum()
    vert = np.zeros(n2, bool)
    vert[np.unique(nd2[:, [0, 2, 5, 9]])] = True
    assert (got[vert] < 0).all() and (got[~vert] > 0).all()
    mesh.close()


def test_taylor_hood_error_paths(O):
    """Weak-Dirichlet or normal-flow faces without boundary values, and a
    product pattern asked of a handle that is not a Taylor-Hood pattern, are
    argument errors, and the handles stay usable."""
    import torch
    nd, X = M.cube_mesh(3)
    nd2, n2 = O.make_global_numbering_p2(nd)
    mesh = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    pat = PR.TaylorHoodPattern(mesh)
    faces6, xf, fe = M.boundary_faces_p2(nd, nd2)
    nf = xf.shape[0]
    ct = PR.assemble_divergence_matrix_p2p1(mesh, pat, integrate_by_parts=True)
    rhs = torch.zeros(X.shape[0], dtype=torch.float64, device="cuda")
    for t in (1, 5):
        ty = np.zeros((nf, 3), np.int32)
        ty[:, 0] = t
        with pytest.raises(RuntimeError, match="surface terms"):
            PR.assemble_divergence_faces_p2p1(mesh, pat, ct, faces=xf, vfaces=faces6, face_ele=fe, bc_type=ty,
                                              ct_rhs=rhs)
    with pytest.raises(RuntimeError, match="Taylor-Hood pattern"):
        PR.TaylorHoodProductPattern(mesh)
    ct2 = PR.assemble_divergence_matrix_p2p1(mesh, pat, integrate_by_parts=True)
    PR.assemble_divergence_faces_p2p1(mesh, pat, ct2, faces=xf, vfaces=faces6, face_ele=fe)
    torch.cuda.synchronize()
    assert torch.isfinite(ct2).all()
    pat.close()
    mesh.close()
