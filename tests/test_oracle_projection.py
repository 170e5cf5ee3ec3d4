"""CPU oracle of the pressure-projection pieces, pinned against the
reference's known answers and exact identities (no GPU)."""
import numpy as np
import pytest
import scipy.sparse as sp

from fluidity_gb300 import meshgen as M
from oracle import oracle as O


@pytest.fixture(scope="module")
def mesh4():
    nd, X = M.cube_mesh(4)
    f, c, _ = O.make_sparsity(nd)
    return nd, X, f, c


def test_simplex_tensor_known_answer():
    # error_measures/tests/test_simplex_tensor.F90: tests/data/triangle.1 has
    # vertices (0, 0.5), (0, -0.5), (1, 0) and the metric diag(0.75, 1)
    m = O.simplex_tensor(np.array([[0.0, 0.5], [0.0, -0.5], [1.0, 0.0]]))
    assert np.allclose(m, [[0.75, 0.0], [0.0, 1.0]], rtol=0, atol=4 * np.finfo(float).eps)


def test_simplex_tensor_unit_edges(mesh4):
    # error_measures/tests/test_simplex_tensor_edgelens.F90: in the metric every
    # edge has unit length (tolerance 201 epsilon)
    nd, X, _, _ = mesh4
    for e in range(0, len(nd), 7):
        P = X[nd[e]]
        m = O.simplex_tensor(P)
        h = O.edge_length_metric(m)
        for i in range(4):
            for j in range(i + 1, 4):
                d = P[j] - P[i]
                assert abs(np.sqrt(d @ m @ d) - 1.0) < 201 * np.finfo(float).eps
        assert np.abs(h @ m @ h - np.eye(3)).max() < 1e-13


def test_lumped_mass_is_the_volume(mesh4):
    nd, X, f, c = mesh4
    ml = O.lumped_mass(nd, nd, X, len(X))
    assert abs(ml.sum() - 1.0) < 1e-14
    assert (ml > 0).all()


def test_divergence_by_parts_identity(mesh4):
    # integral(N_i dN_j/dx) = -integral(dN_i/dx N_j) + surface integral(N_i N_j n)
    nd, X, f, c = mesh4
    ct, _, dml, gml = O.assemble_divergence_p1(nd, X, f, c)
    faces, fe = M.boundary_faces(nd)
    ct2, rhs2, _, _ = O.assemble_divergence_p1(nd, X, f, c, by_parts=True, faces=faces, face_ele=fe)
    assert np.abs(ct - ct2).max() < 1e-15 * 1e3 * np.abs(ct).max()
    assert np.array_equal(dml, gml)
    assert not rhs2.any()
    # divergence of a constant field is zero away from the boundary
    bn = M.boundary_nodes(X)
    inner = np.setdiff1d(np.arange(len(X)), bn)
    for d in range(3):
        A = sp.csr_matrix((ct[d], c, f), shape=(len(X),) * 2)
        assert np.abs((A @ np.ones(len(X)))[inner]).max() < 1e-16


def test_divergence_surface_types(mesh4):
    # weak Dirichlet moves the face term to ct_rhs; types 2-4 drop the face
    nd, X, f, c = mesh4
    faces, fe = M.boundary_faces(nd)
    nf = len(faces)
    ty0 = np.zeros((nf, 3), np.int32)
    ct0, _, _, _ = O.assemble_divergence_p1(nd, X, f, c, by_parts=True, faces=faces, face_ele=fe, bc_type=ty0)
    ty = ty0.copy()
    ty[:, 0] = 1
    g = np.random.default_rng(3).random((nf, 3, 3))
    ct1, rhs1, _, _ = O.assemble_divergence_p1(nd, X, f, c, by_parts=True, faces=faces, face_ele=fe, bc_type=ty,
                                               bc_val=g)
    ctn, _, _, _ = O.assemble_divergence_p1(nd, X, f, c, by_parts=True)
    # dimension 0 lost its face terms, the others kept them
    assert np.abs(ct1[0] - ctn[0]).max() < 1e-17
    assert np.abs(ct1[1:] - ct0[1:]).max() == 0.0
    assert np.abs(rhs1).max() > 0.0


def test_secondorder_pattern_is_the_structural_square(mesh4):
    nd, X, f, c = mesh4
    sf, sc = O.sparsity_secondorder(f, c)
    A = sp.csr_matrix((np.ones(len(c)), c, f), shape=(len(X),) * 2)
    B = (A @ A).tocsr()
    B.sort_indices()
    assert np.array_equal(B.indptr, sf) and np.array_equal(B.indices, sc)


def test_row_products_match_the_triple_product(mesh4):
    nd, X, f, c = mesh4
    N = len(X)
    ct, _, _, _ = O.assemble_divergence_p1(nd, X, f, c)
    sf, sc = O.sparsity_secondorder(f, c)
    w = np.random.default_rng(1).random((N, 3)) + 0.5
    cmc = O.mult_div_vector_div_T(f, c, ct, w, ct, sf, sc)
    blk = [sp.csr_matrix((ct[d], c, f), shape=(N, N)) for d in range(3)]
    ref = sum(blk[d] @ sp.diags(w[:, d]) @ blk[d].T for d in range(3))
    assert abs(sp.csr_matrix((cmc, sc, sf), shape=(N, N)) - ref).max() < 1e-15 * abs(ref).max()
    ml = O.lumped_mass(nd, nd, X, N)
    for theta in (1.0, 0.6):
        kt, kmk = O.assemble_kmk(nd, X, f, c, ml, sf, sc, theta_pg=theta)
        K = sp.csr_matrix((kt, c, f), shape=(N, N))
        assert abs(K - K.T).max() < 1e-16
        ref = K @ sp.diags(1.0 / (theta * ml)) @ K.T
        got = sp.csr_matrix((kmk, sc, sf), shape=(N, N))
        assert abs(got - ref).max() < 1e-13 * abs(ref).max()


@pytest.mark.parametrize("n", [1, 3, 6])
def test_boundary_faces_of_the_cube(n):
    """The surface mesh of the six-tet cube: 2 triangles per boundary square,
    each face a face of its element, lying on one cube face."""
    nd, X = M.cube_mesh(n)
    faces, fe = M.boundary_faces(nd)
    assert len(faces) == 12 * n * n
    for f, e in zip(faces, fe):
        assert set(f.tolist()) < set(nd[e].tolist())
        P = X[f]
        on = [np.all(np.abs(P[:, a] - v) < 1e-14) for a in range(3) for v in (0.0, 1.0)]
        assert sum(on) == 1


def test_projection_goldens():
    """The oracle's projection pieces on the 2^3 cube reproduce the committed
    fixtures (tests/golden/projection_goldens.npz, written by
    tests/golden/make_golden.py --projection): integer arrays bit-exact,
    values to 1e-14 of each array's largest magnitude."""
    import importlib.util
    import os

    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(here, "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    want = np.load(os.path.join(here, "projection_goldens.npz"))
    got = mg.projection_goldens()
    assert sorted(got) == sorted(want.files)
    for k in want.files:
        w, g = want[k], np.asarray(got[k])
        assert g.shape == w.shape, k
        if w.dtype.kind in "iu":
            assert np.array_equal(g, w), k
        else:
            assert np.abs(g - w).max() <= 1e-14 * max(np.abs(w).max(), 1e-300), k


def test_projection_identities_on_the_unstructured_mesh(aniso_mesh):
    """On the reference's own unstructured tet mesh
    (tests/data/cube_anisotropic.msh):
    - the lumped mass sums to the volume;
    - C^T by parts with its surface terms equals C^T not by parts;
    - the second-order pattern is the structural square;
    - both row products equal scipy's triple products."""
    nd, X = aniso_mesh
    N = X.shape[0]
    f, c, _ = O.make_sparsity(nd)
    ml = O.lumped_mass(nd, nd, X, N)
    assert (ml > 0).all()
    # the mesh fills the unit cube
    assert abs(ml.sum() - 1.0) < 1e-12
    ct, _, dml, _ = O.assemble_divergence_p1(nd, X, f, c)
    faces, fe = M.boundary_faces(nd)
    ctb, rhsb, _, _ = O.assemble_divergence_p1(nd, X, f, c, by_parts=True, faces=faces, face_ele=fe)
    assert np.abs(ct - ctb).max() < 1e-12 * np.abs(ct).max()
    assert not rhsb.any()
    sf, sc = O.sparsity_secondorder(f, c)
    A = sp.csr_matrix((np.ones(len(c)), c, f), shape=(N, N))
    B = (A @ A).tocsr()
    B.sort_indices()
    assert np.array_equal(B.indptr, sf) and np.array_equal(B.indices, sc)
    w = np.random.default_rng(2).random((N, 3)) + 0.5
    cmc = O.mult_div_vector_div_T(f, c, ct, w, ct, sf, sc)
    blk = [sp.csr_matrix((ct[d], c, f), shape=(N, N)) for d in range(3)]
    ref = sum(blk[d] @ sp.diags(w[:, d]) @ blk[d].T for d in range(3))
    assert abs(sp.csr_matrix((cmc, sc, sf), shape=(N, N)) - ref).max() < 1e-14 * abs(ref).max()
    kt, kmk = O.assemble_kmk(nd, X, f, c, ml, sf, sc, theta_pg=1.0)
    K = sp.csr_matrix((kt, c, f), shape=(N, N))
    assert abs(K - K.T).max() <= 1e-15 * abs(K).max()
    ref = K @ sp.diags(1.0 / ml) @ K.T
    assert abs(sp.csr_matrix((kmk, sc, sf), shape=(N, N)) - ref).max() < 1e-13 * abs(ref).max()


def _taylor_hood(nd, X):
    nd2, n2 = O.make_global_numbering_p2(nd)
    f, c = O.make_sparsity_rect(nd, nd2)
    X2 = M.p2_coordinates(nd, nd2, X, O.tet_counts(2))
    return nd2, n2, f, c, X2


@pytest.mark.parametrize("which", ["cube", "unstructured"])
def test_taylor_hood_divergence_pins(which, aniso_mesh):
    """Divergence matrix of P2 velocity / P1 pressure (oracle only; the GPU
    kernel is the next step of this row), pinned by exact identities:
    - the pattern is make_sparsity(p_mesh, u_mesh): each pressure row holds the
      velocity nodes of its elements;
    - C_d applied to the P2 interpolant of x_e is delta_de times the P1 lumped
      pressure mass (integral of N_i), and of x_0^2 it is integral(N_i 2 x_0)
      = sum_e 2 V_e / 20 (x_i + sum_k x_k), both exact at this quadrature;
    - column sums vanish for velocity nodes off the boundary (sum_i N_i = 1);
    - by parts without surface terms equals not by parts for velocities that
      vanish on the boundary."""
    nd, X = M.cube_mesh(3) if which == "cube" else aniso_mesh
    N = X.shape[0]
    nd2, n2, f, c, X2 = _taylor_hood(nd, X)
    want = [set() for _ in range(N)]
    for e in range(len(nd)):
        for i in nd[e]:
            want[i].update(nd2[e].tolist())
    for i in range(N):
        assert c[f[i]:f[i + 1]].tolist() == sorted(want[i])
    ct = O.assemble_divergence_p2p1(nd, nd2, X, f, c)
    C3 = [sp.csr_matrix((ct[d], c, f), shape=(N, n2)) for d in range(3)]
    ml = O.lumped_mass(nd, nd, X, N)
    for d in range(3):
        for a in range(3):
            got = C3[d] @ X2[:, a]
            assert np.abs(got - (ml if a == d else 0.0)).max() < 1e-14 * ml.max()
    J = np.stack([X[nd[:, k]] - X[nd[:, 3]] for k in range(3)], axis=1)   # (E, 3, 3)
    vol = np.abs(np.linalg.det(J)) / 6.0
    ref = np.zeros(N)
    xs = X[nd, 0].sum(axis=1)
    for k in range(4):
        np.add.at(ref, nd[:, k], 2.0 * vol / 20.0 * (X[nd[:, k], 0] + xs))
    assert np.abs(C3[0] @ (X2[:, 0] ** 2) - ref).max() < 1e-14 * np.abs(ref).max()
    interior = np.ones(n2, bool)
    interior[M.boundary_nodes(X2)] = False
    for d in range(3):
        colsum = np.asarray(C3[d].sum(axis=0)).ravel()
        assert np.abs(colsum[interior]).max() < 1e-14 * np.abs(ct[d]).max()
    ctb = O.assemble_divergence_p2p1(nd, nd2, X, f, c, by_parts=True)
    u = np.prod(X2 * (1.0 - X2), axis=1) * 64.0 * (1.0 + X2[:, 1])
    u[~interior] = 0.0
    for d in range(3):
        Cb = sp.csr_matrix((ctb[d], c, f), shape=(N, n2))
        assert np.abs(Cb @ u - C3[d] @ u).max() < 1e-13 * np.abs(C3[d] @ u).max()


def _outward_normals(nd, X, xf, fe):
    a, b, c = X[xf[:, 0]], X[xf[:, 1]], X[xf[:, 2]]
    n = np.cross(a - c, b - c)
    out = (a + b + c) / 3.0 - X[nd[fe]].mean(axis=1)
    n *= np.sign(np.einsum("ij,ij->i", n, out))[:, None]
    return n / np.linalg.norm(n, axis=1)[:, None]


@pytest.mark.parametrize("which", ["cube", "unstructured"])
def test_taylor_hood_surface_terms_pins(which, aniso_mesh):
    """The by-parts surface loop for P1 pressure / P2 velocity faces, pinned by
    integration by parts, which the rules integrate exactly (element integrands
    of degree <= 2, face integrands of degree <= 3):
    - by parts with every face's terms (type 0) equals not by parts, entry by
      entry;
    - weak-Dirichlet faces (type 1 in every dimension) with the boundary values
      of a field u move exactly the face terms of u into ct_rhs:
      C_bp u - ct_rhs = C u;
    - prescribed normal flow (type 5) with g = u . n at the face nodes does the
      same through the normal-flow integral;
    - faces with a type 2, 3 or 4 in any dimension add nothing."""
    nd, X = M.cube_mesh(3) if which == "cube" else aniso_mesh
    N = X.shape[0]
    nd2, n2, f, c, X2 = _taylor_hood(nd, X)
    faces6, xf, fe = M.boundary_faces_p2(nd, nd2)
    nf = xf.shape[0]
    kw = dict(pfaces=xf, ufaces=faces6, face_ele=fe, ndglno_x=nd, coords=X, findrm=f, colm=c)
    ct = O.assemble_divergence_p2p1(nd, nd2, X, f, c)
    ctb = O.assemble_divergence_p2p1(nd, nd2, X, f, c, by_parts=True)
    full = ctb.copy()
    assert O.assemble_divergence_p2p1_faces(full, None, **kw) == 0
    for d in range(3):
        assert np.abs(full[d] - ct[d]).max() <= 1e-13 * np.abs(ct[d]).max()
    u = np.stack([np.sin(1.0 + X2[:, 0] + 2 * X2[:, 1]), X2[:, 2] ** 2 - X2[:, 0], np.cos(X2[:, 1] * X2[:, 2])],
                 axis=1)
    Cu = np.stack([sp.csr_matrix((ct[d], c, f), shape=(N, n2)) @ u[:, d] for d in range(3)]).sum(axis=0)
    Cbu = np.stack([sp.csr_matrix((ctb[d], c, f), shape=(N, n2)) @ u[:, d] for d in range(3)]).sum(axis=0)
    tol = 1e-13 * np.abs(Cu).max()
    # weak Dirichlet everywhere
    rhs = np.zeros(N)
    cw = ctb.copy()
    bv = u[faces6]  # (nf, 6, 3)
    assert O.assemble_divergence_p2p1_faces(cw, rhs, bc_type=np.ones((nf, 3), np.int32), bc_val=bv, **kw) == 0
    assert np.array_equal(cw, ctb)
    assert np.abs(Cbu - rhs - Cu).max() <= tol
    # prescribed normal flow everywhere
    nrm = _outward_normals(nd, X, xf, fe)
    g = np.zeros((nf, 6, 3))
    g[:, :, 0] = np.einsum("fjd,fd->fj", bv, nrm)
    rhs5 = np.zeros(N)
    c5 = ctb.copy()
    ty5 = np.zeros((nf, 3), np.int32)
    ty5[:, 0] = 5
    assert O.assemble_divergence_p2p1_faces(c5, rhs5, bc_type=ty5, bc_val=g, **kw) == 0
    assert np.array_equal(c5, ctb)
    assert np.abs(Cbu - rhs5 - Cu).max() <= tol
    # skipped types
    for t in (2, 3, 4):
        ty = np.zeros((nf, 3), np.int32)
        ty[:, 2] = t
        cs, rs = ctb.copy(), np.zeros(N)
        assert O.assemble_divergence_p2p1_faces(cs, rs, bc_type=ty, bc_val=bv, **kw) == 0
        assert np.array_equal(cs, ctb) and not rs.any()
