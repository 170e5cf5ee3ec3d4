"""Pins of the oracle's surface loop of assemble_advection_diffusion_cg
(Advection_Diffusion_CG.F90:608-640, :1228-1378) and of the element
advection integrated by parts (:1019-1057), by exact identities:

* a Neumann flux g adds int_{boundary} N_i g: summed over i it is the
  surface integral of g (6 g for a constant on the unit cube, 3 for g = x);
* the Robin matrix is g2 times the boundary mass matrix (summing to 6 g2),
  and its product with t leaves the rhs;
* integration by parts: the by-parts element matrix plus the face term of
  every surface element equals the not-by-parts element matrix, for any beta
  (exact when the face rule integrates the cubic N_i N_j u.n, degree 4);
  and weak Dirichlet faces move the face term to the rhs with theta (g - t);
* a weak Dirichlet face with a diffusivity is the reference's FLExit;
* internal faces are skipped.
Each identity is checked on the jittered cube and on the reference's
unstructured mesh (tests/data/cube_anisotropic.msh).
"""
import numpy as np
import pytest
import scipy.sparse as sp

from fluidity_gb300 import meshgen as M


def _mesh(kind, aniso_mesh):
    return M.cube_mesh(3) if kind == "cube" else aniso_mesh


def _surface(nd, X):
    faces, fe = M.boundary_faces(nd)
    return faces, faces.copy(), fe


def _zero(f):
    return np.zeros(f[-1]), None


@pytest.mark.parametrize("kind", ["cube", "aniso"])
def test_neumann_flux_integrates_the_boundary(O, aniso_mesh, kind):
    nd, X = _mesh(kind, aniso_mesh)
    f, c, _ = O.make_sparsity(nd)
    faces, xf, fe = _surface(nd, X)
    nf = faces.shape[0]
    for g_of, total in ((lambda x: np.ones(len(x)), 6.0), (lambda x: x[:, 0], 3.0)):
        val = np.zeros(c.size)
        rhs = np.zeros(X.shape[0])
        bc = g_of(X[faces.reshape(-1)]).reshape(nf, 3)
        st = O.assemble_advdif_faces(val, rhs, faces=faces, xfaces=xf, face_ele=fe, ndglno_x=nd, coords=X,
                                     findrm=f, colm=c, bc_type=np.ones(nf, np.int32), bc_value=bc,
                                     diffusivity=1.0, theta=0.5, dt=0.1)
        assert st == 0
        assert not val.any()
        assert rhs.sum() == pytest.approx(total, rel=1e-13)
        # only boundary rows change
        inner = np.setdiff1d(np.arange(X.shape[0]), faces.reshape(-1))
        assert not rhs[inner].any()


@pytest.mark.parametrize("kind", ["cube", "aniso"])
def test_robin_is_the_boundary_mass_matrix(O, aniso_mesh, kind):
    nd, X = _mesh(kind, aniso_mesh)
    f, c, _ = O.make_sparsity(nd)
    faces, xf, fe = _surface(nd, X)
    nf = faces.shape[0]
    n = X.shape[0]
    theta, dt, g2 = 0.5, 0.2, 1.7
    T = 0.25 + X[:, 1]
    val = np.zeros(c.size)
    rhs = np.zeros(n)
    st = O.assemble_advdif_faces(val, rhs, faces=faces, xfaces=xf, face_ele=fe, ndglno_x=nd, coords=X, findrm=f,
                                 colm=c, bc_type=np.full(nf, 4, np.int32), bc_value=np.zeros((nf, 3)),
                                 bc_value2=np.full((nf, 3), g2), diffusivity=1.0, theta=theta, dt=dt, T=T)
    assert st == 0
    A = sp.csr_matrix((val, c, f), shape=(n, n))
    assert A.sum() == pytest.approx(dt * theta * g2 * 6.0, rel=1e-13)
    assert abs(A - A.T).max() < 1e-15
    # rhs = -(g2 boundary mass) T = -A T / (dt theta)
    assert np.abs(rhs + A @ T / (dt * theta)).max() < 1e-14


@pytest.mark.parametrize("kind", ["cube", "aniso"])
@pytest.mark.parametrize("beta", [0.0, 1.0, 0.3])
def test_advection_by_parts_plus_faces_equals_not_by_parts(O, aniso_mesh, kind, beta):
    nd, X = _mesh(kind, aniso_mesh)
    n = X.shape[0]
    f, c, _ = O.make_sparsity(nd)
    faces, xf, fe = _surface(nd, X)
    nf = faces.shape[0]
    u = M.advdif_velocity(X) + np.array([0.3, -0.2, 0.1]) * X  # nonzero divergence
    T = M.gaussian_tracer(X, sigma=0.3)
    kw = dict(ndglno_t=nd, nt=n, ndglno_x=nd, coords=X, findrm=f, colm=c, theta=0.5, dt=0.1, beta=beta,
              velocity=u, T=T, quad_degree=4)
    v0, r0, st0 = O.assemble_advdif(**kw)
    v1, r1, st1 = O.assemble_advdif(by_parts=True, **kw)
    assert st0 == st1 == 0
    assert np.abs(v1 - v0).max() > 1e-6  # the forms differ element by element
    st = O.assemble_advdif_faces(v1, r1, faces=faces, xfaces=xf, face_ele=fe, ndglno_x=nd, coords=X, findrm=f,
                                 colm=c, bc_type=np.zeros(nf, np.int32), velocity=u, T=T, theta=0.5, dt=0.1,
                                 beta=beta, quad_degree=4, by_parts=True)
    assert st == 0
    assert np.abs(v1 - v0).max() <= 1e-13 * np.abs(v0).max()
    assert np.abs(r1 - r0).max() <= 1e-13 * np.abs(r0).max()


def test_weak_dirichlet_advection_face_moves_to_the_rhs(O):
    """A weak Dirichlet face adds -theta A_f (g - t) to the rhs instead of
    dt theta A_f to the matrix; with g = t only -A_f t remains."""
    nd, X = M.cube_mesh(3)
    n = X.shape[0]
    f, c, _ = O.make_sparsity(nd)
    faces, xf, fe = _surface(nd, X)
    nf = faces.shape[0]
    u = M.advdif_velocity(X)
    T = M.gaussian_tracer(X, sigma=0.3)
    common = dict(faces=faces, xfaces=xf, face_ele=fe, ndglno_x=nd, coords=X, findrm=f, colm=c, velocity=u, T=T,
                  theta=0.5, dt=0.1, by_parts=True)
    v_none, r_none = np.zeros(c.size), np.zeros(n)
    assert O.assemble_advdif_faces(v_none, r_none, bc_type=np.zeros(nf, np.int32), **common) == 0
    v_wd, r_wd = np.zeros(c.size), np.zeros(n)
    assert O.assemble_advdif_faces(v_wd, r_wd, bc_type=np.full(nf, 2, np.int32), bc_value=T[faces], **common) == 0
    assert not v_wd.any()
    assert np.abs(r_wd - r_none).max() < 1e-15
    A_f = sp.csr_matrix((v_none / 0.05, c, f), shape=(n, n))
    g = T + 0.1
    v2, r2 = np.zeros(c.size), np.zeros(n)
    assert O.assemble_advdif_faces(v2, r2, bc_type=np.full(nf, 2, np.int32), bc_value=g[faces], **common) == 0
    assert np.abs(r2 - (r_none - 0.5 * (A_f @ (g - T)))).max() < 1e-14


def test_weak_dirichlet_with_diffusivity_and_internal_faces(O):
    nd, X = M.cube_mesh(2)
    f, c, _ = O.make_sparsity(nd)
    faces, xf, fe = _surface(nd, X)
    nf = faces.shape[0]
    common = dict(faces=faces, xfaces=xf, face_ele=fe, ndglno_x=nd, coords=X, findrm=f, colm=c,
                  bc_value=np.ones((nf, 3)), diffusivity=1.0)
    val, rhs = np.zeros(c.size), np.zeros(X.shape[0])
    assert O.assemble_advdif_faces(val, rhs, bc_type=np.full(nf, 2, np.int32), **common) != 0  # FLExit
    val, rhs = np.zeros(c.size), np.zeros(X.shape[0])
    assert O.assemble_advdif_faces(val, rhs, bc_type=np.full(nf, 3, np.int32), **common) == 0
    assert not val.any() and not rhs.any()


def test_p2_neumann_and_robin(O):
    """P2 faces (six nodes, degree-4 rule): a constant flux integrates to 6 g
    and the Robin matrix sums to 6 g2 (the P2 face functions sum to one)."""
    nd, X = M.cube_mesh(2)
    nd2, n2 = O.make_global_numbering_p2(nd)
    f, c, _ = O.make_sparsity(nd2)
    faces6, xf, fe = M.boundary_faces_p2(nd, nd2)
    nf = faces6.shape[0]
    val, rhs = np.zeros(c.size), np.zeros(n2)
    st = O.assemble_advdif_faces(val, rhs, faces=faces6, xfaces=xf, face_ele=fe, ndglno_x=nd, coords=X, findrm=f,
                                 colm=c, bc_type=np.full(nf, 4, np.int32), bc_value=np.full((nf, 6), 2.0),
                                 bc_value2=np.full((nf, 6), 0.5), diffusivity=1.0, quad_degree=4)
    assert st == 0
    assert rhs.sum() == pytest.approx(12.0, rel=1e-13)
    assert val.sum() == pytest.approx(3.0, rel=1e-13)
