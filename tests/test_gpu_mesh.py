"""GPU sparsity, colouring and P2 numbering are bit-exact with the oracle's
restatement of make_sparsity, COLOURING_CG1 and make_global_numbering."""
import numpy as np
import pytest

from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu


def _meshes(O, aniso):
    out = []
    for n in (1, 2, 3, 8):
        nd, X = M.cube_mesh(n)
        out.append((f"cube{n}", nd, X))
    out.append(("aniso", aniso[0], aniso[1]))
    return out


def test_sparsity_bit_exact(O, aniso_mesh):
    for name, nd, X in _meshes(O, aniso_mesh):
        m = ft.Mesh(nd, X)
        sp = m.sparsity()
        f, c, ce = O.make_sparsity(nd)
        assert np.array_equal(sp.findrm, f), name
        assert np.array_equal(sp.colm, c), name
        assert np.array_equal(sp.centrm, ce), name
        m.close()


def test_colouring_bit_exact(O, aniso_mesh):
    for name, nd, X in _meshes(O, aniso_mesh):
        m = ft.Mesh(nd, X)
        col, ptr, el = m.colouring()
        ocol, ncol = O.colour_cg1(nd)
        assert m.ncolours == ncol, name
        assert np.array_equal(col, ocol), name
        optr, oel = O.colour_sets(ocol, ncol)
        assert np.array_equal(ptr, optr), name
        assert np.array_equal(el, oel), name
        m.close()


def test_colouring_larger_mesh(O):
    nd, X = M.cube_mesh(24)
    m = ft.Mesh(nd, X)
    col, _, _ = m.colouring()
    ocol, ncol = O.colour_cg1(nd)
    assert np.array_equal(col, ocol) and m.ncolours == ncol


def test_p2_numbering_bit_exact(O, aniso_mesh):
    for name, nd, X in _meshes(O, aniso_mesh):
        g, n2 = ft.make_global_numbering_p2(nd)
        o, on2 = O.make_global_numbering_p2(nd)
        assert n2 == on2, name
        assert np.array_equal(g, o), name


def test_p2_mesh_sparsity_and_colouring(O):
    nd, X = M.cube_mesh(3)
    nd2, n2 = O.make_global_numbering_p2(nd)
    m = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    sp = m.sparsity()
    f, c, ce = O.make_sparsity(nd2)
    assert np.array_equal(sp.findrm, f) and np.array_equal(sp.colm, c)
    col, _, _ = m.colouring()
    ocol, _ = O.colour_cg1(nd)
    assert np.array_equal(col, ocol)
    assert m.nnz == M.cube_counts(3)["nnz2"]


def test_bad_connectivity_is_an_error():
    nd, X = M.cube_mesh(2)
    bad = nd.copy()
    bad[3, 1] = X.shape[0] + 5
    with pytest.raises(ft._lib.FlError):
        ft.Mesh(bad, X, nodes=X.shape[0])


def test_unused_nodes_and_shuffled_numbering(O):
    """Ragged numbering: the nodes of a cube mesh permuted at random, plus three
    node ids that no element uses (empty CSR rows, centrm -1).  Sparsity,
    colouring and the assembled Poisson matrix match the oracle."""
    nd, X = M.cube_mesh(4)
    rng = np.random.default_rng(7)
    N0 = X.shape[0]
    perm = rng.permutation(N0 + 3)[:N0]          # old id -> new id, leaving 3 ids unused
    nd2 = perm[nd].astype(np.int32)
    N = N0 + 3
    X2 = np.zeros((N, 3))
    X2[perm] = X
    m = ft.Mesh(nd2, X2, nodes=N)
    s = m.sparsity()
    f, c, ce = O.make_sparsity(nd2, N)
    assert np.array_equal(s.findrm, f) and np.array_equal(s.colm, c) and np.array_equal(s.centrm, ce)
    unused = np.setdiff1d(np.arange(N), perm)
    assert np.all(np.diff(s.findrm)[unused] == 0) and np.all(s.centrm[unused] == -1)
    col, _, _ = m.colouring()
    ocol, ncol = O.colour_cg1(nd2, N)
    assert np.array_equal(col, ocol) and m.ncolours == ncol
    src = M.poisson_source(X2)
    p = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, source=src)
    oval, orhs, st = O.assemble_advdif(ndglno_t=nd2, nt=N, ndglno_x=nd2, coords=X2, findrm=f, colm=c,
                                       diffusivity=1.0, source=src, colours=O.colour_sets(ocol, ncol))
    assert st == 0
    scale = np.abs(oval).max()
    assert np.abs(val - oval).max() <= 1e-12 * scale
    assert np.abs(rhs - orhs).max() <= 1e-12 * np.abs(orhs).max()
    assert np.all(rhs[unused] == 0.0)
    m.close()
