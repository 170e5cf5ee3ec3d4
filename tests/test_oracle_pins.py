"""Pins of the CPU oracle against the reference's own known-answer tests.

* femtools/tests/test_quadrature.F90 -- every tet rule integrates x^p exactly
  for p <= degree (answer p!/(p+3)! on the unit simplex);
* femtools/tests/test_shape_functions.F90 -- the Lagrange basis reproduces
  monomials up to its degree, values and first derivatives (eps 1e-12);
* femtools/tests/test_jacobian.F90 -- sum(detwei) = sqrt(2) for the triangle
  (0,0,0),(2,0,0),(0,1,1);
* femtools/tests/test_colouring.F90 -- colour count <= max degree + 1, no two
  neighbours share a colour, colour sets partition the elements.
"""
import math

import numpy as np
import pytest

from fluidity_gb300 import meshgen as M


def simplex_answer(p, dim=3):
    if p < 0:
        return 0.0
    return math.factorial(p) / math.factorial(p + dim)


@pytest.mark.parametrize("degree", [1, 2, 3, 4])
def test_quadrature_exactness(O, degree):
    l, w, actual = O.tet_quadrature(degree)
    assert actual == degree
    for p in range(degree + 1):
        got = float(np.sum(w * l[:, 0] ** p))
        assert abs(got - simplex_answer(p)) <= 1e-14, (degree, p, got)


def test_quadrature_point_counts(O):
    assert [O.tet_quadrature(d)[0].shape[0] for d in (1, 2, 3, 4)] == [1, 4, 5, 11]


@pytest.mark.parametrize("degree", [1, 2])
def test_shape_function_exactness(O, degree):
    n, dn = O.tet_shape(degree, 4)
    l, w, _ = O.tet_quadrature(4)
    counts = O.tet_counts(degree)
    nodes_l = counts / degree  # local coordinates of the nodes
    for p in range(degree + 1):
        f = nodes_l[:, 0] ** p
        val = float(np.sum(f[:, None] * n * w[None, :]))
        assert abs(val - simplex_answer(p)) < 1e-12
        dval = float(np.sum(f[:, None] * dn[:, :, 0] * w[None, :]))
        assert abs(dval - p * simplex_answer(p - 1)) < 1e-12


def test_p2_local_numbering(O):
    c = O.tet_counts(2)
    assert c.tolist() == [[2, 0, 0, 0], [1, 1, 0, 0], [0, 2, 0, 0], [1, 0, 1, 0], [0, 1, 1, 0],
                          [0, 0, 2, 0], [1, 0, 0, 1], [0, 1, 0, 1], [0, 0, 1, 1], [0, 0, 0, 2]]


def test_jacobian_known_answer(O):
    X = np.array([[0.0, 0.0, 0.0], [2.0, 0.0, 0.0], [0.0, 1.0, 1.0]])
    assert abs(O.triangle_detwei_sum(X) - math.sqrt(2.0)) <= 1e-10


def _check_colouring(nd, colour, ncol):
    E = nd.shape[0]
    nv = int(nd.max()) + 1
    # element graph: elements sharing a vertex
    rows = np.repeat(np.arange(E), 4)
    inc = np.zeros((nv, 0)).tolist()
    lists = [[] for _ in range(nv)]
    for e in range(E):
        for v in nd[e]:
            lists[v].append(e)
    maxdeg = 0
    for e in range(E):
        nb = set()
        for v in nd[e]:
            nb.update(lists[v])
        maxdeg = max(maxdeg, len(nb))
        for f in nb:
            if f < e:
                assert colour[f] != colour[e]
    assert ncol <= maxdeg + 1
    assert colour.min() == 1 and colour.max() == ncol
    del rows, inc


def test_colouring_valid_cube(O):
    nd, _ = M.cube_mesh(4)
    colour, ncol = O.colour_cg1(nd)
    _check_colouring(nd, colour, ncol)
    ptr, el = O.colour_sets(colour, ncol)
    assert int(el.astype(np.int64).sum()) == sum(range(nd.shape[0]))  # partition (sum-of-ids)


def test_colouring_valid_unstructured(O, aniso_mesh):
    nd, _ = aniso_mesh
    colour, ncol = O.colour_cg1(nd)
    _check_colouring(nd, colour, ncol)


def test_colouring_greedy_definition(O, aniso_mesh):
    """c(e) = lowest colour not used by a lower-numbered vertex neighbour."""
    nd, _ = aniso_mesh
    colour, _ = O.colour_cg1(nd)
    lists = [[] for _ in range(int(nd.max()) + 1)]
    for e in range(nd.shape[0]):
        for v in nd[e]:
            lists[v].append(e)
    for e in range(0, nd.shape[0], 7):
        used = {colour[f] for v in nd[e] for f in lists[v] if f < e}
        c = 1
        while c in used:
            c += 1
        assert colour[e] == c


@pytest.mark.parametrize("n", [1, 2, 3, 5])
def test_sparsity_closed_forms(O, n):
    nd, X = M.cube_mesh(n)
    f, c, ce = O.make_sparsity(nd)
    cnt = M.cube_counts(n)
    assert c.size == cnt["nnz1"]
    for i in range(f.size - 1):
        row = c[f[i]:f[i + 1]]
        assert np.all(np.diff(row) > 0)
        assert row[ce[i] - f[i]] == i
    nd2, n2 = O.make_global_numbering_p2(nd)
    assert n2 == cnt["N2"]
    f2, c2, _ = O.make_sparsity(nd2)
    assert c2.size == cnt["nnz2"]


def test_p2_numbering_order(O, aniso_mesh):
    """Vertices first-touch, then edges in (old node, neighbour) ascending order."""
    nd, _ = aniso_mesh
    nd2, n2 = O.make_global_numbering_p2(nd)
    nv = int(nd.max()) + 1
    vpos = [0, 2, 5, 9]
    # first-touch: the sequence of new vertex ids in element-major order first
    # appears in increasing order 0, 1, 2, ...
    seen, nxt = set(), 0
    for e in range(nd.shape[0]):
        for a in range(4):
            v = nd2[e, vpos[a]]
            if v not in seen:
                assert v == nxt
                seen.add(v)
                nxt += 1
    assert nxt == nv
    # edges: key (min old, max old) -> number strictly increasing in key order
    epos = {(0, 1): 1, (0, 2): 3, (1, 2): 4, (0, 3): 6, (1, 3): 7, (2, 3): 8}
    num = {}
    for e in range(nd.shape[0]):
        for (a, b), p in epos.items():
            k = (min(nd[e, a], nd[e, b]), max(nd[e, a], nd[e, b]))
            if k in num:
                assert num[k] == nd2[e, p]
            num[k] = nd2[e, p]
    keys = sorted(num)
    vals = [num[k] for k in keys]
    assert vals == list(range(nv, nv + len(keys)))
    assert n2 == nv + len(keys)


def test_oracle_goldens(O, goldens):
    nd, X = M.cube_mesh(2)
    f, c, ce = O.make_sparsity(nd)
    assert np.array_equal(f, goldens["cube2_findrm"]) and np.array_equal(c, goldens["cube2_colm"])
    col, _ = O.colour_cg1(nd)
    assert np.array_equal(col, goldens["cube2_colour"])
    p2, _ = O.make_global_numbering_p2(nd)
    assert np.array_equal(p2, goldens["cube2_p2"])
    val, rhs, st = O.assemble_advdif(ndglno_t=nd, nt=X.shape[0], ndglno_x=nd, coords=X, findrm=f,
                                     colm=c, diffusivity=1.0, source=M.poisson_source(X))
    assert st == 0
    np.testing.assert_allclose(val, goldens["cube2_poisson_val"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(rhs, goldens["cube2_poisson_rhs"], rtol=0, atol=1e-15)


def test_unstructured_colour_golden(O, aniso_mesh, goldens):
    nd, _ = aniso_mesh
    col, _ = O.colour_cg1(nd)
    assert np.array_equal(col, goldens["aniso_colour"])
