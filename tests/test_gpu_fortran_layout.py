"""The C-ABI called the way the Fortran shim calls it: 1-based connectivity,
pattern, Dirichlet nodes and surface mesh, host arrays in Fluidity's layouts
(ndglno element-major, positions%val xyz per node, csr findrm/colm/centrm
1-based).  Every result must equal the 0-based path's bit for bit: the index
base is a convention of the boundary, not of the arithmetic.

This stands in for compiling fl_gpu_bindings.F90 (no Fortran compiler here):
the shim passes exactly these arrays through these entry points.
"""
import ctypes as C

import numpy as np
import pytest

from fluidity_gb300 import _lib
from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu


def _p(a):
    return a.ctypes.data


def test_one_based_boundary_equals_zero_based(O, aniso_mesh):
    lib = _lib.load()
    nd, X = aniso_mesh
    N = X.shape[0]
    m0 = ft.Mesh(nd, X)
    m1 = ft.Mesh(nd + 1, X, index_base=1, nodes=N)
    # pattern and colouring copied out 1-based (the csr_sparsity Fluidity caches)
    f1 = np.empty(N + 1, np.int32)
    c1 = np.empty(m1.nnz, np.int32)
    d1 = np.empty(N, np.int32)
    _lib.check(lib.fl_gpu_sparsity_copy(m1.handle, _p(f1), _p(c1), _p(d1), 1), "sparsity 1-based")
    s0 = m0.sparsity()
    assert np.array_equal(f1, s0.findrm + 1) and np.array_equal(c1, s0.colm + 1)
    assert np.array_equal(d1, s0.centrm + 1)
    of, oc, oce = O.make_sparsity(nd)
    assert np.array_equal(f1 - 1, of) and np.array_equal(c1 - 1, oc)
    col1 = np.empty(m1.E, np.int32)
    ptr1 = np.empty(m1.ncolours + 1, np.int32)
    el1 = np.empty(m1.E, np.int32)
    _lib.check(lib.fl_gpu_colouring_copy(m1.handle, _p(col1), _p(ptr1), _p(el1), 1), "colouring 1-based")
    col0, ptr0, el0 = m0.colouring()
    assert np.array_equal(col1, col0) and np.array_equal(ptr1, ptr0 + 1) and np.array_equal(el1, el0 + 1)

    # host-pointer assembly of an advection-diffusion step with by-parts advection
    u = M.advdif_velocity(X)
    T = M.gaussian_tracer(X, sigma=0.3)
    p = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True, diffusivity=0.05,
                         integrate_advection_by_parts=True)
    v0, r0 = ft.assemble_advection_diffusion_cg(m0, p, t=T, velocity=u)
    v1, r1 = ft.assemble_advection_diffusion_cg(m1, p, t=T, velocity=u)
    assert v1.tobytes() == v0.tobytes() and r1.tobytes() == r0.tobytes()

    # surface loop with 1-based faces (face_global_nodes, face_ele)
    faces, fe = M.boundary_faces(nd)
    nf = faces.shape[0]
    rng = np.random.default_rng(2)
    types = np.array([0, 1, 4], np.int32)[rng.integers(0, 3, nf)]
    b1, b2 = rng.standard_normal((nf, 3)), rng.random((nf, 3))
    ft.assemble_advection_diffusion_faces(m0, p, v0, r0, faces=faces, xfaces=faces, face_ele=fe, bc_type=types,
                                          bc_value=b1, bc_value2=b2, t=T, velocity=u)
    ft.assemble_advection_diffusion_faces(m1, p, v1, r1, faces=faces + 1, xfaces=faces + 1, face_ele=fe + 1,
                                          bc_type=types, bc_value=b1, bc_value2=b2, t=T, velocity=u,
                                          index_base=1)
    assert v1.tobytes() == v0.tobytes() and r1.tobytes() == r0.tobytes()

    # strong Dirichlet with a 1-based node list, then the solve
    bn = M.boundary_nodes(X)
    g = np.zeros(bn.size)
    ina0 = np.zeros(N, np.uint8)
    ina1 = np.zeros(N, np.uint8)
    _lib.check(lib.fl_gpu_apply_dirichlet(m0.handle, bn.size, _p(bn), 0, _p(g), _p(T), 0.01, _p(r0), _p(ina0)),
               "dirichlet 0")
    bn1 = (bn + 1).astype(np.int32)
    _lib.check(lib.fl_gpu_apply_dirichlet(m1.handle, bn.size, _p(bn1), 1, _p(g), _p(T), 0.01, _p(r1), _p(ina1)),
               "dirichlet 1")
    assert np.array_equal(ina0, ina1) and r1.tobytes() == r0.tobytes()
    opts = ft.solver_options(ksp="gmres", restart=30, rtol=1e-10, start_from_zero=True)
    x0 = np.zeros(N)
    x1 = np.zeros(N)
    rep0 = ft.petsc_solve(m0, x0, v0, r0, opts, inactive=ina0)
    rep1 = ft.petsc_solve(m1, x1, v1, r1, opts, inactive=ina1)
    assert rep0["reason"] == rep1["reason"] == 2 and rep0["iterations"] == rep1["iterations"]
    assert x0.tobytes() == x1.tobytes()

    # a pattern-only handle registered from the 1-based csr_sparsity (matrixdump path)
    ph = C.c_void_p()
    _lib.check(lib.fl_gpu_pattern_register(N, _p(f1), _p(c1), 1, C.byref(ph)), "pattern 1-based")
    try:
        xp = np.zeros(N)
        rep = np.zeros(1)
        from fluidity_gb300._lib import SolveReport
        sr = SolveReport()
        _lib.check(lib.fl_gpu_petsc_solve(ph, C.byref(opts), _p(v0), _p(ina0), _p(r0), _p(xp), C.byref(sr)),
                   "pattern solve")
        assert sr.reason == 2 and sr.iterations == rep0["iterations"]
        assert xp.tobytes() == x0.tobytes()
        del rep
    finally:
        lib.fl_gpu_mesh_destroy(ph)
    m0.close()
    m1.close()


def test_one_based_p2_numbering(O):
    nd, X = M.cube_mesh(3)
    lib = _lib.load()
    g0, n0 = ft.make_global_numbering_p2(nd)
    nd1 = np.ascontiguousarray(nd + 1, np.int32)
    out = np.empty((nd.shape[0], 10), np.int32)
    n2 = C.c_int32()
    _lib.check(lib.fl_gpu_make_global_numbering_p2(X.shape[0], nd.shape[0], _p(nd1), 1, _p(out), C.byref(n2)),
               "p2 numbering 1-based")
    assert n2.value == n0 and np.array_equal(out, g0 + 1)
