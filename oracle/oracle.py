"""ctypes wrapper of the CPU oracle (``fl_oracle.cpp``).

TEST INFRASTRUCTURE ONLY: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` -- never by the product package.
Indices are 0-based numpy arrays; CSR row pointers are int64.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libfl_oracle.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++ -O3 -fopenmp)."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "fl_oracle.cpp"))
    ):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        _lib.orc_make_sparsity.restype = C.c_int64
        _lib.orc_triangle_detwei_sum.restype = C.c_double
    return _lib


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def num_threads() -> int:
    return lib().orc_num_threads()


def tet_quadrature(degree: int):
    """(l (ngi,4), w (ngi,), actual degree) -- Quadrature.F90:649-735."""
    l = np.zeros((16, 4))
    w = np.zeros(16)
    ngi, deg = C.c_int(), C.c_int()
    rc = lib().orc_tet_quadrature(degree, C.byref(ngi), C.byref(deg), _p(l), _p(w))
    if rc:
        raise ValueError(f"no tet quadrature of degree {degree}")
    return l[: ngi.value].copy(), w[: ngi.value].copy(), deg.value


def tet_shape(degree: int, quad_degree: int):
    """(n (loc,ngi), dn (loc,ngi,3)) -- Shape_Functions.F90:128-329."""
    n = np.zeros(10 * 16)
    dn = np.zeros(10 * 16 * 3)
    loc, ngi = C.c_int(), C.c_int()
    rc = lib().orc_tet_shape(degree, quad_degree, C.byref(loc), C.byref(ngi), _p(n), _p(dn))
    if rc:
        raise ValueError("bad shape request")
    L, G = loc.value, ngi.value
    return n[: L * G].reshape(L, G).copy(), dn[: L * G * 3].reshape(L, G, 3).copy()


def tet_counts(degree: int) -> np.ndarray:
    c = np.zeros(40, dtype=np.int32)
    loc = lib().orc_tet_counts(degree, _p(c))
    return c[: 4 * loc].reshape(loc, 4).copy()


def triangle_detwei_sum(X: np.ndarray) -> float:
    X = np.ascontiguousarray(X, dtype=np.float64)
    return lib().orc_triangle_detwei_sum(_p(X))


def transform_cache(ndglno_x: np.ndarray, coords: np.ndarray):
    E = ndglno_x.shape[0]
    nx = np.ascontiguousarray(ndglno_x, dtype=np.int32)
    X = np.ascontiguousarray(coords, dtype=np.float64)
    JT = np.zeros((E, 3, 3))
    invJ = np.zeros((E, 3, 3))
    det = np.zeros(E)
    lib().orc_transform_cache(E, _p(nx), _p(X), _p(JT), _p(invJ), _p(det))
    return JT, invJ, det


def make_sparsity(ndglno: np.ndarray, nrows: int | None = None):
    """(findrm int64 (N+1), colm int32, centrm int64) -- Sparsity_Patterns.F90:47."""
    nd = np.ascontiguousarray(ndglno, dtype=np.int32)
    E, loc = nd.shape
    if nrows is None:
        nrows = int(nd.max()) + 1
    findrm = np.zeros(nrows + 1, dtype=np.int64)
    centrm = np.zeros(nrows, dtype=np.int64)
    nnz = lib().orc_make_sparsity(nrows, E, loc, _p(nd), _p(findrm), None, 0, _p(centrm))
    colm = np.zeros(nnz, dtype=np.int32)
    lib().orc_make_sparsity(nrows, E, loc, _p(nd), _p(findrm), _p(colm), nnz, _p(centrm))
    return findrm, colm, centrm


def colour_cg1(ndglno_vertices: np.ndarray, nvert: int | None = None):
    """(colour per element, 1-based; ncolours) -- Colouring.F90:85-199."""
    nd = np.ascontiguousarray(ndglno_vertices, dtype=np.int32)
    E, nvl = nd.shape
    if nvert is None:
        nvert = int(nd.max()) + 1
    colour = np.zeros(E, dtype=np.int32)
    ncol = lib().orc_colour_cg1(E, nvl, _p(nd), nvert, _p(colour))
    return colour, ncol


def colour_sets(colour: np.ndarray, ncol: int):
    """(colour_ptr int64 (ncol+1), elements ascending within each colour)."""
    order = np.lexsort((np.arange(colour.size), colour))
    counts = np.bincount(colour, minlength=ncol + 1)[1:]
    ptr = np.zeros(ncol + 1, dtype=np.int64)
    np.cumsum(counts, out=ptr[1:])
    return ptr, order.astype(np.int32)


def make_global_numbering_p2(ndglno1: np.ndarray, nvert: int | None = None):
    """(ndglno2 (E,10) int32 0-based, N2) -- Global_Numbering.F90:291-634."""
    nd = np.ascontiguousarray(ndglno1, dtype=np.int32)
    E = nd.shape[0]
    if nvert is None:
        nvert = int(nd.max()) + 1
    out = np.zeros((E, 10), dtype=np.int32)
    n2 = lib().orc_make_global_numbering_p2(nvert, E, _p(nd), _p(out))
    return out, n2


class _Params(C.Structure):
    _fields_ = [
        ("theta", C.c_double), ("dt", C.c_double), ("beta", C.c_double),
        ("have_mass", C.c_int), ("lump_mass", C.c_int), ("have_advection", C.c_int),
        ("have_diffusivity", C.c_int), ("isotropic", C.c_int), ("have_source", C.c_int),
        ("have_absorption", C.c_int), ("quad_degree", C.c_int), ("t_degree", C.c_int),
        ("u_degree", C.c_int), ("diffusivity", C.c_double * 9), ("by_parts", C.c_int),
        ("pad", C.c_int),
    ]


def _make_params(theta, dt, beta, have_mass, lump_mass, have_advection, have_source, have_absorption,
                 diffusivity, quad_degree, t_degree, u_degree, by_parts):
    P = _Params()
    P.theta, P.dt, P.beta = theta, dt, beta
    P.have_mass, P.lump_mass = int(have_mass), int(lump_mass)
    P.have_advection = int(have_advection)
    P.have_source = int(have_source)
    P.have_absorption = int(have_absorption)
    P.quad_degree, P.t_degree, P.u_degree = quad_degree, t_degree, u_degree
    P.by_parts = int(by_parts)
    if diffusivity is None:
        P.have_diffusivity = 0
        P.isotropic = 1
    else:
        K = np.asarray(diffusivity, dtype=np.float64)
        if K.ndim == 0:
            K = np.eye(3) * float(K)
        P.have_diffusivity = 1
        P.isotropic = int(np.allclose(K, np.eye(3) * K[0, 0], rtol=0, atol=0))
        for a in range(9):
            P.diffusivity[a] = K.reshape(-1)[a]
    return P


def assemble_advdif(*, ndglno_t, nt, ndglno_x, coords, findrm, colm,
                    theta=1.0, dt=1.0, beta=0.0, have_mass=False, lump_mass=False,
                    velocity=None, ndglno_u=None, u_degree=1, T=None, source=None,
                    absorption=None, diffusivity=None, quad_degree=2, t_degree=1,
                    colours=None, nthreads=0, by_parts=False):
    """(val, rhs, status) of the element loop -- Advection_Diffusion_CG.F90:228-659.

    ``diffusivity`` is a 3x3 constant tensor (isotropic if it is a multiple of
    the identity), a scalar, or None.  ``colours`` = (colour_ptr, elements) or
    None for element order (serial build).  ``by_parts`` is
    integrate_advection_by_parts.
    """
    P = _make_params(theta, dt, beta, have_mass, lump_mass, velocity is not None, source is not None,
                     absorption is not None, diffusivity, quad_degree, t_degree, u_degree, by_parts)
    nd_t = np.ascontiguousarray(ndglno_t, dtype=np.int32)
    nd_x = np.ascontiguousarray(ndglno_x, dtype=np.int32)
    X = np.ascontiguousarray(coords, dtype=np.float64)
    E = nd_t.shape[0]
    nd_u = np.ascontiguousarray(ndglno_u if ndglno_u is not None else nd_x, dtype=np.int32)
    U = np.ascontiguousarray(velocity, dtype=np.float64) if velocity is not None else None
    Tv = np.ascontiguousarray(T, dtype=np.float64) if T is not None else None
    S = np.ascontiguousarray(source, dtype=np.float64) if source is not None else None
    A = np.ascontiguousarray(absorption, dtype=np.float64) if absorption is not None else None
    f = np.ascontiguousarray(findrm, dtype=np.int64)
    c = np.ascontiguousarray(colm, dtype=np.int32)
    val = np.zeros(c.size)
    rhs = np.zeros(nt)
    if colours is None:
        ncol, cptr, celems = 0, None, None
    else:
        cptr = np.ascontiguousarray(colours[0], dtype=np.int64)
        celems = np.ascontiguousarray(colours[1], dtype=np.int32)
        ncol = cptr.size - 1
    st = lib().orc_assemble_advdif(
        C.byref(P), E, _p(nd_t), nt, _p(nd_x), _p(X), _p(nd_u), _p(U), _p(Tv), _p(S), _p(A),
        _p(f), _p(c), _p(val), _p(rhs), ncol, _p(cptr), _p(celems), int(nthreads))
    return val, rhs, st


def assemble_advdif_faces(val, rhs, *, faces, xfaces, face_ele, ndglno_x, coords, findrm, colm,
                          bc_type, bc_value=None, bc_value2=None, theta=1.0, dt=1.0, beta=0.0,
                          velocity=None, T=None, diffusivity=None, quad_degree=2, by_parts=False):
    """The surface loop of assemble_advection_diffusion_cg (Advection_Diffusion_CG.F90:
    608-640 -> :1228-1378), added into ``val`` and ``rhs`` in place; returns the
    status.  ``faces`` (nf, floc) field nodes of each surface element in the
    triangle's local order, ``xfaces`` (nf, 3) its coordinate vertices,
    ``face_ele`` (nf,) its element; ``bc_type`` 0 none, 1 neumann,
    2 weakdirichlet, 3 internal, 4 robin; ``bc_value``/``bc_value2`` (nf, floc)
    the boundary-condition fields at the face nodes."""
    fcs = np.ascontiguousarray(faces, dtype=np.int32)
    nf, floc = fcs.shape
    P = _make_params(theta, dt, beta, False, False, velocity is not None, False, False, diffusivity,
                     quad_degree, 1 if floc == 3 else 2, 1, by_parts)
    xf = np.ascontiguousarray(xfaces, dtype=np.int32)
    fe = np.ascontiguousarray(face_ele, dtype=np.int32)
    nx = np.ascontiguousarray(ndglno_x, dtype=np.int32)
    X = np.ascontiguousarray(coords, dtype=np.float64)
    U = np.ascontiguousarray(velocity, dtype=np.float64) if velocity is not None else None
    Tv = np.ascontiguousarray(T, dtype=np.float64) if T is not None else None
    bt = np.ascontiguousarray(bc_type, dtype=np.int32)
    b1 = np.ascontiguousarray(bc_value, dtype=np.float64) if bc_value is not None else None
    b2 = np.ascontiguousarray(bc_value2, dtype=np.float64) if bc_value2 is not None else None
    f = np.ascontiguousarray(findrm, dtype=np.int64)
    c = np.ascontiguousarray(colm, dtype=np.int32)
    assert val.dtype == np.float64 and val.flags.c_contiguous and rhs.flags.c_contiguous
    return lib().orc_assemble_advdif_faces(C.byref(P), nf, floc, _p(fcs), _p(xf), _p(fe), _p(nx), _p(X), _p(U),
                                           _p(Tv), _p(bt), _p(b1), _p(b2), _p(f), _p(c), _p(val), _p(rhs))


def apply_dirichlet(nodes, g, T, dt, rhs, inactive):
    nodes = np.ascontiguousarray(nodes, dtype=np.int32)
    g = np.ascontiguousarray(g, dtype=np.float64)
    Tv = np.ascontiguousarray(T, dtype=np.float64) if T is not None else None
    lib().orc_apply_dirichlet(nodes.size, _p(nodes), _p(g), _p(Tv), C.c_double(float(dt or 0.0)), _p(rhs),
                              _p(inactive))


def petsc_solve(findrm, colm, val, inactive, rhs, x0=None, *, ksp="cg", restart=30,
                rtol=1e-10, atol=0.0, dtol=1e5, max_its=10000, start_from_zero=True,
                nthreads=0, history=False, norm="preconditioned"):
    """(x, its, reason, final_rnorm[, history]) -- Solvers.F90:111-1302 + PETSc KSP.

    ``norm`` is KSPSetNormType's choice for the convergence test:
    "preconditioned" (||B r||, PETSc's default) or, for CG, "unpreconditioned"
    (||r||, so rtol bounds the true relative residual)."""
    n = findrm.size - 1
    f = np.ascontiguousarray(findrm, dtype=np.int64)
    c = np.ascontiguousarray(colm, dtype=np.int32)
    v = np.ascontiguousarray(val, dtype=np.float64)
    ina = np.ascontiguousarray(inactive, dtype=np.uint8) if inactive is not None else None
    b = np.ascontiguousarray(rhs, dtype=np.float64)
    x = np.zeros(n) if x0 is None else np.array(x0, dtype=np.float64)
    its, reason, rn = C.c_int(), C.c_int(), C.c_double()
    cap = max_its + 64 if history else 0
    hist = np.zeros(cap) if history else None
    nh = lib().orc_petsc_solve(
        n, _p(f), _p(c), _p(v), _p(ina), _p(b), _p(x), 0 if ksp == "cg" else 1, int(restart),
        C.c_double(rtol), C.c_double(atol), C.c_double(dtol), int(max_its), int(bool(start_from_zero)),
        C.byref(its), C.byref(reason), C.byref(rn), _p(hist), cap, int(nthreads),
        1 if norm == "unpreconditioned" else 0)
    if history:
        return x, its.value, reason.value, rn.value, hist[: min(nh, cap)]
    return x, its.value, reason.value, rn.value


def csr_mult(findrm, colm, val, x):
    n = findrm.size - 1
    y = np.zeros(n)
    lib().orc_csr_mult(n, _p(np.ascontiguousarray(findrm, dtype=np.int64)),
                       _p(np.ascontiguousarray(colm, dtype=np.int32)),
                       _p(np.ascontiguousarray(val, dtype=np.float64)),
                       _p(np.ascontiguousarray(x, dtype=np.float64)), _p(y))
    return y


# ------------------------------------------------ pressure projection (P1P1) --
def lumped_mass(ndglno, ndglno_x, coords, n, degree=1, quad_degree=2):
    """compute_lumped_mass (FEFields.F90:161-214), unit density."""
    nd = np.ascontiguousarray(ndglno, dtype=np.int32)
    ndx = np.ascontiguousarray(ndglno_x, dtype=np.int32)
    X = np.ascontiguousarray(coords, dtype=np.float64)
    out = np.zeros(n)
    st = lib().orc_lumped_mass(nd.shape[0], degree, _p(nd), _p(ndx), _p(X), quad_degree, n, _p(out))
    assert st == 0, st
    return out


def assemble_divergence_p1(ndglno, coords, findrm, colm, *, by_parts=False, faces=None, face_ele=None,
                           bc_type=None, bc_val=None, quad_degree=2):
    """(ct (3, nnz), ct_rhs, div_mass_lumped, grad_mass_lumped) --
    assemble_divergence_matrix_cg (Divergence_Matrix_CG.F90:67-375), P1P1."""
    nd = np.ascontiguousarray(ndglno, dtype=np.int32)
    X = np.ascontiguousarray(coords, dtype=np.float64)
    f = np.ascontiguousarray(findrm, dtype=np.int64)
    c = np.ascontiguousarray(colm, dtype=np.int32)
    n = f.size - 1
    nf = 0 if faces is None else len(faces)
    fa = np.ascontiguousarray(faces, dtype=np.int32) if nf else None
    fe = np.ascontiguousarray(face_ele, dtype=np.int32) if nf else None
    ty = (np.ascontiguousarray(bc_type, dtype=np.int32) if bc_type is not None
          else np.zeros((nf, 3), np.int32)) if nf else None
    bv = (np.ascontiguousarray(bc_val, dtype=np.float64) if bc_val is not None
          else np.zeros((nf, 3, 3))) if nf else None
    ct = np.zeros((3, c.size))
    ct_rhs, dml, gml = np.zeros(n), np.zeros(n), np.zeros(n)
    st = lib().orc_assemble_divergence_p1(nd.shape[0], _p(nd), _p(X), n, _p(f), _p(c), quad_degree,
                                          int(bool(by_parts)), nf, _p(fa), _p(fe), _p(ty), _p(bv), _p(ct),
                                          _p(ct_rhs), _p(dml), _p(gml))
    assert st == 0, st
    return ct, ct_rhs, dml, gml


def make_sparsity_rect(nd_rows, nd_cols, nrows: int | None = None):
    """(findrm int64, colm int32) of make_sparsity(rowmesh, colmesh)
    (Sparsity_Patterns.F90:47-85): rows of the row mesh, columns of the
    column mesh's nodes sharing an element, ascending."""
    r = np.ascontiguousarray(nd_rows, dtype=np.int32)
    c = np.ascontiguousarray(nd_cols, dtype=np.int32)
    E, lr = r.shape
    lc = c.shape[1]
    if nrows is None:
        nrows = int(r.max()) + 1
    fn = lib().orc_make_sparsity_rect
    fn.restype = C.c_int64
    fn.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p,
                   C.c_int64]
    f = np.zeros(nrows + 1, dtype=np.int64)
    nnz = fn(nrows, E, lr, _p(r), lc, _p(c), _p(f), None, 0)
    colm = np.zeros(nnz, dtype=np.int32)
    fn(nrows, E, lr, _p(r), lc, _p(c), _p(f), _p(colm), nnz)
    return f, colm


def assemble_divergence_p2p1(ndglno_p, ndglno_u, coords, findrm, colm, *, by_parts=False, quad_degree=4):
    """ct (3, nnz) -- the element terms of assemble_divergence_matrix_cg
    (Divergence_Matrix_CG.F90:67-375) for P1 pressure (rows, the coordinate
    mesh's vertices) and P2 velocity (columns) on the pattern of
    make_sparsity_rect."""
    p_ = np.ascontiguousarray(ndglno_p, dtype=np.int32)
    u_ = np.ascontiguousarray(ndglno_u, dtype=np.int32)
    X = np.ascontiguousarray(coords, dtype=np.float64)
    f = np.ascontiguousarray(findrm, dtype=np.int64)
    c = np.ascontiguousarray(colm, dtype=np.int32)
    fn = lib().orc_assemble_divergence_p2p1
    fn.restype = C.c_int
    fn.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                   C.c_int, C.c_void_p]
    ct = np.zeros((3, c.size))
    st = fn(p_.shape[0], _p(p_), _p(u_), _p(X), f.size - 1, _p(f), _p(c), quad_degree, int(bool(by_parts)),
            _p(ct))
    assert st == 0, st
    return ct


def assemble_divergence_p2p1_faces(ct, ct_rhs, *, pfaces, ufaces, face_ele, ndglno_x, coords, findrm, colm,
                                   bc_type=None, bc_val=None, quad_degree=4):
    """Adds the by-parts surface terms of assemble_divergence_matrix_cg
    (Divergence_Matrix_CG.F90:312-366) for P1 pressure / P2 velocity faces to
    ct (3, nnz) and ct_rhs (pressure nodes, or None)."""
    pf = np.ascontiguousarray(pfaces, dtype=np.int32)
    uf = np.ascontiguousarray(ufaces, dtype=np.int32)
    fe = np.ascontiguousarray(face_ele, dtype=np.int32)
    nd = np.ascontiguousarray(ndglno_x, dtype=np.int32)
    X = np.ascontiguousarray(coords, dtype=np.float64)
    f = np.ascontiguousarray(findrm, dtype=np.int64)
    c = np.ascontiguousarray(colm, dtype=np.int32)
    nf = pf.shape[0]
    ty = np.ascontiguousarray(bc_type if bc_type is not None else np.zeros((nf, 3)), dtype=np.int32)
    bv = None if bc_val is None else np.ascontiguousarray(bc_val, dtype=np.float64)
    assert ct.flags.c_contiguous and ct.dtype == np.float64
    fn = lib().orc_assemble_divergence_p2p1_faces
    fn.restype = C.c_int
    fn.argtypes = [C.c_int] + [C.c_void_p] * 5 + [C.c_int, C.c_void_p, C.c_void_p, C.c_int] + [C.c_void_p] * 4
    return fn(nf, _p(pf), _p(uf), _p(fe), _p(nd), _p(X), f.size - 1, _p(f), _p(c), quad_degree, _p(ty),
              _p(bv) if bv is not None else None, _p(ct), _p(ct_rhs) if ct_rhs is not None else None)


def sparsity_secondorder(findrm, colm):
    """(findrm int64, colm int32) of make_sparsity_transpose (Sparsity_Patterns.F90:87-148)."""
    f = np.ascontiguousarray(findrm, dtype=np.int64)
    c = np.ascontiguousarray(colm, dtype=np.int32)
    n = f.size - 1
    lib().orc_sparsity_secondorder.restype = C.c_int64
    of = np.zeros(n + 1, dtype=np.int64)
    nnz = lib().orc_sparsity_secondorder(n, _p(f), _p(c), _p(of), None, 0)
    oc = np.zeros(nnz, dtype=np.int32)
    lib().orc_sparsity_secondorder(n, _p(f), _p(c), _p(of), _p(oc), nnz)
    return of, oc


def mult_div_vector_div_T(findrm, colm, a, w, b, pf, pc):
    """mult_div_vector_div_T (Sparse_Matrices_Fields.F90:590-671); a, b: (ndim, nnz); w: (ncols, ndim)."""
    a = np.ascontiguousarray(a, dtype=np.float64)
    ndim = a.shape[0]
    out = np.zeros(len(pc))
    lib().orc_mult_div_vector_div_T(len(findrm) - 1, ndim, _p(np.ascontiguousarray(findrm, dtype=np.int64)),
                                    _p(np.ascontiguousarray(colm, dtype=np.int32)), _p(a),
                                    _p(np.ascontiguousarray(w, dtype=np.float64)),
                                    _p(np.ascontiguousarray(b, dtype=np.float64)),
                                    _p(np.ascontiguousarray(pf, dtype=np.int64)),
                                    _p(np.ascontiguousarray(pc, dtype=np.int32)), _p(out))
    return out


def mult_div_invscalar_div_T(findrm, colm, a, s, b, pf, pc):
    """mult_div_invscalar_div_T (Sparse_Matrices_Fields.F90:673-748), a and b on one pattern."""
    f = np.ascontiguousarray(findrm, dtype=np.int64)
    c = np.ascontiguousarray(colm, dtype=np.int32)
    out = np.zeros(len(pc))
    lib().orc_mult_div_invscalar_div_T(len(f) - 1, _p(f), _p(c), _p(np.ascontiguousarray(a, dtype=np.float64)),
                                       _p(np.ascontiguousarray(s, dtype=np.float64)), _p(f), _p(c),
                                       _p(np.ascontiguousarray(b, dtype=np.float64)),
                                       _p(np.ascontiguousarray(pf, dtype=np.int64)),
                                       _p(np.ascontiguousarray(pc, dtype=np.int32)), _p(out))
    return out


def simplex_tensor(X):
    """simplex_tensor (Metric_tools.F90:852-941) of one simplex; X is (dim+1, dim)."""
    X = np.ascontiguousarray(X, dtype=np.float64)
    dim = X.shape[1]
    m = np.zeros((dim, dim))
    lib().orc_simplex_tensor(dim, _p(X), _p(m))
    return m


def edge_length_metric(m):
    """edge_length_from_eigenvalue_metric (Metric_tools.F90:157-164)."""
    m = np.ascontiguousarray(m, dtype=np.float64)
    out = np.zeros_like(m)
    lib().orc_edge_length_metric(m.shape[0], _p(m), _p(out))
    return out


def assemble_kmk(ndglno, coords, findrm, colm, p_masslump, so_findrm, so_colm, theta_pg=1.0, quad_degree=2):
    """(kt, kmk) -- assemble_kmk_matrix (Momentum_CG.F90:2707-2766)."""
    nd = np.ascontiguousarray(ndglno, dtype=np.int32)
    f = np.ascontiguousarray(findrm, dtype=np.int64)
    c = np.ascontiguousarray(colm, dtype=np.int32)
    kt = np.zeros(c.size)
    kmk = np.zeros(len(so_colm))
    st = lib().orc_assemble_kmk(nd.shape[0], _p(nd), _p(np.ascontiguousarray(coords, dtype=np.float64)),
                                f.size - 1, _p(f), _p(c), quad_degree, C.c_double(theta_pg),
                                _p(np.ascontiguousarray(p_masslump, dtype=np.float64)),
                                _p(np.ascontiguousarray(so_findrm, dtype=np.int64)),
                                _p(np.ascontiguousarray(so_colm, dtype=np.int32)), _p(kt), _p(kmk))
    assert st == 0, st
    return kt, kmk


def _block(findrm, colm, v):
    import scipy.sparse as sp
    n = len(findrm) - 1
    return sp.csr_matrix((v, np.asarray(colm), np.asarray(findrm)), shape=(n, n))


def masslumped_poisson_rhs(findrm, colm, ctp, mom_rhs, ct_rhs, inverse_masslump, velocity, dt, theta_pg):
    """assemble_masslumped_poisson_rhs (Momentum_CG.F90:2670-2705); vector fields are (N, 3)."""
    lm = mom_rhs * inverse_masslump + velocity * (1.0 / dt / theta_pg)
    y = np.zeros(len(findrm) - 1)
    for d in range(3):
        y += _block(findrm, colm, ctp[d]) @ lm[:, d]
    return -y + ct_rhs * (1.0 / dt / theta_pg)


def correct_masslumped_velocity(findrm, colm, ct, inverse_masslump, delta_p, velocity):
    """correct_masslumped_velocity (Momentum_CG.F90:2544-2575): u += M_l^-1 C^T dp."""
    u = np.array(velocity, dtype=np.float64)
    for d in range(3):
        u[:, d] += (_block(findrm, colm, ct[d]).T @ delta_p) * inverse_masslump[:, d]
    return u
