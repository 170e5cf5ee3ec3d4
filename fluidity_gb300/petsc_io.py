"""PETSc binary matrix dumps: the file DumpMatrixEquation writes after a failed
solve (femtools/Petsc_Tools.F90:1487-1504: MatView of the matrix, then VecView
of the rhs and of the initial guess) and tools/petsc_readnsolve.F90 reads.

The format is PETSc's documented binary viewer layout, big-endian:

    Mat (AIJ):  int32 MAT_FILE_CLASSID (1211216), rows, columns, nonzeros,
                int32 row lengths[rows], int32 column indices[nonzeros] (0-based,
                ascending in each row), float64 values[nonzeros]
    Vec:        int32 VEC_FILE_CLASSID (1211214), length, float64 values[length]

``petsc_matrix`` builds the matrix the reference hands to PETSc from a
csr_matrix with inactive (strong Dirichlet) rows: ghost rows carry only the
diagonal ghost_pivot, ghost columns are dropped (Petsc_Tools.F90:960-1056),
and the rhs is lifted (Solvers.F90:1072-1104).  ``petsc_readnsolve`` solves a
dump on the GPU through a pattern-only handle.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from . import femtools as ft
from ._lib import check

MAT_FILE_CLASSID = 1211216
VEC_FILE_CLASSID = 1211214


def write_matrixdump(path, findrm, colm, val, b, x0):
    """Write Mat, rhs Vec and initial-guess Vec (0-based CSR) to `path`."""
    findrm = np.asarray(findrm, dtype=np.int64)
    n = findrm.size - 1
    nnz = int(findrm[-1] - findrm[0])
    with open(path, "wb") as fh:
        np.array([MAT_FILE_CLASSID, n, n, nnz], dtype=">i4").tofile(fh)
        np.diff(findrm).astype(">i4").tofile(fh)
        np.asarray(colm, dtype=">i4").tofile(fh)
        np.asarray(val, dtype=">f8").tofile(fh)
        for v in (b, x0):
            v = np.asarray(v, dtype=np.float64)
            np.array([VEC_FILE_CLASSID, v.size], dtype=">i4").tofile(fh)
            v.astype(">f8").tofile(fh)


def read_matrixdump(path):
    """(findrm int64, colm int32, val, b, x0) of a dump; x0 is None if absent."""
    raw = open(path, "rb").read()
    off = 0

    def ints(k):
        nonlocal off
        a = np.frombuffer(raw, dtype=">i4", count=k, offset=off).astype(np.int64)
        off += 4 * k
        return a

    def doubles(k):
        nonlocal off
        a = np.frombuffer(raw, dtype=">f8", count=k, offset=off).astype(np.float64)
        off += 8 * k
        return a

    cls, m, n, nnz = ints(4)
    if cls != MAT_FILE_CLASSID:
        raise ValueError(f"{path}: not a PETSc matrix (class id {cls})")
    if m != n:
        raise ValueError(f"{path}: matrix is {m} x {n}, not square")
    lens = ints(m)
    colm = ints(nnz).astype(np.int32)
    val = doubles(nnz)
    findrm = np.zeros(m + 1, dtype=np.int64)
    np.cumsum(lens, out=findrm[1:])
    vecs = []
    while off < len(raw) and len(vecs) < 2:
        cls, k = ints(2)
        if cls != VEC_FILE_CLASSID:
            raise ValueError(f"{path}: expected a PETSc vector (class id {cls})")
        vecs.append(doubles(k))
    if not vecs:
        raise ValueError(f"{path}: no right-hand side vector")
    return findrm, colm, val, vecs[0], vecs[1] if len(vecs) > 1 else None


def petsc_matrix(findrm, colm, val, inactive, rhs, x0=None):
    """The system petsc_solve gives PETSc for a csr_matrix with inactive rows:
    (findrm, colm, val, b, x0) with ghost rows = ghost_pivot on the diagonal,
    ghost columns dropped and the rhs lifted; ghost entries of b and x0 are 0
    (the reference solves them to zero and copies the rhs in afterwards)."""
    findrm = np.asarray(findrm, dtype=np.int64)
    colm = np.asarray(colm, dtype=np.int64)
    val = np.asarray(val, dtype=np.float64)
    n = findrm.size - 1
    ghost = np.zeros(n, bool) if inactive is None else np.asarray(inactive).astype(bool)
    rows = np.repeat(np.arange(n), np.diff(findrm))
    act = ~ghost
    if ghost.any():
        # over every row's |diagonal|, ghost rows included (Petsc_Tools.F90:972-983)
        diag = np.zeros(n)
        on = colm == rows
        diag[rows[on]] = np.abs(val[on])
        mind, maxd = diag.min(), diag.max()
        pivot = np.sqrt((maxd + mind) * maxd / 2.0)
    else:
        pivot = 0.0
    xg = np.where(ghost, rhs, 0.0)
    b = np.asarray(rhs, dtype=np.float64) - np.bincount(rows, weights=val * xg[colm], minlength=n)
    b[ghost] = 0.0
    keep = act[rows] & act[colm]
    keep |= ghost[rows] & (colm == rows)
    nv = np.where(ghost[rows] & (colm == rows), pivot, val)[keep]
    nc = colm[keep].astype(np.int32)
    nf = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows[keep], minlength=n), out=nf[1:])
    x = np.zeros(n) if x0 is None else np.where(ghost, 0.0, np.asarray(x0, dtype=np.float64))
    return nf, nc, nv, b, x


class PatternHandle(ft.Mesh):
    """A handle with a CSR pattern and no elements (fl_gpu_pattern_register)."""

    def __init__(self, findrm, colm):
        self.lib = _lib.load()
        f = np.ascontiguousarray(findrm, dtype=np.int32)
        c = np.ascontiguousarray(colm, dtype=np.int32)
        self.N = int(f.size - 1)
        self.E, self.loc, self.Nx = 0, 0, 0
        h = C.c_void_p()
        check(self.lib.fl_gpu_pattern_register(self.N, f.ctypes.data, c.ctypes.data, 0, C.byref(h)),
              "fl_gpu_pattern_register")
        self.handle = h
        self.nnz = int(f[-1])
        self.ncolours = 0
        self._sparsity = None


def petsc_readnsolve(path, options):
    """Solve a matrixdump on the GPU (the counterpart of tools/petsc_readnsolve):
    returns (x, solve report) with the dump's x0 as the initial guess."""
    findrm, colm, val, b, x0 = read_matrixdump(path)
    h = PatternHandle(findrm, colm)
    x = np.zeros(b.size) if x0 is None else x0.copy()
    rep = ft.petsc_solve(h, x, val, b, options)
    h.close()
    return x, rep
