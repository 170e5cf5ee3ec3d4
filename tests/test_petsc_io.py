"""PETSc binary matrixdump files (DumpMatrixEquation / petsc_readnsolve):
the byte layout against a hand-packed file, round trips, and the ghost-row
form of the system petsc_solve gives PETSc."""
import struct

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from fluidity_gb300 import meshgen as M
from fluidity_gb300 import petsc_io as P


def test_reads_hand_packed_file(tmp_path):
    # [[4, -1], [-1, 3]], b = (1, 2), x0 = (0.5, 0.25), big-endian PETSc layout
    raw = struct.pack(">4i", 1211216, 2, 2, 4) + struct.pack(">2i", 2, 2) + struct.pack(">4i", 0, 1, 0, 1)
    raw += struct.pack(">4d", 4.0, -1.0, -1.0, 3.0)
    raw += struct.pack(">2i", 1211214, 2) + struct.pack(">2d", 1.0, 2.0)
    raw += struct.pack(">2i", 1211214, 2) + struct.pack(">2d", 0.5, 0.25)
    f = tmp_path / "matrixdump"
    f.write_bytes(raw)
    findrm, colm, val, b, x0 = P.read_matrixdump(f)
    assert list(findrm) == [0, 2, 4] and list(colm) == [0, 1, 0, 1]
    assert list(val) == [4.0, -1.0, -1.0, 3.0] and list(b) == [1.0, 2.0] and list(x0) == [0.5, 0.25]
    # the writer produces the same bytes
    g = tmp_path / "again"
    P.write_matrixdump(g, findrm, colm, val, b, x0)
    assert g.read_bytes() == raw


def test_round_trip_random(tmp_path):
    rng = np.random.default_rng(4)
    A = sp.random(50, 50, density=0.1, random_state=5, format="csr") + sp.eye(50)
    A.sort_indices()
    b, x0 = rng.standard_normal(50), rng.standard_normal(50)
    f = tmp_path / "d"
    P.write_matrixdump(f, A.indptr, A.indices, A.data, b, x0)
    findrm, colm, val, b2, x02 = P.read_matrixdump(f)
    assert np.array_equal(findrm, A.indptr) and np.array_equal(colm, A.indices)
    assert np.array_equal(val, A.data) and np.array_equal(b2, b) and np.array_equal(x02, x0)


def test_rejects_other_files(tmp_path):
    f = tmp_path / "x"
    f.write_bytes(struct.pack(">4i", 1211214, 2, 2, 2))
    with pytest.raises(ValueError):
        P.read_matrixdump(f)


def test_ghost_form_solves_the_dirichlet_system(O):
    nd, X = M.cube_mesh(4)
    findrm, colm, _ = O.make_sparsity(nd)
    val, rhs, st = O.assemble_advdif(ndglno_t=nd, nt=X.shape[0], ndglno_x=nd, coords=X, findrm=findrm,
                                     colm=colm, diffusivity=1.0, source=M.poisson_source(X))
    assert st == 0
    bn = M.boundary_nodes(X)
    ina = np.zeros(X.shape[0], dtype=np.uint8)
    g = np.linspace(0.1, 0.2, bn.size)
    O.apply_dirichlet(bn, g, np.zeros(X.shape[0]), 0.0, rhs, ina)
    nf, nc, nv, b, x0 = P.petsc_matrix(findrm, colm, val, ina, rhs)
    n = X.shape[0]
    A = sp.csr_matrix((nv, nc, nf), shape=(n, n))
    # ghost rows hold only the diagonal pivot; no active row refers to a ghost
    for i in bn[:5]:
        assert list(A[i].indices) == [i]
    assert (abs(A[:, bn][np.nonzero(ina == 0)[0]]).sum()) == 0
    y = spla.spsolve(A.tocsc(), b)
    x = np.where(ina == 1, rhs, y)
    ox, its, reason, _ = O.petsc_solve(findrm.astype(np.int64), colm, val, ina, rhs, ksp="cg", rtol=1e-12)
    assert np.abs(x - ox).max() <= 1e-9 * np.abs(ox).max()
