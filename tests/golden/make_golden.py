"""Regenerates the committed fixtures of tests/golden/.

* ``cube_anisotropic_mesh.npz`` -- the unstructured tetrahedral unit-cube mesh
  of the reference's own test data (tests/data/cube_anisotropic.msh, gmsh 2.2
  ASCII), reduced to its tetrahedra (element type 4) as 0-based ``ndglno``
  (E, 4) int32 and ``coords`` (N, 3) float64.  It gives the parity tests a
  genuinely unstructured mesh with the reference's own node and element
  numbering.
* ``oracle_goldens.npz`` -- outputs of the CPU oracle on small inputs (sparsity,
  colouring, P2 numbering, assembled P1 Poisson / P1 advection-diffusion
  systems, a CG solve), so a change to the oracle is caught by the CPU suite.

Run from the repository root in an environment that has the reference checkout:
    python tests/golden/make_golden.py /root/reference
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def read_gmsh_tets(path: str):
    with open(path) as fh:
        lines = fh.read().split("\n")
    i = lines.index("$Nodes")
    nn = int(lines[i + 1])
    ids, xyz = [], []
    for k in range(nn):
        parts = lines[i + 2 + k].split()
        ids.append(int(parts[0]))
        xyz.append([float(v) for v in parts[1:4]])
    id2idx = {v: k for k, v in enumerate(ids)}
    j = lines.index("$Elements")
    ne = int(lines[j + 1])
    tets = []
    for k in range(ne):
        parts = [int(v) for v in lines[j + 2 + k].split()]
        etype, ntags = parts[1], parts[2]
        if etype == 4:
            tets.append([id2idx[v] for v in parts[3 + ntags:3 + ntags + 4]])
    return np.asarray(tets, dtype=np.int32), np.asarray(xyz, dtype=np.float64)


def main(ref_root: str) -> None:
    from oracle import oracle as O
    from fluidity_gb300 import meshgen as M

    nd, X = read_gmsh_tets(os.path.join(ref_root, "tests", "data", "cube_anisotropic.msh"))
    np.savez_compressed(os.path.join(HERE, "cube_anisotropic_mesh.npz"), ndglno=nd, coords=X)

    g = {}
    nd2, X2 = M.cube_mesh(2)
    f, c, ce = O.make_sparsity(nd2)
    g["cube2_findrm"], g["cube2_colm"], g["cube2_centrm"] = f, c, ce
    col, ncol = O.colour_cg1(nd2)
    g["cube2_colour"] = col
    p2, n2 = O.make_global_numbering_p2(nd2)
    g["cube2_p2"] = p2
    colu, _ = O.colour_cg1(nd)
    g["aniso_colour"] = colu
    # P1 Poisson (kappa = 1, theta = dt = 1, source f) and P1 adv-diff systems
    src = M.poisson_source(X2)
    val, rhs, st = O.assemble_advdif(ndglno_t=nd2, nt=X2.shape[0], ndglno_x=nd2, coords=X2,
                                     findrm=f, colm=c, diffusivity=1.0, source=src)
    g["cube2_poisson_val"], g["cube2_poisson_rhs"] = val, rhs
    u = M.advdif_velocity(X2)
    T0 = M.gaussian_tracer(X2)
    val, rhs, st = O.assemble_advdif(ndglno_t=nd2, nt=X2.shape[0], ndglno_x=nd2, coords=X2,
                                     findrm=f, colm=c, theta=0.5, dt=0.01, have_mass=True,
                                     velocity=u, T=T0, diffusivity=1e-3)
    g["cube2_advdif_val"], g["cube2_advdif_rhs"] = val, rhs
    np.savez_compressed(os.path.join(HERE, "oracle_goldens.npz"), **g)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
