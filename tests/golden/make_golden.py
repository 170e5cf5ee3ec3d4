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
* ``projection_goldens.npz`` -- the oracle's pressure-projection pieces on the
  2^3 six-tet cube: lumped mass, divergence matrix (both forms, surface terms
  of every boundary-condition type), second-order pattern, C M_l^-1 C^T, KMK
  (theta 1 and 0.7), the projection vectors, and the P2-velocity / P1-pressure
  (Taylor-Hood) divergence pattern and element terms.

Run from the repository root in an environment that has the reference
checkout, giving the checkout's root directory as the argument:
    python tests/golden/make_golden.py <reference checkout>
(``--projection`` writes only the projection fixtures, which need no reference
files.)
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


def projection_inputs():
    """Inputs of the projection fixtures (also used by the test that checks them)."""
    from fluidity_gb300 import meshgen as M

    nd, X = M.cube_mesh(2)
    faces, fe = M.boundary_faces(nd)
    rng = np.random.default_rng(20261204)
    ty = np.zeros((len(faces), 3), np.int32)
    ty[::5, 0] = 1   # weak Dirichlet in x
    ty[1::5, 1] = 1  # weak Dirichlet in y
    ty[2::7, 2] = 2  # no_normal_flow: face skipped
    ty[3::4, 0] = 5  # prescribed normal flow
    g = rng.random((len(faces), 3, 3))
    mom = rng.random((X.shape[0], 3))
    ctr = rng.random(X.shape[0])
    dp = rng.random(X.shape[0])
    return dict(nd=nd, X=X, faces=faces, face_ele=fe, bc_type=ty, bc_val=g, mom=mom, ctr=ctr, dp=dp,
                u=M.advdif_velocity(X), bnodes=M.boundary_nodes(X))


def projection_goldens(inp=None):
    """The oracle's projection outputs on projection_inputs()."""
    from oracle import oracle as O

    inp = inp or projection_inputs()
    nd, X = inp["nd"], inp["X"]
    N = X.shape[0]
    f, c, _ = O.make_sparsity(nd)
    g = {}
    g["ml"] = O.lumped_mass(nd, nd, X, N)
    ct, rhs, dml, gml = O.assemble_divergence_p1(nd, X, f, c)
    g["ct"], g["dml"] = ct, dml
    ctb, rhsb, _, _ = O.assemble_divergence_p1(nd, X, f, c, by_parts=True, faces=inp["faces"],
                                               face_ele=inp["face_ele"], bc_type=inp["bc_type"],
                                               bc_val=inp["bc_val"])
    g["ct_by_parts"], g["ct_rhs_by_parts"] = ctb, rhsb
    sf, sc = O.sparsity_secondorder(f, c)
    g["so_findrm"], g["so_colm"] = sf, sc
    inv = np.repeat((1.0 / gml)[:, None], 3, axis=1)
    inv[inp["bnodes"]] = 0.0
    g["cmc"] = O.mult_div_vector_div_T(f, c, ct, inv, ct, sf, sc)
    for name, theta in (("kmk1", 1.0), ("kmk07", 0.7)):
        kt, kmk = O.assemble_kmk(nd, X, f, c, g["ml"], sf, sc, theta_pg=theta)
        g[name + "_kt"], g[name] = kt, kmk
    g["poisson_rhs"] = O.masslumped_poisson_rhs(f, c, ct, inp["mom"], inp["ctr"], inv, inp["u"], 0.1, 0.5)
    g["corrected_u"] = O.correct_masslumped_velocity(f, c, ct, inv, inp["dp"], inp["u"])
    # P2 velocity / P1 pressure (Taylor-Hood): pattern and element terms
    nd2, _ = O.make_global_numbering_p2(nd)
    tf, tc = O.make_sparsity_rect(nd, nd2)
    g["th_findrm"], g["th_colm"] = tf, tc
    g["th_ct"] = O.assemble_divergence_p2p1(nd, nd2, X, tf, tc)
    g["th_ct_by_parts"] = O.assemble_divergence_p2p1(nd, nd2, X, tf, tc, by_parts=True)
    return g


if __name__ == "__main__":
    if "--projection" not in sys.argv:
        if len(sys.argv) < 2 or sys.argv[1].startswith("-"):
            sys.exit("usage: make_golden.py <reference checkout> | --projection")
        main(sys.argv[1])
    np.savez_compressed(os.path.join(HERE, "projection_goldens.npz"), **projection_goldens())
    print("wrote projection fixtures to", HERE)
