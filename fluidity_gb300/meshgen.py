"""Synthetic six-tet unit-cube meshes and the fields the benchmark workloads use.

The meshes stand in for gmsh/triangle inputs that Fluidity reads through
``read_mesh_files``: a unit cube of ``n`` hexes per side, each hex cut into six
tetrahedra along its main diagonal (Kuhn/Freudenthal split), interior vertices
jittered by a seeded, portable generator.  Layout follows Fluidity's own data
types (femtools/Fields_Data_Types.F90:61-76,187-216):

* ``ndglno`` -- element-major connectivity, ``loc`` ints per element
  (``mesh%ndglno``), 0-based here; the C-ABI accepts either base.
* ``coords`` -- ``(N, 3)`` float64, xyz interleaved per node, i.e. the memory
  of ``vector_field%val(3, N)``.

Vertex ``(i, j, k)`` has id ``i + (n+1)*(j + (n+1)*k)``; hexes are visited with
``i`` fastest; the six tets of a hex follow the permutations of (x, y, z) in
lexicographic order: ``v0, v0+e_s1, v0+e_s1+e_s2, v0+(1,1,1)``.
"""
from __future__ import annotations

import itertools

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)

#: Seeds of the workloads (jitter of the benchmark meshes, per-field
#: coefficients of the 32-field batch, jitter of the uneven mesh batch).
SEED_MESH = 20261204
SEED_FIELDS = 20261205
SEED_MESHES = 20261206


def splitmix64(seed: int, count: int, start: int = 0) -> np.ndarray:
    """Outputs ``start+1 .. start+count`` of splitmix64 seeded with ``seed``."""
    k = np.arange(start + 1, start + count + 1, dtype=np.uint64)
    with np.errstate(over="ignore"):
        z = np.uint64(seed) + k * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed: int, count: int, start: int = 0) -> np.ndarray:
    """``(u >> 11) * 2**-53`` for the splitmix64 stream: doubles in [0, 1)."""
    return (splitmix64(seed, count, start) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)


_PERMS = list(itertools.permutations(range(3)))  # lexicographic order


def cube_connectivity(n: int) -> np.ndarray:
    """``(6*n**3, 4)`` int32 connectivity of the six-tet cube (0-based)."""
    m = n + 1
    i, j, k = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    # hex order: i fastest, then j, then k
    i = i.transpose(2, 1, 0).ravel()
    j = j.transpose(2, 1, 0).ravel()
    k = k.transpose(2, 1, 0).ravel()
    v0 = (i + m * (j + m * k)).astype(np.int64)
    step = np.array([1, m, m * m], dtype=np.int64)
    tets = np.empty((n ** 3, 6, 4), dtype=np.int64)
    for t, (s1, s2, _s3) in enumerate(_PERMS):
        tets[:, t, 0] = v0
        tets[:, t, 1] = v0 + step[s1]
        tets[:, t, 2] = v0 + step[s1] + step[s2]
        tets[:, t, 3] = v0 + step.sum()
    return tets.reshape(-1, 4).astype(np.int32)


def cube_coordinates(n: int, seed: int = SEED_MESH, jitter: float = 0.2) -> np.ndarray:
    """``((n+1)**3, 3)`` float64 vertex positions.

    Three uniforms are drawn per vertex in vertex-id order (x, y, z); interior
    vertices move by ``(2u - 1) * jitter * h`` per coordinate, boundary
    vertices keep their lattice position.
    """
    m = n + 1
    h = 1.0 / n
    idx = np.arange(m ** 3, dtype=np.int64)
    i, j, k = idx % m, (idx // m) % m, idx // (m * m)
    xyz = np.stack([i, j, k], axis=1).astype(np.float64) * h
    if jitter != 0.0 and seed is not None:
        u = uniform01(seed, 3 * m ** 3).reshape(-1, 3)
        interior = (i > 0) & (i < n) & (j > 0) & (j < n) & (k > 0) & (k < n)
        xyz[interior] += (2.0 * u[interior] - 1.0) * (jitter * h)
    return xyz


def boundary_nodes(coords: np.ndarray, tol: float = 1e-14) -> np.ndarray:
    """Nodes on the faces of the unit cube (strong Dirichlet set), ascending."""
    c = coords
    on = np.any((np.abs(c) <= tol) | (np.abs(c - 1.0) <= tol), axis=1)
    return np.nonzero(on)[0].astype(np.int32)


def boundary_faces(ndglno: np.ndarray):
    """Surface mesh of a tet mesh: ``(faces (nf, 3) int32, face_ele (nf,) int32)``.

    The faces that belong to one element only, in (element, local face)
    order; local face ``f`` holds the element's vertices other than ``f`` in
    ascending local order.  ``face_ele`` is the owning element (the
    reference's ``face_ele``).
    """
    nd = np.asarray(ndglno, dtype=np.int64)
    E = nd.shape[0]
    drop = [[1, 2, 3], [0, 2, 3], [0, 1, 3], [0, 1, 2]]
    tri = np.stack([nd[:, d] for d in drop], axis=1).reshape(-1, 3)   # (4E, 3)
    key = np.sort(tri, axis=1)
    _, inv, cnt = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    once = cnt[inv.reshape(-1)] == 1
    idx = np.nonzero(once)[0]
    return tri[idx].astype(np.int32), (idx // 4).astype(np.int32)


def boundary_faces_p2(ndglno1: np.ndarray, ndglno2: np.ndarray):
    """Surface mesh of a P2 tet mesh: ``(faces (nf, 6), xfaces (nf, 3), face_ele (nf,))``.

    The faces of :func:`boundary_faces` on the P1 vertices ``ndglno1``, with
    their six P2 nodes from ``ndglno2`` in the triangle's local order (vertex
    a, edge ab, vertex b, edge ac, edge bc, vertex c for the face's local
    vertices a < b < c), and their three vertices.
    """
    xf, fe = boundary_faces(ndglno1)
    nd1 = np.asarray(ndglno1)
    nd2 = np.asarray(ndglno2)
    # local vertex ids of each face: the element's vertices other than the dropped one
    loc = np.empty((xf.shape[0], 3), dtype=np.int64)
    for k in range(3):
        loc[:, k] = np.argmax(nd1[fe] == xf[:, k:k + 1], axis=1)
    # P2 local index of vertex v and of edge (v, w) from the barycentric counts
    vid = {}
    eid = {}
    for li, c in enumerate(P2_COUNTS):
        nz = np.nonzero(c)[0]
        if len(nz) == 1:
            vid[int(nz[0])] = li
        else:
            eid[(int(nz[0]), int(nz[1]))] = li
    faces = np.empty((xf.shape[0], 6), dtype=np.int32)
    rows = np.arange(xf.shape[0])
    a, b, c = loc[:, 0], loc[:, 1], loc[:, 2]
    vmap = np.array([vid[v] for v in range(4)])
    emap = np.full((4, 4), -1)
    for (v, w), li in eid.items():
        emap[v, w] = emap[w, v] = li
    for col, idx in enumerate((vmap[a], emap[a, b], vmap[b], emap[a, c], emap[b, c], vmap[c])):
        faces[:, col] = nd2[fe, idx]
    return faces, xf, fe


def p2_coordinates(ndglno1: np.ndarray, ndglno2: np.ndarray, coords1: np.ndarray,
                   counts: np.ndarray) -> np.ndarray:
    """Positions of P2 nodes of an affine mesh: ``sum_j (count_j / 2) X_j``.

    ``counts`` is the ``(10, 4)`` barycentric count table of the local P2 node
    order (femtools/Element_Numbering.F90:389-472).
    """
    n2 = int(ndglno2.max()) + 1
    X = coords1[ndglno1]                      # (E, 4, 3)
    w = counts.astype(np.float64) / 2.0       # (10, 4)
    P = np.einsum("lj,ejd->eld", w, X)        # (E, 10, 3)
    out = np.empty((n2, 3), dtype=np.float64)
    out[ndglno2.reshape(-1)] = P.reshape(-1, 3)
    return out


def poisson_source(coords: np.ndarray) -> np.ndarray:
    """``f = sin(pi x) sin(pi y) sin(pi z)`` at the nodes."""
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    return np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z)


def advdif_velocity(coords: np.ndarray) -> np.ndarray:
    """``u = (sin 2 pi y, cos 2 pi x, 0.5 sin 2 pi z)`` at the nodes, (N, 3)."""
    x, y, z = coords[:, 0], coords[:, 1], coords[:, 2]
    return np.stack([np.sin(2 * np.pi * y), np.cos(2 * np.pi * x), 0.5 * np.sin(2 * np.pi * z)],
                    axis=1)


def gaussian_tracer(coords: np.ndarray, sigma: float = 0.1, centre=(0.5, 0.5, 0.5)) -> np.ndarray:
    """``T0 = exp(-|x - c|^2 / (2 sigma^2))``."""
    d = coords - np.asarray(centre)[None, :]
    return np.exp(-np.sum(d * d, axis=1) / (2.0 * sigma * sigma))


def cube_mesh(n: int, seed: int = SEED_MESH, jitter: float = 0.2):
    """``(ndglno (E,4) int32, coords (N,3) float64)`` of the jittered six-tet cube."""
    return cube_connectivity(n), cube_coordinates(n, seed, jitter)


def cube_counts(n: int) -> dict:
    """Closed-form sizes of the six-tet cube (P1 and P2)."""
    return {
        "E": 6 * n ** 3,
        "N1": (n + 1) ** 3,
        "nnz1": 15 * n ** 3 + 21 * n ** 2 + 9 * n + 1,
        "N2": (2 * n + 1) ** 3,
        "nnz2": 230 * n ** 3 + 138 * n ** 2 + 24 * n + 1,
    }


def batch_tracer_params(nfields: int = 32, seed: int = SEED_FIELDS):
    """Per-field ``(kappa, s)`` of the batched tracers: kappa log-uniform in
    [1e-4, 1e-1] and velocity scale s uniform in [0.5, 2], two uniforms per
    field drawn in field order (kappa first)."""
    u = uniform01(seed, 2 * nfields).reshape(nfields, 2)
    kappa = 10.0 ** (-4.0 + 3.0 * u[:, 0])
    scale = 0.5 + 1.5 * u[:, 1]
    return kappa, scale


#: Sides of the unevenly sized meshes solved alongside the batched tracers.
BATCH_MESH_SIDES = (24, 32, 40, 48, 64, 72, 88, 96)


def batch_mesh(index: int, n: int | None = None):
    """Jittered six-tet cube number ``index`` of the uneven-mesh batch (seed
    SEED_MESHES + index); ``n`` overrides its side for small tests."""
    side = BATCH_MESH_SIDES[index] if n is None else n
    return cube_mesh(side, seed=SEED_MESHES + index)


#: Barycentric counts (x2) of the ten local P2 nodes in the local node order of
#: femtools/Element_Numbering.F90:389-472 (vertex 1, edge 12, vertex 2, edge 13,
#: edge 23, vertex 3, edge 14, edge 24, edge 34, vertex 4).
P2_COUNTS = np.array([[2, 0, 0, 0], [1, 1, 0, 0], [0, 2, 0, 0], [1, 0, 1, 0], [0, 1, 1, 0],
                      [0, 0, 2, 0], [1, 0, 0, 1], [0, 1, 0, 1], [0, 0, 1, 1], [0, 0, 0, 2]],
                     dtype=np.int32)
