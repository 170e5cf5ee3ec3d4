"""GPU element assembly against the oracle's restatement of
assemble_advection_diffusion_cg, entry by entry.

Tolerance (floating point): |a - a_ref| <= 1e-12 * max_j |a_ref(i, j)| per row
for the matrix, and the same row scale for the right-hand side.
"""
import numpy as np
import pytest

from conftest import row_scaled_error
from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu
TOL = 1e-12


def _oracle(O, nd, X, ndt, nt, f, c, colours=None, **kw):
    val, rhs, st = O.assemble_advdif(ndglno_t=ndt, nt=nt, ndglno_x=nd, coords=X, findrm=f, colm=c,
                                     colours=colours, **kw)
    assert st == 0
    return val, rhs


def _compare(val, rhs, oval, orhs, f, tol=TOL):
    assert row_scaled_error(val, oval, f) <= tol
    # rhs scaled by the largest |rhs| of the row's neighbourhood
    scale = max(np.abs(orhs).max(), 1e-300)
    assert np.abs(rhs - orhs).max() <= tol * scale


CASES = {
    "poisson": dict(diffusivity=1.0, source=True),
    "anisotropic": dict(diffusivity=np.diag([1.0, 1.0, 1e-3]), source=True),
    "advdif": dict(theta=0.5, dt=0.01, have_mass=True, velocity=True, T=True, diffusivity=1e-3),
    "advdif_beta1": dict(theta=0.5, dt=0.01, have_mass=True, velocity=True, T=True,
                         diffusivity=1e-3, beta=1.0),
    "advdif_by_parts": dict(theta=0.5, dt=0.01, have_mass=True, velocity=True, T=True,
                            diffusivity=1e-3, beta=0.3, by_parts=True),
    "lumped_absorption": dict(theta=1.0, dt=0.1, have_mass=True, lump_mass=True, absorption=True,
                              T=True, diffusivity=0.5, source=True),
    "mass_only": dict(have_mass=True, source=True),
    # the double-float P1 advection-diffusion kernel: lumped mass with a
    # divergence term, a diagonal kappa with a source, no diffusion
    "advdif_lumped_beta": dict(theta=0.5, dt=0.01, have_mass=True, lump_mass=True, velocity=True, T=True,
                               diffusivity=1e-3, beta=0.5),
    "advdif_diag_kappa_source": dict(theta=1.0, dt=0.05, have_mass=True, velocity=True, T=True,
                                     diffusivity=np.diag([1e-2, 1e-3, 1e-4]), source=True),
    "advection_only_by_parts": dict(theta=1.0, dt=0.1, have_mass=True, velocity=True, T=True, beta=0.2,
                                    by_parts=True),
}


def _fields(X, case):
    out = {}
    for k, v in case.items():
        if v is True and k in ("source", "velocity", "T", "absorption"):
            out[k] = {"source": M.poisson_source(X), "velocity": M.advdif_velocity(X),
                      "T": M.gaussian_tracer(X), "absorption": 1.0 + X[:, 0]}[k]
        else:
            out[k] = v
    return out


def _params(case, quad_degree):
    return ft.advdif_params(theta=case.get("theta", 1.0), dt=case.get("dt", 1.0),
                            beta=case.get("beta", 0.0), have_mass=case.get("have_mass", False),
                            lump_mass=case.get("lump_mass", False),
                            have_advection="velocity" in case,
                            diffusivity=case.get("diffusivity"), have_source="source" in case,
                            have_absorption="absorption" in case, quad_degree=quad_degree,
                            integrate_advection_by_parts=case.get("by_parts", False))


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("mesh", ["cube4", "aniso"])
def test_p1_assembly_matches_oracle(O, aniso_mesh, name, mesh):
    nd, X = M.cube_mesh(4) if mesh == "cube4" else aniso_mesh
    case = CASES[name]
    fl = _fields(X, case)
    m = ft.Mesh(nd, X)
    f, c, _ = O.make_sparsity(nd)
    ocol, ncol = O.colour_cg1(nd)
    colours = O.colour_sets(ocol, ncol)
    kw = {k: v for k, v in fl.items() if k not in ("theta", "dt", "beta", "have_mass", "lump_mass", "by_parts")}
    kw.update({k: case[k] for k in ("theta", "dt", "beta", "have_mass", "lump_mass", "by_parts") if k in case})
    oval, orhs = _oracle(O, nd, X, nd, X.shape[0], f, c, colours=colours, **kw)
    val, rhs = ft.assemble_advection_diffusion_cg(m, _params(case, 2), t=fl.get("T"),
                                                  velocity=fl.get("velocity"),
                                                  source=fl.get("source"),
                                                  absorption=fl.get("absorption"))
    _compare(val, rhs, oval, orhs, f)


@pytest.mark.parametrize("qdeg", [1, 3, 4])
@pytest.mark.parametrize("name", ["advdif", "advdif_by_parts"])
def test_p1_advdif_quadrature_degrees(O, name, qdeg):
    """The P1 advection-diffusion terms under every tet rule (the closed form
    takes the rule's reference mass; degree 1 is not exact for it)."""
    nd, X = M.cube_mesh(4)
    case = CASES[name]
    fl = _fields(X, case)
    m = ft.Mesh(nd, X)
    f, c, _ = O.make_sparsity(nd)
    ocol, ncol = O.colour_cg1(nd)
    kw = {k: v for k, v in fl.items() if k not in ("theta", "dt", "beta", "have_mass", "lump_mass", "by_parts")}
    kw.update({k: case[k] for k in ("theta", "dt", "beta", "have_mass", "lump_mass", "by_parts") if k in case})
    oval, orhs = _oracle(O, nd, X, nd, X.shape[0], f, c, colours=O.colour_sets(ocol, ncol), quad_degree=qdeg, **kw)
    val, rhs = ft.assemble_advection_diffusion_cg(m, _params(case, qdeg), t=fl.get("T"),
                                                  velocity=fl.get("velocity"), source=fl.get("source"))
    _compare(val, rhs, oval, orhs, f)


@pytest.mark.parametrize("name", ["poisson", "anisotropic", "advdif", "advdif_by_parts", "lumped_absorption"])
def test_p2_assembly_matches_oracle(O, name):
    nd, X = M.cube_mesh(3)
    nd2, n2 = O.make_global_numbering_p2(nd)
    X2 = M.p2_coordinates(nd, nd2, X, O.tet_counts(2))
    case = CASES[name]
    fl = _fields(X2, case)
    if "velocity" in fl:
        fl["velocity"] = M.advdif_velocity(X)  # velocity lives on the P1 coordinate mesh
    m = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    f, c, _ = O.make_sparsity(nd2)
    kw = {k: v for k, v in fl.items() if k not in ("theta", "dt", "beta", "have_mass", "lump_mass", "by_parts")}
    kw.update({k: case[k] for k in ("theta", "dt", "beta", "have_mass", "lump_mass", "by_parts") if k in case})
    oval, orhs = _oracle(O, nd, X, nd2, n2, f, c, quad_degree=4, t_degree=2, **kw)
    val, rhs = ft.assemble_advection_diffusion_cg(m, _params(case, 4), t=fl.get("T"),
                                                  velocity=fl.get("velocity"),
                                                  source=fl.get("source"),
                                                  absorption=fl.get("absorption"))
    _compare(val, rhs, oval, orhs, f)


def test_assembly_deterministic_and_device_path(O):
    import torch
    nd, X = M.cube_mesh(16)
    m = ft.Mesh(nd, X)
    p = _params(CASES["poisson"], 2)
    src = M.poisson_source(X)
    v1, r1 = ft.assemble_advection_diffusion_cg(m, p, source=src)
    v2, r2 = ft.assemble_advection_diffusion_cg(m, p, source=src)
    assert v1.tobytes() == v2.tobytes() and r1.tobytes() == r2.tobytes()
    dsrc = torch.from_numpy(src).cuda()
    dv, dr = ft.assemble_advection_diffusion_cg(m, p, source=dsrc)
    torch.cuda.synchronize()
    assert dv.cpu().numpy().tobytes() == v1.tobytes()
    assert dr.cpu().numpy().tobytes() == r1.tobytes()


def test_large_mesh_properties():
    """64^3 (1.57M tets): symmetric Laplacian with zero row sums and rhs summing
    to the integral of the interpolated source -- size-independent checks."""
    import scipy.sparse as sp
    n = 64
    nd, X = M.cube_mesh(n)
    m = ft.Mesh(nd, X)
    assert m.nnz == M.cube_counts(n)["nnz1"]
    s = m.sparsity()
    ones = np.ones(X.shape[0])
    val, rhs = ft.assemble_advection_diffusion_cg(m, _params(CASES["poisson"], 2), source=ones)
    A = sp.csr_matrix((val, s.colm, s.findrm))
    assert abs(A - A.T).max() <= 1e-15 * np.abs(val).max()
    assert np.abs(A @ ones).max() <= 1e-12 * np.abs(val).max()
    assert abs(rhs.sum() - 1.0) <= 1e-12


def test_invalid_options_are_errors():
    """Bad options raise FlError (FLAbort/FLExit in the reference) and leave the handle usable."""
    nd, X = M.cube_mesh(2)
    m = ft.Mesh(nd, X)
    with pytest.raises(ft._lib.FlError):
        ft.assemble_advection_diffusion_cg(m, ft.advdif_params(diffusivity=1.0, quad_degree=7))
    with pytest.raises(ft._lib.FlError):  # advection without a velocity field
        ft.assemble_advection_diffusion_cg(m, ft.advdif_params(have_advection=True))
    val, rhs = ft.assemble_advection_diffusion_cg(m, _params(CASES["poisson"], 2),
                                                  source=np.ones(X.shape[0]))
    assert np.isfinite(val).all()


@pytest.mark.parametrize("n", [5, 33])
def test_host_pointer_assembly_pinned_and_pageable(n):
    """The host-pointer entry point gives the device path's bits whether the
    output arrays are pinned (written in place by the row pass) or pageable
    (staged and copied)."""
    import torch
    nd, X = M.cube_mesh(n)
    m = ft.Mesh(nd, X)
    p = _params(CASES["poisson"], 2)
    src = M.poisson_source(X)
    dval, drhs = ft.assemble_advection_diffusion_cg(m, p, source=torch.tensor(src, device="cuda"))
    dval, drhs = dval.cpu().numpy(), drhs.cpu().numpy()
    pv = torch.empty(m.nnz, dtype=torch.float64).pin_memory().numpy()
    pr = torch.empty(m.N, dtype=torch.float64).pin_memory().numpy()
    pv[:] = np.nan
    pr[:] = np.nan
    ft.assemble_advection_diffusion_cg(m, p, source=src, val=pv, rhs=pr)
    assert np.array_equal(pv, dval) and np.array_equal(pr, drhs)
    hv, hr = ft.assemble_advection_diffusion_cg(m, p, source=src)
    assert np.array_equal(hv, dval) and np.array_equal(hr, drhs)


@pytest.mark.parametrize("case", ["poisson", "anisotropic", "diffusion_mass_t", "shuffled"])
def test_host_pointer_pipelined_chunks(case):
    """Pinned outputs of the P1 double-float forms on a 64^3 mesh (32 MB of
    val) are assembled in row chunks, elements in highest-node order, each
    chunk's val and rhs copied to the host while later chunks run: the device
    path's bits, also under a random node numbering (chunks that need almost
    every element) and with consistent mass and old-field terms."""
    import torch
    nd, X = M.cube_mesh(64)
    if case == "shuffled":
        perm = np.random.default_rng(17).permutation(len(X))
        inv = np.empty_like(perm)
        inv[perm] = np.arange(len(X))
        nd, X = perm[nd].astype(nd.dtype), X[inv]
    spec = {"poisson": CASES["poisson"], "anisotropic": CASES["anisotropic"], "shuffled": CASES["poisson"],
            "diffusion_mass_t": dict(theta=0.5, dt=0.01, have_mass=True, T=True, diffusivity=1e-3,
                                     source=True)}[case]
    fl = _fields(X, spec)
    kw = dict(source=fl.get("source"), t=fl.get("T"))
    m = ft.Mesh(nd, X)
    p = _params(spec, 2)
    dkw = {k: (torch.tensor(v, device="cuda") if v is not None else None) for k, v in kw.items()}
    dval, drhs = ft.assemble_advection_diffusion_cg(m, p, **dkw)
    dval, drhs = dval.cpu().numpy(), drhs.cpu().numpy()
    pv = torch.empty(m.nnz, dtype=torch.float64).pin_memory().numpy()
    pr = torch.empty(m.N, dtype=torch.float64).pin_memory().numpy()
    for _ in range(2):
        pv[:] = np.nan
        pr[:] = np.nan
        k0 = ft.kernel_launch_count()
        ft.assemble_advection_diffusion_cg(m, p, val=pv, rhs=pr, **kw)
        launches = ft.kernel_launch_count() - k0
        assert np.array_equal(pv, dval) and np.array_equal(pr, drhs)
    assert launches >= 8  # an element and a row launch per chunk
    m.close()
