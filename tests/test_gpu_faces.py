"""The GPU surface loop of assemble_advection_diffusion_cg and the element
advection integrated by parts, against the oracle's restatement
(Advection_Diffusion_CG.F90:608-640, :1019-1057, :1228-1378).

Tolerance (floating point): |a - a_ref| <= 1e-12 max_j |a_ref(i, j)| per row,
rhs within 1e-12 of max |rhs_ref|.
"""
import numpy as np
import pytest

from conftest import row_scaled_error
from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu
TOL = 1e-12

CASES = {
    # diffusivity with every face type but weak Dirichlet
    "diffusion_neumann_robin": dict(diffusivity=0.7, types=(0, 1, 3, 4), theta=0.5, dt=0.1),
    # advection by parts (no diffusivity) with weak Dirichlet faces
    "advection_by_parts_weakdirichlet": dict(types=(0, 2, 3), by_parts=True, theta=0.5, dt=0.1, beta=0.3),
    # both, implicit
    "advdif_by_parts_neumann_robin": dict(diffusivity=1e-2, types=(0, 1, 4), by_parts=True, theta=1.0, dt=0.05,
                                          beta=1.0),
    # explicit (dt theta = 0): nothing enters the matrix
    "explicit_robin": dict(diffusivity=0.3, types=(1, 4), theta=0.0, dt=0.1),
}


def _case_inputs(nd, X, floc_faces, case, rng):
    faces, xf, fe = floc_faces
    nf, floc = faces.shape
    types = np.asarray(case["types"], np.int32)[rng.integers(0, len(case["types"]), nf)]
    bc1 = rng.standard_normal((nf, floc))
    bc2 = 0.5 + rng.random((nf, floc))
    return faces, xf, fe, types, bc1, bc2


def _run(O, m, nd, X, ndt, nt, faces, xf, fe, types, bc1, bc2, case, quad_degree, t_degree, T, u, f, c,
         colours):
    diff = case.get("diffusivity")
    by_parts = case.get("by_parts", False)
    theta, dt, beta = case["theta"], case["dt"], case.get("beta", 0.0)
    kw = dict(theta=theta, dt=dt, beta=beta, velocity=u if by_parts else None, T=T, diffusivity=diff,
              quad_degree=quad_degree)
    oval, orhs, st = O.assemble_advdif(ndglno_t=ndt, nt=nt, ndglno_x=nd, coords=X, findrm=f, colm=c,
                                       have_mass=True, t_degree=t_degree, colours=colours, by_parts=by_parts, **kw)
    assert st == 0
    st = O.assemble_advdif_faces(oval, orhs, faces=faces, xfaces=xf, face_ele=fe, ndglno_x=nd, coords=X,
                                 findrm=f, colm=c, bc_type=types, bc_value=bc1, bc_value2=bc2, by_parts=by_parts,
                                 **kw)
    assert st == 0
    p = ft.advdif_params(theta=theta, dt=dt, beta=beta, have_mass=True, have_advection=by_parts,
                         diffusivity=diff, quad_degree=quad_degree, integrate_advection_by_parts=by_parts)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, t=T, velocity=u if by_parts else None)
    val, rhs = ft.assemble_advection_diffusion_faces(m, p, val, rhs, faces=faces, xfaces=xf, face_ele=fe,
                                                     bc_type=types, bc_value=bc1, bc_value2=bc2, t=T,
                                                     velocity=u if by_parts else None)
    return val, rhs, oval, orhs


@pytest.mark.parametrize("name", list(CASES))
@pytest.mark.parametrize("mesh", ["cube4", "aniso"])
def test_p1_faces_match_oracle(O, aniso_mesh, name, mesh):
    nd, X = M.cube_mesh(4) if mesh == "cube4" else aniso_mesh
    case = CASES[name]
    rng = np.random.default_rng(7)
    m = ft.Mesh(nd, X)
    f, c, _ = O.make_sparsity(nd)
    ocol, ncol = O.colour_cg1(nd)
    faces, fe = M.boundary_faces(nd)
    args = _case_inputs(nd, X, (faces, faces.copy(), fe), case, rng)
    T = M.gaussian_tracer(X, sigma=0.3)
    u = M.advdif_velocity(X) + np.array([0.3, -0.2, 0.1]) * X
    val, rhs, oval, orhs = _run(O, m, nd, X, nd, X.shape[0], *args, case, 2, 1, T, u, f, c,
                                O.colour_sets(ocol, ncol))
    assert row_scaled_error(val, oval, f) <= TOL
    assert np.abs(rhs - orhs).max() <= TOL * np.abs(orhs).max()
    m.close()


@pytest.mark.parametrize("name", ["diffusion_neumann_robin", "advdif_by_parts_neumann_robin"])
def test_p2_faces_match_oracle(O, name):
    nd, X = M.cube_mesh(3)
    nd2, n2 = O.make_global_numbering_p2(nd)
    X2 = M.p2_coordinates(nd, nd2, X, O.tet_counts(2))
    case = CASES[name]
    rng = np.random.default_rng(11)
    m = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    f, c, _ = O.make_sparsity(nd2)
    ocol, ncol = O.colour_cg1(nd)
    args = _case_inputs(nd, X, M.boundary_faces_p2(nd, nd2), case, rng)
    T = M.gaussian_tracer(X2, sigma=0.3)
    u = M.advdif_velocity(X)
    val, rhs, oval, orhs = _run(O, m, nd, X, nd2, n2, *args, case, 4, 2, T, u, f, c, O.colour_sets(ocol, ncol))
    assert row_scaled_error(val, oval, f) <= TOL
    assert np.abs(rhs - orhs).max() <= TOL * np.abs(orhs).max()
    m.close()


def test_device_and_host_entry_points_agree_and_repeat(O):
    import torch
    nd, X = M.cube_mesh(5)
    m = ft.Mesh(nd, X)
    faces, fe = M.boundary_faces(nd)
    nf = faces.shape[0]
    rng = np.random.default_rng(3)
    types = np.array([0, 1, 4], np.int32)[rng.integers(0, 3, nf)]
    bc1, bc2 = rng.standard_normal((nf, 3)), rng.random((nf, 3))
    T = M.gaussian_tracer(X)
    u = M.advdif_velocity(X)
    p = ft.advdif_params(theta=0.5, dt=0.1, have_mass=True, have_advection=True, diffusivity=0.1,
                         integrate_advection_by_parts=True)
    v0, r0 = ft.assemble_advection_diffusion_cg(m, p, t=T, velocity=u)
    hv, hr = v0.copy(), r0.copy()
    ft.assemble_advection_diffusion_faces(m, p, hv, hr, faces=faces, xfaces=faces, face_ele=fe, bc_type=types,
                                          bc_value=bc1, bc_value2=bc2, t=T, velocity=u)
    for _ in range(2):
        dv, dr = torch.from_numpy(v0).cuda(), torch.from_numpy(r0).cuda()
        ft.assemble_advection_diffusion_faces(m, p, dv, dr, faces=torch.from_numpy(faces).cuda(),
                                              xfaces=torch.from_numpy(faces).cuda(),
                                              face_ele=torch.from_numpy(fe).cuda(),
                                              bc_type=torch.from_numpy(types).cuda(),
                                              bc_value=torch.from_numpy(bc1).cuda(),
                                              bc_value2=torch.from_numpy(bc2).cuda(), t=torch.from_numpy(T).cuda(),
                                              velocity=torch.from_numpy(u).cuda())
        torch.cuda.synchronize()
        assert dv.cpu().numpy().tobytes() == hv.tobytes() and dr.cpu().numpy().tobytes() == hr.tobytes()
    assert np.abs(hv - v0).max() > 0 and np.abs(hr - r0).max() > 0
    m.close()


def test_weak_dirichlet_with_diffusivity_is_an_error():
    nd, X = M.cube_mesh(3)
    m = ft.Mesh(nd, X)
    faces, fe = M.boundary_faces(nd)
    nf = faces.shape[0]
    p = ft.advdif_params(diffusivity=1.0)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p)
    with pytest.raises(RuntimeError, match="weak Dirichlet"):
        ft.assemble_advection_diffusion_faces(m, p, val, rhs, faces=faces, xfaces=faces, face_ele=fe,
                                              bc_type=np.full(nf, 2, np.int32), bc_value=np.ones((nf, 3)))
    m.close()


def test_by_parts_step_solves_like_not_by_parts(O):
    """With no flux through the boundary faces' weak form changed, the by-parts
    system plus its face terms and the not-by-parts system give the same
    solve (degree-4 rule, where the two forms are equal to rounding)."""
    nd, X = M.cube_mesh(6)
    m = ft.Mesh(nd, X)
    faces, fe = M.boundary_faces(nd)
    nf = faces.shape[0]
    u = M.advdif_velocity(X) + np.array([0.3, -0.2, 0.1]) * X
    T = M.gaussian_tracer(X)
    base = dict(theta=0.5, dt=0.01, beta=0.0, have_mass=True, have_advection=True, diffusivity=1e-3, quad_degree=4)
    pa = ft.advdif_params(**base)
    pb = ft.advdif_params(integrate_advection_by_parts=True, **base)
    va, ra = ft.assemble_advection_diffusion_cg(m, pa, t=T, velocity=u)
    vb, rb = ft.assemble_advection_diffusion_cg(m, pb, t=T, velocity=u)
    ft.assemble_advection_diffusion_faces(m, pb, vb, rb, faces=faces, xfaces=faces, face_ele=fe,
                                          bc_type=np.zeros(nf, np.int32), t=T, velocity=u)
    f = m.sparsity().findrm
    assert row_scaled_error(vb, va, f) <= 1e-12
    assert np.abs(rb - ra).max() <= 1e-12 * np.abs(ra).max()
    m.close()


def test_missing_boundary_values_are_an_error():
    nd, X = M.cube_mesh(3)
    m = ft.Mesh(nd, X)
    faces, fe = M.boundary_faces(nd)
    nf = faces.shape[0]
    p = ft.advdif_params(diffusivity=1.0)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p)
    with pytest.raises(RuntimeError, match="boundary values"):
        ft.assemble_advection_diffusion_faces(m, p, val, rhs, faces=faces, xfaces=faces, face_ele=fe,
                                              bc_type=np.full(nf, 4, np.int32), bc_value=np.ones((nf, 3)))
    m.close()
