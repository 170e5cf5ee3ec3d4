"""Batched steps (CUDA graphs over many fields and meshes) and the assembly
tile autotuner, checked bit for bit against the unbatched entry points, which
the other GPU tests check against the oracle."""
import numpy as np
import pytest

from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu


def _tracer(X, kappa, scale):
    p = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True, diffusivity=kappa)
    return p, M.gaussian_tracer(X), scale * M.advdif_velocity(X)


def _unbatched(torch, m, p, opts, bn, *, t=None, u=None, f=None):
    dev = "cuda"
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, t=t, velocity=u, source=f)
    ina = torch.zeros(m.N, dtype=torch.uint8, device=dev)
    nodes = torch.as_tensor(bn, dtype=torch.int32, device=dev)
    g = torch.zeros(bn.size, dtype=torch.float64, device=dev)
    ft.apply_dirichlet_conditions(m, rhs, ina, nodes, g, t=t, dt=p.dt)
    x = torch.zeros(m.N, dtype=torch.float64, device=dev)
    rep = ft.petsc_solve(m, x, val, rhs, opts, inactive=ina)
    return val, rhs, ina, x, rep


def _members():
    """Two tracers (GMRES) on a shared mesh, a Poisson member (CG) on it, and
    two Poisson members on meshes of other sizes."""
    import torch
    kap, sc = M.batch_tracer_params(2)
    nd, X = M.cube_mesh(8)
    shared = ft.Mesh(nd, X)
    out = []
    for k in range(2):
        p, T0, u = _tracer(X, kap[k], sc[k])
        # the batch replays graph cycles: bitwise equal to the graph schedule
        out.append((shared, p, ft.solver_options(ksp="gmres", restart=30, rtol=1e-10, schedule="graph"),
                    M.boundary_nodes(X),
                    {"t": torch.tensor(T0, device="cuda"), "u": torch.tensor(u, device="cuda")}))
    pois = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
    out.append((shared, pois, ft.solver_options(ksp="cg", rtol=1e-10), M.boundary_nodes(X),
                {"f": torch.tensor(M.poisson_source(X), device="cuda")}))
    for i, n in ((0, 5), (1, 7)):
        ndi, Xi = M.batch_mesh(i, n)
        mi = ft.Mesh(ndi, Xi)
        out.append((mi, pois, ft.solver_options(ksp="cg", rtol=1e-10), M.boundary_nodes(Xi),
                    {"f": torch.tensor(M.poisson_source(Xi), device="cuda")}))
    return out


def test_batch_matches_unbatched_bitwise():
    import torch
    mem = _members()
    b = ft.Batch()
    regs = []
    for m, p, o, bn, fl in mem:
        regs.append(b.add(m, p, o, bc_nodes=bn, bc_values=np.zeros(bn.size), t=fl.get("t"),
                          velocity=fl.get("u"), source=fl.get("f")))
    reps = b.run()
    torch.cuda.synchronize()
    for (m, p, o, bn, fl), r, rep in zip(mem, regs, reps):
        val, rhs, ina, x, urep = _unbatched(torch, m, p, o, bn, t=fl.get("t"), u=fl.get("u"),
                                            f=fl.get("f"))
        assert rep["reason"] == 2, rep
        assert rep["iterations"] == urep["iterations"]
        assert torch.equal(r["val"], val) and torch.equal(r["rhs"], rhs)
        assert torch.equal(r["inactive"], ina)
        assert torch.equal(r["x"], x)
        assert rep["true_rel_residual"] == urep["true_rel_residual"]
        assert rep["true_rel_residual"] < 1e-8
    # a second run re-reads the fields (x is the initial guess again): change
    # one tracer and compare again
    m, p, o, bn, fl = mem[0]
    fl["t"].mul_(0.5)
    for r in regs:
        r["x"].zero_()
    reps = b.run()
    val, rhs, ina, x, urep = _unbatched(torch, m, p, o, bn, t=fl["t"], u=fl["u"])
    assert torch.equal(regs[0]["x"], x) and reps[0]["iterations"] == urep["iterations"]
    b.close()


def test_batch_converged_member_is_stable():
    """Replays past a member's convergence leave its solution unchanged: a
    quickly converging member next to a slow one equals its lone solve."""
    import torch
    nd, X = M.cube_mesh(10)
    m = ft.Mesh(nd, X)
    slow = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
    fast, T0, u = _tracer(X, 1e-4, 0.5)
    bn = M.boundary_nodes(X)
    tt, uu = torch.tensor(T0, device="cuda"), torch.tensor(u, device="cuda")
    ff = torch.tensor(M.poisson_source(X), device="cuda")
    b = ft.Batch()
    r_fast = b.add(m, fast, ft.solver_options(ksp="gmres", restart=5, rtol=1e-10), bc_nodes=bn,
                   bc_values=np.zeros(bn.size), t=tt, velocity=uu)
    b.add(m, slow, ft.solver_options(ksp="cg", rtol=1e-12), bc_nodes=bn,
          bc_values=np.zeros(bn.size), source=ff)
    reps = b.run()
    _, _, _, x, urep = _unbatched(torch, m, fast, ft.solver_options(ksp="gmres", restart=5, rtol=1e-10,
                                                                    schedule="graph"), bn, t=tt, u=uu)
    assert reps[0]["iterations"] == urep["iterations"] < reps[1]["iterations"]
    assert torch.equal(r_fast["x"], x)
    b.close()


def test_batch_iteration_limit():
    import torch
    nd, X = M.cube_mesh(6)
    m = ft.Mesh(nd, X)
    p = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
    bn = M.boundary_nodes(X)
    ff = torch.tensor(M.poisson_source(X), device="cuda")
    b = ft.Batch()
    b.add(m, p, ft.solver_options(ksp="cg", rtol=1e-14, max_its=7), bc_nodes=bn,
          bc_values=np.zeros(bn.size), source=ff)
    pt, T0, u = _tracer(X, 1e-3, 1.0)
    b.add(m, pt, ft.solver_options(ksp="gmres", restart=4, rtol=1e-14, max_its=6), bc_nodes=bn,
          bc_values=np.zeros(bn.size), t=torch.tensor(T0, device="cuda"),
          velocity=torch.tensor(u, device="cuda"))
    reps = b.run()
    assert reps[0]["reason"] == -3 and reps[0]["iterations"] == 7
    assert reps[1]["reason"] == -3 and reps[1]["iterations"] == 6
    b.close()


@pytest.mark.parametrize("case", ["poisson", "tracer"])
def test_autotune_tiles_do_not_change_results(case):
    import torch
    nd, X = M.cube_mesh(12)
    m = ft.Mesh(nd, X)
    if case == "poisson":
        p = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
        kw = {"source": torch.tensor(M.poisson_source(X), device="cuda")}
    else:
        p, T0, u = _tracer(X, 1e-3, 1.0)
        kw = {"t": torch.tensor(T0, device="cuda"), "velocity": torch.tensor(u, device="cuda")}
    val0, rhs0 = ft.assemble_advection_diffusion_cg(m, p, **kw)
    val0, rhs0 = val0.clone(), rhs0.clone()
    val, rhs, tiles = ft.autotune_assembly(m, p, **kw)
    assert tiles[0] in (128, 256) and tiles[1] in (4, 8, 16, 32) and tiles[2] in (0, 1, 2, 3)
    assert torch.equal(val, val0) and torch.equal(rhs, rhs0)
    for eb, esm, rt in ((128, 4, 0), (256, 32, 2), (128, 16, 1), (256, 8, 0), (256, 16, 3)):
        ft.set_assembly_tiles(m, eb, esm, rt)
        v, r = ft.assemble_advection_diffusion_cg(m, p, **kw)
        assert torch.equal(v, val0) and torch.equal(r, rhs0), (eb, esm, rt)


FUSED_CASES = {
    "poisson": dict(diffusivity=1.0, have_source=True),
    "aniso_mass_t": dict(diffusivity=[[1.0, 0, 0], [0, 1.0, 0], [0, 0, 1e-3]], have_source=True, have_mass=True,
                         theta=0.5, dt=0.1),
    "mass_t_only": dict(diffusivity=0.3, have_mass=True, theta=1.0, dt=0.05),
}


@pytest.mark.parametrize("n", [9, 40])
@pytest.mark.parametrize("case", sorted(FUSED_CASES))
def test_fused_p1_pass_is_bit_identical(n, case):
    """The fused element + row pass (row tile 3) gives the two-kernel pass's
    values and rhs bit for bit, on every call (the queue and the flags are
    reset per call)."""
    import torch
    nd, X = M.cube_mesh(n)
    m = ft.Mesh(nd, X)
    kw0 = FUSED_CASES[case]
    p = ft.advdif_params(quad_degree=2, **kw0)
    kw = {}
    if kw0.get("have_source"):
        kw["source"] = torch.tensor(M.poisson_source(X), device="cuda")
    if kw0.get("have_mass"):
        kw["t"] = torch.tensor(M.gaussian_tracer(X), device="cuda")
    ft.set_assembly_tiles(m, 256, 16, 1)
    v0, r0 = ft.assemble_advection_diffusion_cg(m, p, **kw)
    v0, r0 = v0.clone(), r0.clone()
    ft.set_assembly_tiles(m, 256, 16, 3)
    for _ in range(3):
        v, r = ft.assemble_advection_diffusion_cg(m, p, **kw)
        assert torch.equal(v, v0) and torch.equal(r, r0)
    m.close()
