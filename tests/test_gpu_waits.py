"""The bounded device waits run out cleanly (failure detection without a GPU
fault).

Two kernels wait on flags that other threads set: the colouring dataflow (an
element waits for its lower neighbours' colours) and the fused P1 element +
row pass (a row item waits for the element items it reads).  The test hook
fl_set_wait_test keeps one such flag unset -- a flag that nothing sets -- and
shortens the waits to a few milliseconds: the waiting threads record
FL_ERR_TIMEOUT and stop, every kernel finishes, the call returns the status,
and the next call without the hook gives the normal, oracle-checked results
in the same CUDA context.  This is the device side of the reference's
failure path (a solver or assembly failure reported to the caller,
femtools/Solvers.F90:1369-1479), without a trap, fault or hang.
"""
import numpy as np
import pytest

from fluidity_gb300 import _lib
from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu
FL_ERR_TIMEOUT = 4


@pytest.fixture
def hook():
    lib = _lib.load()
    yield lib
    assert lib.fl_set_wait_test(-1, 0.0) == 0


def test_colouring_wait_runs_out(O, hook):
    nd, X = M.cube_mesh(6)
    assert hook.fl_set_wait_test(600, 5.0) == 0   # element 600 never publishes its colour
    with pytest.raises(_lib.FlError) as err:
        ft.Mesh(nd, X)
    assert err.value.status == FL_ERR_TIMEOUT
    assert "bounded device wait ran out" in str(err.value)
    assert hook.fl_set_wait_test(-1, 0.0) == 0
    m = ft.Mesh(nd, X)                               # same context, normal result
    col, _, _ = m.colouring()
    ocol, ncol = O.colour_cg1(nd)
    assert np.array_equal(col, ocol) and m.ncolours == ncol
    m.close()


def test_fused_pass_wait_runs_out(hook):
    import torch
    nd, X = M.cube_mesh(9)
    m = ft.Mesh(nd, X)
    p = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
    src = torch.tensor(M.poisson_source(X), device="cuda")
    ft.set_assembly_tiles(m, 256, 16, 1)
    v0, r0 = ft.assemble_advection_diffusion_cg(m, p, source=src)
    v0, r0 = v0.clone(), r0.clone()
    ft.set_assembly_tiles(m, 256, 16, 3)             # the fused pass
    assert hook.fl_set_wait_test(0, 5.0) == 0        # element-item group 0 never completes
    with pytest.raises(_lib.FlError) as err:
        ft.assemble_advection_diffusion_cg(m, p, source=src)
    assert err.value.status == FL_ERR_TIMEOUT
    assert hook.fl_set_wait_test(-1, 0.0) == 0
    for _ in range(2):                               # the handle stays usable
        v, r = ft.assemble_advection_diffusion_cg(m, p, source=src)
        assert torch.equal(v, v0) and torch.equal(r, r0)
    m.close()


def test_hook_arguments(hook):
    assert hook.fl_set_wait_test(3, 0.0) == 1        # a withheld flag needs a limit
    assert hook.fl_set_wait_test(-2, 1.0) == 1
    assert hook.fl_set_wait_test(-1, 0.0) == 0


def test_gmres_grid_barrier_runs_out(O, hook):
    """The cooperative GMRES solve: block 1 never arrives at a grid barrier,
    the other blocks' waits run out, every block leaves, the solve reports
    FL_ERR_TIMEOUT; the next solve in the same context matches the oracle."""
    nd, X = M.cube_mesh(16)
    m = ft.Mesh(nd, X)
    T0 = M.gaussian_tracer(X)
    p = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True, diffusivity=1e-3)
    val, rhs = ft.assemble_advection_diffusion_cg(m, p, t=T0, velocity=M.advdif_velocity(X))
    ina = np.zeros(m.N, dtype=np.uint8)
    bn = M.boundary_nodes(X)
    ft.apply_dirichlet_conditions(m, rhs, ina, bn, np.zeros(bn.size), t=T0, dt=0.01)
    opts = ft.solver_options(ksp="gmres", restart=30, rtol=1e-10, schedule="persistent")
    assert hook.fl_set_wait_test(1, 5.0) == 0       # block 1 of the cooperative solve never arrives
    with pytest.raises(_lib.FlError) as err:
        ft.petsc_solve(m, np.zeros(m.N), val, rhs, opts, inactive=ina)
    assert err.value.status == FL_ERR_TIMEOUT
    assert "bounded device wait ran out" in str(err.value)
    assert hook.fl_set_wait_test(-1, 0.0) == 0
    x = np.zeros(m.N)
    rep = ft.petsc_solve(m, x, val, rhs, opts, inactive=ina)
    s = m.sparsity()
    ox, oits, oreason, _ = O.petsc_solve(s.findrm.astype(np.int64), s.colm, val, ina, rhs, ksp="gmres",
                                         restart=30, rtol=1e-10)
    assert rep["reason"] == oreason == 2 and abs(rep["iterations"] - oits) <= 1
    assert np.abs(x - ox).max() <= 1e-8 * np.abs(ox).max()
    m.close()
