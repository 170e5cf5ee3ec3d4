"""The allocation-free P1 diffusion assembly entry point.

Callers that cannot allocate device memory while they assemble (for example
an application whose memory manager has reserved the whole device, or a loop
that must avoid cudaMalloc because it can synchronise the device) use
fl_dev_assemble_p1_diffusion_noalloc, whose scratch is a fixed array inside the
library.  These tests call it through the C-ABI twice in a row and check each
result against the allocating entry point, with the tolerance the other
assembly tests use, and check that meshes above the array's limit are refused.
The file is named so pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import row_scaled_error
from fluidity_gb300 import _lib
from fluidity_gb300 import femtools as ft
from fluidity_gb300 import meshgen as M

pytestmark = pytest.mark.gpu
TOL = 1e-12
LIMIT = 131072  # elements the library's scratch array holds


def _noalloc(lib, mesh, params, fields, val, rhs, stream):
    return lib.fl_dev_assemble_p1_diffusion_noalloc(mesh.handle, C.byref(params), C.byref(fields),
                                                    val.data_ptr(), rhs.data_ptr(), stream)


def test_noalloc_matches_allocating_entry_point_on_two_calls():
    import torch
    lib = _lib.load()
    nd, X = M.cube_mesh(16)
    m = ft.Mesh(nd, X)
    s = m.sparsity()
    p = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
    src = torch.from_numpy(M.poisson_source(X)).cuda()
    ref_val, ref_rhs = ft.assemble_advection_diffusion_cg(m, p, source=src)
    torch.cuda.synchronize()
    ref_val, ref_rhs = ref_val.cpu().numpy(), ref_rhs.cpu().numpy()
    fields = _lib.Fields(None, None, src.data_ptr(), None)
    stream = ft._stream_ptr(torch.cuda.current_stream())
    for _ in range(2):
        val = torch.full((m.nnz,), float("nan"), dtype=torch.float64, device="cuda")
        rhs = torch.full((m.N,), float("nan"), dtype=torch.float64, device="cuda")
        _lib.check(_noalloc(lib, m, p, fields, val, rhs, stream), "noalloc assembly")
        torch.cuda.synchronize()
        v, r = val.cpu().numpy(), rhs.cpu().numpy()
        assert np.isfinite(v).all() and np.isfinite(r).all()
        assert row_scaled_error(v, ref_val, s.findrm) <= TOL
        assert np.abs(r - ref_rhs).max() <= TOL * np.abs(ref_rhs).max()


def test_noalloc_after_another_mesh_and_with_mass():
    """The shared scratch keeps the previous call's contents; results must not depend on them."""
    import torch
    lib = _lib.load()
    stream = ft._stream_ptr(torch.cuda.current_stream())
    p = ft.advdif_params(theta=0.5, dt=0.1, diffusivity=np.diag([1.0, 1.0, 1e-3]), have_mass=True,
                         have_source=True, quad_degree=2)
    for n in (12, 7):
        nd, X = M.cube_mesh(n)
        m = ft.Mesh(nd, X)
        src = torch.from_numpy(M.poisson_source(X)).cuda()
        t = torch.from_numpy(M.gaussian_tracer(X)).cuda()
        ref_val, ref_rhs = ft.assemble_advection_diffusion_cg(m, p, t=t, source=src)
        val = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
        rhs = torch.empty(m.N, dtype=torch.float64, device="cuda")
        fields = _lib.Fields(t.data_ptr(), None, src.data_ptr(), None)
        _lib.check(_noalloc(lib, m, p, fields, val, rhs, stream), "noalloc assembly")
        torch.cuda.synchronize()
        assert row_scaled_error(val.cpu().numpy(), ref_val.cpu().numpy(), m.sparsity().findrm) <= TOL
        rr = ref_rhs.cpu().numpy()
        assert np.abs(rhs.cpu().numpy() - rr).max() <= TOL * np.abs(rr).max()


def test_noalloc_rejects_meshes_above_the_limit():
    import torch
    lib = _lib.load()
    nd, X = M.cube_mesh(28)
    assert nd.shape[0] > LIMIT
    m = ft.Mesh(nd, X)
    p = ft.advdif_params(diffusivity=1.0, quad_degree=2)
    val = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
    rhs = torch.empty(m.N, dtype=torch.float64, device="cuda")
    st = _noalloc(lib, m, p, _lib.Fields(None, None, None, None), val, rhs,
                  ft._stream_ptr(torch.cuda.current_stream()))
    assert st == 1  # FL_ERR_ARG
    assert b"allocation-free limit" in lib.fl_last_error()
