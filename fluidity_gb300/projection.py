"""Pressure-projection matrices of the P1-P1 discretisation on the GPU.

The names mirror the reference's routines (assemble/Divergence_Matrix_CG.F90,
assemble/Assemble_CMC.F90, assemble/Momentum_CG.F90, femtools/
Sparse_Matrices_Fields.F90, femtools/Sparsity_Patterns_Meshes.F90) and call
the fl_dev_* entry points of the CUDA library on device tensors:

    ct = assemble_divergence_matrix_cg(mesh, ...)          # C^T, lumped masses
    so = get_csr_sparsity_secondorder(mesh)                # CMC / KMK pattern
    cmc = assemble_masslumped_cmc(so, ct, inverse_masslump, ct)
    kmk, kt = assemble_kmk_matrix(mesh, so, p_masslump, theta_pg)
    add_kmk_matrix(so, cmc, kmk)
    rhs = assemble_masslumped_poisson_rhs(mesh, ct, ...)
    femtools.petsc_solve(so, delta_p, cmc, rhs, options, inactive=...)
    correct_masslumped_velocity(mesh, ct, inverse_masslump, delta_p, u)

Block matrices are (3, nnz) tensors (block (1, dim) in row dim); vector
fields are (N, 3) tensors, vector_field%val(3, N) in memory.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from . import femtools as ft
from ._lib import DivergenceParams, check


def _torch():
    import torch
    return torch


def _dev(a, dtype):
    """A contiguous device tensor of the given torch dtype (numpy is uploaded)."""
    torch = _torch()
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return torch.as_tensor(np.ascontiguousarray(a)).to(device="cuda", dtype=dtype)
    assert a.is_cuda and a.dtype == dtype and a.is_contiguous(), "device tensor of the right dtype"
    return a


def _ptrs(blocks):
    arr = (C.c_void_p * 3)()
    for d in range(3):
        arr[d] = blocks[d].data_ptr() if d < len(blocks) and blocks[d] is not None else None
    return arr


class SecondOrderPattern(ft.Mesh):
    """The second-order sparsity of a P1 mesh (get_csr_sparsity_secondorder),
    a pattern-only handle: solves, SpMVs and Dirichlet conditions run on it as
    on a mesh.  It keeps its mesh alive."""

    def __init__(self, mesh: ft.Mesh):
        self.lib = _lib.load()
        self.parent = mesh
        h = C.c_void_p()
        check(self.lib.fl_gpu_secondorder_register(mesh.handle, C.byref(h)), "fl_gpu_secondorder_register")
        self.handle = h
        nnz, ncol = C.c_int64(), C.c_int32()
        check(self.lib.fl_gpu_mesh_info(h, C.byref(nnz), C.byref(ncol)), "fl_gpu_mesh_info")
        self.N, self.E, self.loc, self.Nx = mesh.N, 0, 0, 0
        self.nnz, self.ncolours = nnz.value, 0
        self._sparsity = None


def get_csr_sparsity_secondorder(mesh: ft.Mesh) -> SecondOrderPattern:
    return SecondOrderPattern(mesh)


class TaylorHoodPattern(ft.Mesh):
    """make_sparsity(pressure mesh, velocity mesh) of a P2 velocity mesh with
    P1 pressure on its vertices (fl_gpu_rect_register): rows are the
    vertices, columns the P2 nodes.  A pattern-only handle; it keeps its
    mesh alive."""

    def __init__(self, mesh: ft.Mesh):
        self.lib = _lib.load()
        self.parent = mesh
        h = C.c_void_p()
        check(self.lib.fl_gpu_rect_register(mesh.handle, C.byref(h)), "fl_gpu_rect_register")
        self.handle = h
        nnz, ncol = C.c_int64(), C.c_int32()
        check(self.lib.fl_gpu_mesh_info(h, C.byref(nnz), C.byref(ncol)), "fl_gpu_mesh_info")
        self.N, self.E, self.loc, self.Nx = mesh.Nx, 0, 0, 0
        self.nnz, self.ncolours = nnz.value, 0
        self._sparsity = None


class TaylorHoodProductPattern(ft.Mesh):
    """The pattern of the Taylor-Hood cmc_m (fl_gpu_rect_secondorder_register):
    C C^T of a TaylorHoodPattern through the velocity nodes, pressure rows and
    columns.  A pattern-only handle for mult_div_vector_div_T, solves and
    SpMVs; it keeps its pattern alive."""

    def __init__(self, pattern: TaylorHoodPattern):
        self.lib = _lib.load()
        self.parent = pattern
        h = C.c_void_p()
        check(self.lib.fl_gpu_rect_secondorder_register(pattern.handle, C.byref(h)),
              "fl_gpu_rect_secondorder_register")
        self.handle = h
        nnz, ncol = C.c_int64(), C.c_int32()
        check(self.lib.fl_gpu_mesh_info(h, C.byref(nnz), C.byref(ncol)), "fl_gpu_mesh_info")
        self.N, self.E, self.loc, self.Nx = pattern.N, 0, 0, 0
        self.nnz, self.ncolours = nnz.value, 0
        self._sparsity = None


def assemble_divergence_matrix_p2p1(mesh: ft.Mesh, pattern: TaylorHoodPattern, *, integrate_by_parts=False,
                                    quad_degree=4, ct=None, stream=None):
    """The element terms of C^T for P2 velocity (mesh) and P1 pressure on its
    vertices, blocks (1, dim) on the Taylor-Hood pattern: a (3, nnz) device
    tensor."""
    torch = _torch()
    if ct is None:
        ct = torch.empty((3, pattern.nnz), dtype=torch.float64, device="cuda")
    check(_lib.load().fl_dev_assemble_divergence_p2p1(mesh.handle, pattern.handle, int(bool(integrate_by_parts)),
                                                      int(quad_degree), _ptrs([ct[0], ct[1], ct[2]]),
                                                      ft._stream_ptr(stream)),
          "fl_dev_assemble_divergence_p2p1")
    return ct


def assemble_divergence_faces_p2p1(mesh: ft.Mesh, pattern: TaylorHoodPattern, ct, *, faces, vfaces, face_ele,
                                   bc_type=None, bc_val=None, ct_rhs=None, quad_degree=4, index_base=0,
                                   stream=None):
    """The by-parts surface terms of C^T for the Taylor-Hood pair, added to ct
    (3, nnz) and subtracted from ct_rhs (pressure nodes, or None): faces (nf, 3)
    pressure (vertex) nodes, vfaces (nf, 6) velocity nodes in the P2
    triangle's order, face_ele (nf,), bc_type (nf, 3), bc_val (nf, 6, 3)."""
    torch = _torch()

    def dev(a, dt):
        return _dev(np.asarray(a, dtype=np.int32 if dt == torch.int32 else np.float64)
                    if isinstance(a, np.ndarray) else a, dt)

    fa, va, fe = dev(faces, torch.int32), dev(vfaces, torch.int32), dev(face_ele, torch.int32)
    ty = dev(bc_type, torch.int32) if bc_type is not None else None
    bv = dev(bc_val, torch.float64) if bc_val is not None else None
    P = DivergenceParams()
    P.integrate_by_parts = 1
    P.index_base = int(index_base)
    P.nfaces = int(fa.shape[0])
    P.faces, P.face_ele = fa.data_ptr(), fe.data_ptr()
    P.bc_type = ty.data_ptr() if ty is not None else None
    P.bc_val = bv.data_ptr() if bv is not None else None
    check(_lib.load().fl_dev_assemble_divergence_p2p1_faces(
        mesh.handle, pattern.handle, C.byref(P), va.data_ptr(), int(quad_degree), _ptrs([ct[0], ct[1], ct[2]]),
        ct_rhs.data_ptr() if ct_rhs is not None else None, ft._stream_ptr(stream)),
        "fl_dev_assemble_divergence_p2p1_faces")
    del fa, va, fe, ty, bv
    return ct


def assemble_divergence_matrix_cg(mesh: ft.Mesh, *, integrate_by_parts=False, faces=None, face_ele=None,
                                  bc_type=None, bc_val=None, ct=None, ct_rhs=None, div_mass_lumped=None,
                                  grad_mass_lumped=None, stream=None):
    """C^T of a P1 pressure / P1 velocity pair on one mesh (blocks (1, dim)),
    ct_rhs and the lumped div/grad masses; faces (nf, 3), face_ele (nf,),
    bc_type (nf, 3) and bc_val (nf, 3 nodes, 3 dims) describe the surface mesh
    for the integrated-by-parts form.  Returns a dict of device tensors."""
    torch = _torch()
    dev = torch.device("cuda")
    if ct is None:
        ct = torch.empty((3, mesh.nnz), dtype=torch.float64, device=dev)
    if ct_rhs is None:
        ct_rhs = torch.empty(mesh.N, dtype=torch.float64, device=dev)
    if div_mass_lumped is None:
        div_mass_lumped = torch.empty(mesh.N, dtype=torch.float64, device=dev)
    if grad_mass_lumped is None:
        grad_mass_lumped = torch.empty(mesh.N, dtype=torch.float64, device=dev)
    P = DivergenceParams()
    P.integrate_by_parts = int(bool(integrate_by_parts))
    keep = []
    if integrate_by_parts and faces is not None and len(faces):
        fa = _dev(np.asarray(faces, dtype=np.int32) if isinstance(faces, np.ndarray) else faces, torch.int32)
        fe = _dev(np.asarray(face_ele, dtype=np.int32) if isinstance(face_ele, np.ndarray) else face_ele,
                  torch.int32)
        ty = _dev(np.asarray(bc_type, dtype=np.int32) if isinstance(bc_type, np.ndarray) else bc_type,
                  torch.int32) if bc_type is not None else None
        bv = _dev(np.asarray(bc_val, dtype=np.float64) if isinstance(bc_val, np.ndarray) else bc_val,
                  torch.float64) if bc_val is not None else None
        keep = [fa, fe, ty, bv]
        P.nfaces = int(fa.shape[0])
        P.faces, P.face_ele = fa.data_ptr(), fe.data_ptr()
        P.bc_type = ty.data_ptr() if ty is not None else None
        P.bc_val = bv.data_ptr() if bv is not None else None
    lib = _lib.load()
    check(lib.fl_dev_assemble_divergence_cg(mesh.handle, C.byref(P), _ptrs([ct[0], ct[1], ct[2]]),
                                            ct_rhs.data_ptr(), div_mass_lumped.data_ptr(),
                                            grad_mass_lumped.data_ptr(), ft._stream_ptr(stream)),
          "fl_dev_assemble_divergence_cg")
    del keep
    return {"ct": ct, "ct_rhs": ct_rhs, "div_mass_lumped": div_mass_lumped, "grad_mass_lumped": grad_mass_lumped}


def compute_lumped_mass(mesh: ft.Mesh, out=None, stream=None):
    torch = _torch()
    if out is None:
        out = torch.empty(mesh.N, dtype=torch.float64, device="cuda")
    check(_lib.load().fl_dev_lumped_mass(mesh.handle, out.data_ptr(), ft._stream_ptr(stream)),
          "fl_dev_lumped_mass")
    return out


def inverse_lumped_mass(lumped_mass, dirichlet_nodes=None):
    """The momentum solve's inverse_masslump (Momentum_CG.F90:847-877): the
    lumped mass per component, inverted, zero at each component's strong
    Dirichlet nodes (apply_dirichlet_conditions_inverse_mass).
    ``dirichlet_nodes`` is one index array per component, or one for all."""
    torch = _torch()
    inv = (1.0 / lumped_mass).unsqueeze(1).repeat(1, 3).contiguous()
    if dirichlet_nodes is not None:
        per = dirichlet_nodes if isinstance(dirichlet_nodes, (list, tuple)) else [dirichlet_nodes] * 3
        for d, nodes in enumerate(per):
            idx = torch.as_tensor(np.asarray(nodes, dtype=np.int64), device=inv.device)
            inv[idx, d] = 0.0
    return inv


def mult_div_vector_div_T(product: SecondOrderPattern, a, w, b, out=None, stream=None):
    """product = a diag(w) b^T with ndim blocks (mult_div_vector_div_T)."""
    torch = _torch()
    ndim = a.shape[0]
    if out is None:
        out = torch.empty(product.nnz, dtype=torch.float64, device="cuda")
    check(_lib.load().fl_dev_mult_div_vector_div_T(product.handle, ndim, _ptrs([a[d] for d in range(ndim)]),
                                                  w.data_ptr(), _ptrs([b[d] for d in range(ndim)]),
                                                  out.data_ptr(), ft._stream_ptr(stream)),
          "fl_dev_mult_div_vector_div_T")
    return out


def mult_div_invscalar_div_T(product: SecondOrderPattern, a, s, b, out=None, stream=None):
    torch = _torch()
    if out is None:
        out = torch.empty(product.nnz, dtype=torch.float64, device="cuda")
    check(_lib.load().fl_dev_mult_div_invscalar_div_T(product.handle, a.data_ptr(), s.data_ptr(), b.data_ptr(),
                                                     out.data_ptr(), ft._stream_ptr(stream)),
          "fl_dev_mult_div_invscalar_div_T")
    return out


def assemble_masslumped_cmc(product: SecondOrderPattern, ctp, inverse_masslump, ct, out=None, stream=None):
    """C_P^T M_l^-1 C (Assemble_CMC.F90:119-135)."""
    return mult_div_vector_div_T(product, ctp, inverse_masslump, ct, out, stream)


def assemble_kmk_matrix(mesh: ft.Mesh, product: SecondOrderPattern, p_masslump, theta_pg=1.0, kmk=None, kt=None,
                        stream=None):
    """(kmk, kt) of assemble_kmk_matrix (Momentum_CG.F90:2707-2766)."""
    torch = _torch()
    if kmk is None:
        kmk = torch.empty(product.nnz, dtype=torch.float64, device="cuda")
    if kt is None:
        kt = torch.empty(mesh.nnz, dtype=torch.float64, device="cuda")
    check(_lib.load().fl_dev_assemble_kmk(mesh.handle, product.handle, float(theta_pg), p_masslump.data_ptr(),
                                         kt.data_ptr(), kmk.data_ptr(), ft._stream_ptr(stream)),
          "fl_dev_assemble_kmk")
    return kmk, kt


def add_kmk_matrix(product: SecondOrderPattern, cmc, kmk, stream=None):
    check(_lib.load().fl_dev_csr_addto(product.handle, cmc.data_ptr(), kmk.data_ptr(), 1.0, ft._stream_ptr(stream)),
          "fl_dev_csr_addto")
    return cmc


def assemble_masslumped_poisson_rhs(mesh: ft.Mesh, ctp, mom_rhs, ct_rhs, inverse_masslump, velocity, dt,
                                    theta_pg, out=None, stream=None):
    torch = _torch()
    if out is None:
        out = torch.empty(mesh.N, dtype=torch.float64, device="cuda")
    check(_lib.load().fl_dev_masslumped_poisson_rhs(
        mesh.handle, _ptrs([ctp[0], ctp[1], ctp[2]]), mom_rhs.data_ptr() if mom_rhs is not None else None,
        ct_rhs.data_ptr() if ct_rhs is not None else None,
        inverse_masslump.data_ptr() if inverse_masslump is not None else None, velocity.data_ptr(),
        float(dt), float(theta_pg), out.data_ptr(), ft._stream_ptr(stream)), "fl_dev_masslumped_poisson_rhs")
    return out


def correct_masslumped_velocity(mesh: ft.Mesh, ct, inverse_masslump, delta_p, velocity, stream=None):
    check(_lib.load().fl_dev_correct_masslumped_velocity(mesh.handle, _ptrs([ct[0], ct[1], ct[2]]),
                                                         inverse_masslump.data_ptr(), delta_p.data_ptr(),
                                                         velocity.data_ptr(), ft._stream_ptr(stream)),
          "fl_dev_correct_masslumped_velocity")
    return velocity
