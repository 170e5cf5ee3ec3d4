"""ctypes binding of ``libfluidity_gb300.so`` (the C-ABI of include/fluidity_gb300.h).

The structures below mirror the C declarations field for field.  Loading fails
loudly when the library cannot be built or loaded: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import threading

from . import build as _build

FL_OK = 0
STATUS = {
    0: "FL_OK", 1: "FL_ERR_ARG", 2: "FL_ERR_CUDA", 3: "FL_ERR_OUTSIDE_PATTERN",
    4: "FL_ERR_TIMEOUT", 5: "FL_ERR_COLOURS", 6: "FL_ERR_NOMEM", 7: "FL_ERR_UNSUPPORTED",
}
REASONS = {
    2: "KSP_CONVERGED_RTOL", 3: "KSP_CONVERGED_ATOL", -2: "KSP_DIVERGED_NULL",
    -3: "KSP_DIVERGED_ITS", -4: "KSP_DIVERGED_DTOL", -5: "KSP_DIVERGED_BREAKDOWN",
    -8: "KSP_DIVERGED_INDEFINITE_PC", -9: "KSP_DIVERGED_NANORINF",
    -10: "KSP_DIVERGED_INDEFINITE_MAT",
}


class FlError(RuntimeError):
    """A non-OK fl_status from the library (FLAbort/FLExit in the reference)."""

    def __init__(self, status: int, where: str, message: str):
        super().__init__(f"{where}: {STATUS.get(status, status)}: {message}")
        self.status = status


class MeshDesc(C.Structure):
    _fields_ = [
        ("nodes", C.c_int32), ("elements", C.c_int32), ("loc", C.c_int32),
        ("index_base", C.c_int32), ("ndglno", C.c_void_p), ("x_nodes", C.c_int32),
        ("x_ndglno", C.c_void_p), ("coords", C.c_void_p),
    ]


class AdvDifParams(C.Structure):
    _fields_ = [
        ("theta", C.c_double), ("dt", C.c_double), ("beta", C.c_double),
        ("have_mass", C.c_int32), ("lump_mass", C.c_int32), ("have_advection", C.c_int32),
        ("have_diffusivity", C.c_int32), ("isotropic_diffusivity", C.c_int32),
        ("have_source", C.c_int32), ("have_absorption", C.c_int32), ("quad_degree", C.c_int32),
        ("diffusivity", C.c_double * 9), ("integrate_advection_by_parts", C.c_int32), ("pad", C.c_int32),
    ]


class FaceBcs(C.Structure):
    _fields_ = [
        ("nfaces", C.c_int32), ("floc", C.c_int32), ("index_base", C.c_int32), ("pad", C.c_int32),
        ("faces", C.c_void_p), ("xfaces", C.c_void_p), ("face_ele", C.c_void_p), ("bc_type", C.c_void_p),
        ("bc_value", C.c_void_p), ("bc_value2", C.c_void_p),
    ]


class Fields(C.Structure):
    _fields_ = [("t", C.c_void_p), ("velocity", C.c_void_p), ("source", C.c_void_p),
                ("absorption", C.c_void_p)]


class SolverOpts(C.Structure):
    _fields_ = [
        ("ksp_type", C.c_int32), ("restart", C.c_int32), ("rtol", C.c_double),
        ("atol", C.c_double), ("dtol", C.c_double), ("max_its", C.c_int32),
        ("start_from_zero", C.c_int32), ("precision", C.c_int32), ("inner_rtol", C.c_double),
        ("norm_type", C.c_int32), ("schedule", C.c_int32),
    ]


class DivergenceParams(C.Structure):
    _fields_ = [
        ("integrate_by_parts", C.c_int32), ("nfaces", C.c_int32), ("index_base", C.c_int32),
        ("pad", C.c_int32), ("faces", C.c_void_p), ("face_ele", C.c_void_p), ("bc_type", C.c_void_p),
        ("bc_val", C.c_void_p),
    ]


class SolveReport(C.Structure):
    _fields_ = [
        ("iterations", C.c_int32), ("reason", C.c_int32), ("final_rnorm", C.c_double),
        ("rnorm0", C.c_double), ("true_rel_residual", C.c_double),
        ("outer_iterations", C.c_int32), ("pad", C.c_int32),
    ]


#: Every entry point declared in include/fluidity_gb300.h.
EXPORTS = [
    "fl_last_error", "fl_gpu_mesh_register", "fl_gpu_mesh_destroy", "fl_gpu_mesh_info",
    "fl_gpu_sparsity_copy", "fl_gpu_colouring_copy", "fl_gpu_make_global_numbering_p2",
    "fl_gpu_assemble_advdif_cg", "fl_dev_assemble_advdif_cg", "fl_gpu_apply_dirichlet",
    "fl_dev_apply_dirichlet", "fl_gpu_petsc_solve", "fl_dev_petsc_solve", "fl_dev_solve_field_equation_cg",
    "fl_dev_csr_mult",
    "fl_kernel_launch_count", "fl_set_kernel_timing", "fl_last_assembly_kernel_ms",
    "fl_dev_assemble_p1_diffusion_noalloc", "fl_dev_autotune_assembly", "fl_set_assembly_tiles",
    "fl_get_assembly_tiles",
    "fl_batch_create", "fl_batch_add", "fl_batch_run", "fl_batch_size", "fl_batch_destroy",
    "fl_gnn_num_params", "fl_gnn_create", "fl_gnn_destroy", "fl_gnn_set_weights",
    "fl_gnn_get_weights", "fl_gnn_predict", "fl_gnn_gradients", "fl_gnn_train_step",
    "fl_gnn_set_loss", "fl_gpu_pattern_register",
    "fl_amg_create", "fl_amg_solve", "fl_amg_levels", "fl_amg_destroy", "fl_amg_set_norm", "fl_amg_set_precision",
    "fl_gpu_secondorder_register", "fl_dev_assemble_divergence_cg", "fl_dev_lumped_mass",
    "fl_dev_mult_div_vector_div_T", "fl_dev_mult_div_invscalar_div_T", "fl_dev_assemble_kmk",
    "fl_dev_masslumped_poisson_rhs", "fl_dev_correct_masslumped_velocity", "fl_dev_csr_addto",
    "fl_dev_assemble_advdif_faces", "fl_gpu_assemble_advdif_faces", "fl_set_wait_test",
    "fl_dev_projected_guess", "fl_gpu_rect_register", "fl_dev_assemble_divergence_p2p1",
    "fl_dev_assemble_divergence_p2p1_faces", "fl_gpu_rect_secondorder_register",
]

_P = C.c_void_p
_I32 = C.c_int32
_D = C.c_double
#: ctypes signatures of every entry point (pointers are c_void_p so 64-bit
#: host and device addresses pass unchanged).
_SIGNATURES = {
    "fl_last_error": (C.c_char_p, []),
    "fl_gpu_mesh_register": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(C.c_void_p)]),
    "fl_gpu_mesh_destroy": (C.c_int, [_P]),
    "fl_gpu_mesh_info": (C.c_int, [_P, C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "fl_gpu_sparsity_copy": (C.c_int, [_P, _P, _P, _P, _I32]),
    "fl_gpu_colouring_copy": (C.c_int, [_P, _P, _P, _P, _I32]),
    "fl_gpu_make_global_numbering_p2": (C.c_int, [_I32, _I32, _P, _I32, _P,
                                                  C.POINTER(C.c_int32)]),
    "fl_gpu_assemble_advdif_cg": (C.c_int, [_P, C.POINTER(AdvDifParams), C.POINTER(Fields), _P,
                                            _P]),
    "fl_dev_assemble_advdif_cg": (C.c_int, [_P, C.POINTER(AdvDifParams), C.POINTER(Fields), _P,
                                            _P, _P]),
    "fl_dev_assemble_p1_diffusion_noalloc": (C.c_int, [_P, C.POINTER(AdvDifParams),
                                                       C.POINTER(Fields), _P, _P, _P]),
    "fl_gpu_apply_dirichlet": (C.c_int, [_P, _I32, _P, _I32, _P, _P, _D, _P, _P]),
    "fl_dev_apply_dirichlet": (C.c_int, [_P, _I32, _P, _I32, _P, _P, _D, _P, _P, _P]),
    "fl_gpu_petsc_solve": (C.c_int, [_P, C.POINTER(SolverOpts), _P, _P, _P, _P,
                                     C.POINTER(SolveReport)]),
    "fl_dev_petsc_solve": (C.c_int, [_P, C.POINTER(SolverOpts), _P, _P, _P, _P,
                                     C.POINTER(SolveReport), _P]),
    "fl_dev_solve_field_equation_cg": (C.c_int, [_P, C.POINTER(AdvDifParams), C.POINTER(Fields), _I32, _P, _I32,
                                                 _P, C.POINTER(SolverOpts), _P, _P, _P, _P, _P,
                                                 C.POINTER(SolveReport), _P]),
    "fl_dev_csr_mult": (C.c_int, [_P, _P, _P, _P, _P]),
    "fl_kernel_launch_count": (C.c_int64, []),
    "fl_set_kernel_timing": (C.c_int, [_P, _I32]),
    "fl_last_assembly_kernel_ms": (C.c_int, [_P, C.POINTER(C.c_float)]),
    "fl_dev_autotune_assembly": (C.c_int, [_P, C.POINTER(AdvDifParams), C.POINTER(Fields), _P, _P,
                                           _P, C.POINTER(C.c_int32)]),
    "fl_set_assembly_tiles": (C.c_int, [_P, _I32, _I32, _I32]),
    "fl_get_assembly_tiles": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "fl_batch_create": (C.c_int, [C.POINTER(C.c_void_p)]),
    "fl_batch_add": (C.c_int, [_P, _P, C.POINTER(AdvDifParams), C.POINTER(Fields), _I32, _P, _I32,
                               _P, C.POINTER(SolverOpts), _P, _P, _P, _P]),
    "fl_batch_run": (C.c_int, [_P, _P, C.POINTER(SolveReport)]),
    "fl_batch_size": (C.c_int, [_P]),
    "fl_batch_destroy": (C.c_int, [_P]),
    "fl_gnn_num_params": (C.c_int, []),
    "fl_gnn_set_loss": (C.c_int, [_P, _P]),
    "fl_gpu_pattern_register": (C.c_int, [_I32, _P, _P, _I32, C.POINTER(C.c_void_p)]),
    "fl_amg_create": (C.c_int, [_P, _P, _P, _P, C.POINTER(C.c_void_p)]),
    "fl_amg_solve": (C.c_int, [_P, C.POINTER(SolverOpts), _P, _P, C.POINTER(SolveReport), _P]),
    "fl_amg_levels": (C.c_int, [_P, C.POINTER(C.c_int32), _P, _P, _I32]),
    "fl_amg_destroy": (C.c_int, [_P]),
    "fl_amg_set_norm": (C.c_int, [_P, _I32]),
    "fl_amg_set_precision": (C.c_int, [_P, _I32]),
    "fl_gnn_create": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "fl_gnn_destroy": (C.c_int, [_P]),
    "fl_gnn_set_weights": (C.c_int, [_P, _P, _I32]),
    "fl_gnn_get_weights": (C.c_int, [_P, _P, _I32]),
    "fl_gnn_predict": (C.c_int, [_P, _P, _P, _P, _P, _P]),
    "fl_gnn_gradients": (C.c_int, [_P, _P, _P, _P, _P, _P, _I32, _P, C.POINTER(C.c_float), _P]),
    "fl_gnn_train_step": (C.c_int, [_P, _P, _P, _P, _P, _P, _I32, C.c_float, _P, _P]),
    "fl_gpu_secondorder_register": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "fl_dev_assemble_divergence_cg": (C.c_int, [_P, C.POINTER(DivergenceParams), _P, _P, _P, _P, _P]),
    "fl_dev_lumped_mass": (C.c_int, [_P, _P, _P]),
    "fl_dev_mult_div_vector_div_T": (C.c_int, [_P, _I32, _P, _P, _P, _P, _P]),
    "fl_dev_mult_div_invscalar_div_T": (C.c_int, [_P, _P, _P, _P, _P, _P]),
    "fl_dev_assemble_kmk": (C.c_int, [_P, _P, _D, _P, _P, _P, _P]),
    "fl_dev_masslumped_poisson_rhs": (C.c_int, [_P, _P, _P, _P, _P, _P, _D, _D, _P, _P]),
    "fl_dev_correct_masslumped_velocity": (C.c_int, [_P, _P, _P, _P, _P, _P]),
    "fl_dev_csr_addto": (C.c_int, [_P, _P, _P, _D, _P]),
    "fl_dev_assemble_advdif_faces": (C.c_int, [_P, C.POINTER(AdvDifParams), C.POINTER(FaceBcs),
                                               C.POINTER(Fields), _P, _P, _P]),
    "fl_gpu_assemble_advdif_faces": (C.c_int, [_P, C.POINTER(AdvDifParams), C.POINTER(FaceBcs),
                                               C.POINTER(Fields), _P, _P]),
    "fl_set_wait_test": (C.c_int, [_I32, _D]),
    "fl_dev_projected_guess": (C.c_int, [_P, _P, _P, _P, _I32, _P, _P, _P, _P]),
    "fl_gpu_rect_register": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
    "fl_dev_assemble_divergence_p2p1": (C.c_int, [_P, _P, _I32, _I32, _P, _P]),
    "fl_dev_assemble_divergence_p2p1_faces": (C.c_int, [_P, _P, _P, _P, _I32, _P, _P, _P]),
    "fl_gpu_rect_secondorder_register": (C.c_int, [_P, C.POINTER(C.c_void_p)]),
}
assert sorted(_SIGNATURES) == sorted(EXPORTS)

_lib = None
_lock = threading.Lock()


def path() -> str:
    return _build.LIB


def load(build_if_needed: bool = True):
    """Load the CUDA library (building it first when stale)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if build_if_needed and not _build.up_to_date():
            _build.build()
        if not os.path.exists(_build.LIB):
            raise RuntimeError(f"{_build.LIB} is missing; run fluidity_gb300.build.build()")
        lib = C.CDLL(_build.LIB)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def check(status: int, where: str) -> None:
    if status != FL_OK:
        msg = load().fl_last_error().decode(errors="replace")
        raise FlError(status, where, msg)
