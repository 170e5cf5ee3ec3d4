"""Python mirror of Fluidity's CG hot-path interface, backed by the CUDA library.

Names and argument meanings follow the reference routines they replace:

==============================  ================================================
this module                     reference
==============================  ================================================
``Mesh``                        ``mesh_type`` + coordinate ``vector_field``
``make_sparsity``               ``get_csr_sparsity_firstorder`` ->
                                ``make_sparsity`` (Sparsity_Patterns.F90:47)
``get_mesh_colouring``          ``get_mesh_colouring(..., COLOURING_CG1, ...)``
                                (Colouring.F90:85)
``make_global_numbering_p2``    ``make_global_numbering`` (Global_Numbering.F90:291)
``assemble_advection_diffusion_cg``  Advection_Diffusion_CG.F90:228
``apply_dirichlet_conditions``  Boundary_Conditions.F90:1983
``petsc_solve``                 Solvers.F90:111 (petsc_solve_scalar)
``solve_field_equation_cg``     Advection_Diffusion_CG.F90:127
``Batch``                       many ``solve_field_equation_cg`` steps at once
``autotune_assembly``           (no counterpart: assembly tile choice)
==============================  ================================================

Arrays are numpy (host, copied through the ``fl_gpu_*`` entry points) or torch
CUDA tensors (device-resident, ``fl_dev_*`` entry points).  Indices are 0-based.
Every call runs on the GPU; a missing library or device raises.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import AdvDifParams, FaceBcs, Fields, MeshDesc, SolveReport, SolverOpts, check


def _ptr(a):
    """Data pointer of a numpy array or torch tensor (None passes through)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()


def _is_device(a) -> bool:
    return a is not None and not isinstance(a, np.ndarray)


def _stream_ptr(stream):
    """CUDA stream handle for device-path calls: the given stream, or torch's
    current stream so the library's work is ordered with the caller's tensors.
    Torch's default stream is the legacy default stream (handle 0), which the
    C-ABI reads as "the mesh's own stream": it is passed as cudaStreamLegacy."""
    if stream is None:
        import torch
        stream = torch.cuda.current_stream()
    h = getattr(stream, "cuda_stream", stream)
    return h if h else 1  # cudaStreamLegacy


@dataclass
class CsrSparsity:
    """csr_sparsity (Sparse_Tools.F90:48-111), 0-based; centrm = -1 if no diagonal."""
    findrm: np.ndarray
    colm: np.ndarray
    centrm: np.ndarray

    @property
    def nnz(self) -> int:
        return int(self.colm.size)


class Mesh:
    """A field mesh registered on the GPU with its coordinate (P1) mesh.

    ``ndglno`` (E, loc) and ``x_ndglno`` (E, 4) are element-major connectivities,
    ``coords`` is (Nx, 3).  Registration builds the sparsity and the CG1
    colouring on the device and caches them, as the reference caches them in
    state / on the topology mesh.
    """

    def __init__(self, ndglno, coords, x_ndglno=None, nodes=None, index_base=0):
        self.lib = _lib.load()
        nd = np.ascontiguousarray(ndglno, dtype=np.int32)
        self.E, self.loc = nd.shape
        xnd = nd if x_ndglno is None else np.ascontiguousarray(x_ndglno, dtype=np.int32)
        X = np.ascontiguousarray(coords, dtype=np.float64)
        self.N = int(nodes if nodes is not None else nd.max() + 1 - index_base)
        self.Nx = int(X.shape[0])
        d = MeshDesc(self.N, self.E, self.loc, index_base, nd.ctypes.data, self.Nx,
                     xnd.ctypes.data, X.ctypes.data)
        h = C.c_void_p()
        check(self.lib.fl_gpu_mesh_register(C.byref(d), C.byref(h)), "fl_gpu_mesh_register")
        self.handle = h
        nnz, ncol = C.c_int64(), C.c_int32()
        check(self.lib.fl_gpu_mesh_info(h, C.byref(nnz), C.byref(ncol)), "fl_gpu_mesh_info")
        self.nnz, self.ncolours = nnz.value, ncol.value
        self._sparsity = None

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fl_gpu_mesh_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def tiles(self) -> tuple:
        """Assembly tiles in use: (element block, element blocks per SM, row tile)."""
        t = (C.c_int32 * 3)()
        check(self.lib.fl_get_assembly_tiles(self.handle, t), "fl_get_assembly_tiles")
        return tuple(int(v) for v in t)

    def sparsity(self) -> CsrSparsity:
        if self._sparsity is None:
            f = np.empty(self.N + 1, dtype=np.int32)
            c = np.empty(self.nnz, dtype=np.int32)
            d = np.empty(self.N, dtype=np.int32)
            check(self.lib.fl_gpu_sparsity_copy(self.handle, _ptr(f), _ptr(c), _ptr(d), 0),
                  "fl_gpu_sparsity_copy")
            self._sparsity = CsrSparsity(f, c, d)
        return self._sparsity

    def colouring(self):
        """(colour per element 1-based, colour_ptr (ncol+1), colour_elems)."""
        col = np.empty(self.E, dtype=np.int32)
        ptr = np.empty(self.ncolours + 1, dtype=np.int32)
        el = np.empty(self.E, dtype=np.int32)
        check(self.lib.fl_gpu_colouring_copy(self.handle, _ptr(col), _ptr(ptr), _ptr(el), 0),
              "fl_gpu_colouring_copy")
        return col, ptr, el


def make_sparsity(mesh: Mesh) -> CsrSparsity:
    """First-order sparsity of the mesh (get_csr_sparsity_firstorder)."""
    return mesh.sparsity()


def get_mesh_colouring(mesh: Mesh):
    """COLOURING_CG1 colour sets: list of ascending element arrays."""
    _, ptr, el = mesh.colouring()
    return [el[ptr[c]:ptr[c + 1]] for c in range(mesh.ncolours)]


def make_global_numbering_p2(ndglno_p1, nvert: int | None = None):
    """P2 connectivity (E, 10) and node count derived from a P1 tet mesh."""
    lib = _lib.load()
    nd = np.ascontiguousarray(ndglno_p1, dtype=np.int32)
    E = nd.shape[0]
    nv = int(nvert if nvert is not None else nd.max() + 1)
    out = np.empty((E, 10), dtype=np.int32)
    n2 = C.c_int32()
    check(lib.fl_gpu_make_global_numbering_p2(nv, E, _ptr(nd), 0, _ptr(out), C.byref(n2)),
          "fl_gpu_make_global_numbering_p2")
    return out, n2.value


def advdif_params(*, theta=1.0, dt=1.0, beta=0.0, have_mass=False, lump_mass=False,
                  have_advection=False, diffusivity=None, have_source=False,
                  have_absorption=False, quad_degree=2, integrate_advection_by_parts=False) -> AdvDifParams:
    """The options assemble_advection_diffusion_cg reads (Advection_Diffusion_CG.F90:384-465)."""
    p = AdvDifParams()
    p.integrate_advection_by_parts = int(integrate_advection_by_parts)
    p.theta, p.dt, p.beta = theta, dt, beta
    p.have_mass, p.lump_mass = int(have_mass), int(have_mass and lump_mass)
    p.have_advection = int(have_advection)
    p.have_source, p.have_absorption = int(have_source), int(have_absorption)
    p.quad_degree = quad_degree
    if diffusivity is None:
        p.have_diffusivity, p.isotropic_diffusivity = 0, 1
    else:
        K = np.asarray(diffusivity, dtype=np.float64)
        if K.ndim == 0:
            K = np.eye(3) * float(K)
        p.have_diffusivity = 1
        p.isotropic_diffusivity = int(np.array_equal(K, np.eye(3) * K[0, 0]))
        for k in range(9):
            p.diffusivity[k] = K.reshape(-1)[k]
    return p


def assemble_advection_diffusion_cg(mesh: Mesh, params: AdvDifParams, *, t=None, velocity=None,
                                    source=None, absorption=None, val=None, rhs=None, stream=None):
    """Matrix values (nnz) and rhs (N) of the CG advection-diffusion equation.

    Host numpy fields -> host results through fl_gpu_assemble_advdif_cg; torch
    CUDA fields -> device results through fl_dev_assemble_advdif_cg.
    """
    lib = mesh.lib
    dev = any(_is_device(a) for a in (t, velocity, source, absorption, val, rhs))
    if dev:
        import torch
        if val is None:
            val = torch.empty(mesh.nnz, dtype=torch.float64, device="cuda")
        if rhs is None:
            rhs = torch.empty(mesh.N, dtype=torch.float64, device="cuda")
        f = Fields(_ptr(t), _ptr(velocity), _ptr(source), _ptr(absorption))
        check(lib.fl_dev_assemble_advdif_cg(mesh.handle, C.byref(params), C.byref(f), _ptr(val),
                                            _ptr(rhs), _stream_ptr(stream)),
              "fl_dev_assemble_advdif_cg")
        return val, rhs
    keep = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None
            for a in (t, velocity, source, absorption)]
    f = Fields(*[_ptr(a) for a in keep])
    val = np.empty(mesh.nnz) if val is None else val
    rhs = np.empty(mesh.N) if rhs is None else rhs
    check(lib.fl_gpu_assemble_advdif_cg(mesh.handle, C.byref(params), C.byref(f), _ptr(val),
                                        _ptr(rhs)), "fl_gpu_assemble_advdif_cg")
    return val, rhs


BC_NONE, BC_NEUMANN, BC_WEAKDIRICHLET, BC_INTERNAL, BC_ROBIN = 0, 1, 2, 3, 4


def assemble_advection_diffusion_faces(mesh: Mesh, params: AdvDifParams, val, rhs, *, faces, xfaces,
                                       face_ele=None, bc_type=None, bc_value=None, bc_value2=None,
                                       t=None, velocity=None, index_base=0, stream=None):
    """The surface loop of assemble_advection_diffusion_cg (Advection_Diffusion_CG.F90:
    608-640 -> assemble_advection_diffusion_face_cg :1228-1378) added into an
    assembled ``val``/``rhs`` in place, before the strong Dirichlet conditions.

    ``faces`` (nf, floc) field nodes of the surface elements (floc 3 for P1,
    6 for P2 in the triangle's local order), ``xfaces`` (nf, 3) their
    coordinate vertices, ``face_ele`` (nf,) their elements (needed for the
    outward normal with advection by parts); ``bc_type`` (nf,) 0 none,
    1 neumann, 2 weakdirichlet, 3 internal, 4 robin; ``bc_value`` /
    ``bc_value2`` (nf, floc) the condition's fields at the face nodes.
    torch CUDA arrays run the device entry point, numpy arrays the host one.
    """
    lib = mesh.lib
    dev = any(_is_device(a) for a in (val, rhs, faces, t, velocity))
    arrs = {"faces": faces, "xfaces": xfaces, "face_ele": face_ele, "bc_type": bc_type}
    if dev:
        import torch
        conv = {k: (torch.as_tensor(v, dtype=torch.int32, device="cuda").contiguous() if v is not None else None)
                for k, v in arrs.items()}
        dbl = [torch.as_tensor(v, dtype=torch.float64, device="cuda").contiguous() if v is not None else None
               for v in (bc_value, bc_value2)]
    else:
        conv = {k: (np.ascontiguousarray(v, dtype=np.int32) if v is not None else None) for k, v in arrs.items()}
        dbl = [np.ascontiguousarray(v, dtype=np.float64) if v is not None else None for v in (bc_value, bc_value2)]
    fc = conv["faces"]
    nf, floc = int(fc.shape[0]), int(fc.shape[1])
    fb = FaceBcs(nf, floc, index_base, 0, _ptr(fc), _ptr(conv["xfaces"]), _ptr(conv["face_ele"]),
                 _ptr(conv["bc_type"]), _ptr(dbl[0]), _ptr(dbl[1]))
    if dev:
        f = Fields(_ptr(t), _ptr(velocity), None, None)
        check(lib.fl_dev_assemble_advdif_faces(mesh.handle, C.byref(params), C.byref(fb), C.byref(f), _ptr(val),
                                               _ptr(rhs), _stream_ptr(stream)), "fl_dev_assemble_advdif_faces")
        return val, rhs
    keep = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None for a in (t, velocity)]
    f = Fields(_ptr(keep[0]), _ptr(keep[1]), None, None)
    check(lib.fl_gpu_assemble_advdif_faces(mesh.handle, C.byref(params), C.byref(fb), C.byref(f), _ptr(val),
                                           _ptr(rhs)), "fl_gpu_assemble_advdif_faces")
    return val, rhs


def apply_dirichlet_conditions(mesh: Mesh, rhs, inactive, nodes, values, t=None, dt=None,
                               stream=None):
    """Strong Dirichlet: rows inactive, rhs = (g - t)/dt (or g without dt)."""
    lib = mesh.lib
    dtv = float(dt) if dt is not None else 0.0
    if _is_device(rhs):
        check(lib.fl_dev_apply_dirichlet(mesh.handle, int(len(nodes)), _ptr(nodes), 0, _ptr(values),
                                         _ptr(t), C.c_double(dtv), _ptr(rhs), _ptr(inactive),
                                         _stream_ptr(stream)), "fl_dev_apply_dirichlet")
        return
    nodes = np.ascontiguousarray(nodes, dtype=np.int32)
    values = np.ascontiguousarray(values, dtype=np.float64)
    tv = np.ascontiguousarray(t, dtype=np.float64) if t is not None else None
    check(lib.fl_gpu_apply_dirichlet(mesh.handle, int(nodes.size), _ptr(nodes), 0, _ptr(values),
                                     _ptr(tv), C.c_double(dtv), _ptr(rhs), _ptr(inactive)),
          "fl_gpu_apply_dirichlet")


def solver_options(*, ksp="cg", restart=30, rtol=1e-10, atol=0.0, dtol=1e5, max_its=10000,
                   start_from_zero=False, precision="fp64", inner_rtol=1e-5,
                   norm="preconditioned", schedule="auto") -> SolverOpts:
    """solver/ options of the field (Solvers.F90:1566-1660); pc is always jacobi.

    ``norm`` is the residual norm of the convergence test (KSPSetNormType):
    "preconditioned" ||B r|| is PETSc's default; "unpreconditioned" ||r||
    (CG only) makes rtol bound the true relative residual ||b - Ax|| / ||b||.
    ``schedule`` picks how an FP64 GMRES solve is launched: "graph" (a launch
    per Arnoldi phase, cycles replayed as CUDA graphs), "persistent" (one
    cooperative launch for the whole solve) or "auto" (persistent up to
    FL_PERSIST_MAX_ROWS = 81,920 rows)."""
    o = SolverOpts()
    o.ksp_type = {"cg": 0, "gmres": 1}[ksp]
    o.restart, o.rtol, o.atol, o.dtol = restart, rtol, atol, dtol
    o.max_its, o.start_from_zero = max_its, int(start_from_zero)
    o.precision = {"fp64": 0, "mixed": 1, "reliable": 2}[precision]
    o.inner_rtol = inner_rtol
    o.norm_type = {"preconditioned": 0, "unpreconditioned": 1}[norm]
    o.schedule = {"auto": 0, "graph": 1, "persistent": 2}[schedule]
    return o


def petsc_solve(mesh: Mesh, x, val, rhs, options: SolverOpts, inactive=None, stream=None) -> dict:
    """Solve A x = rhs on the mesh pattern; x holds the guess and receives the solution."""
    lib = mesh.lib
    rep = SolveReport()
    if _is_device(x):
        check(lib.fl_dev_petsc_solve(mesh.handle, C.byref(options), _ptr(val), _ptr(inactive),
                                     _ptr(rhs), _ptr(x), C.byref(rep), _stream_ptr(stream)),
              "fl_dev_petsc_solve")
    else:
        v = np.ascontiguousarray(val, dtype=np.float64)
        b = np.ascontiguousarray(rhs, dtype=np.float64)
        ina = np.ascontiguousarray(inactive, dtype=np.uint8) if inactive is not None else None
        check(lib.fl_gpu_petsc_solve(mesh.handle, C.byref(options), _ptr(v), _ptr(ina), _ptr(b),
                                     _ptr(x), C.byref(rep)), "fl_gpu_petsc_solve")
    return _report_dict(rep)


class AmgPreconditioner:
    """Smoothed-aggregation AMG hierarchy of one assembled matrix (fl_amg_*),
    the counterpart of petsc_solve's gamg preconditioner.  `val` and
    `inactive` are device tensors that must not change while it is used."""

    def __init__(self, mesh: Mesh, val, inactive=None, stream=None, unpreconditioned_norm=False):
        self.lib = mesh.lib
        self.mesh = mesh
        self._keep = (val, inactive)
        h = C.c_void_p()
        check(self.lib.fl_amg_create(mesh.handle, _ptr(val), _ptr(inactive), _stream_ptr(stream),
                                     C.byref(h)), "fl_amg_create")
        self.handle = h.value
        if unpreconditioned_norm:
            check(self.lib.fl_amg_set_norm(self.handle, 1), "fl_amg_set_norm")

    def set_precision(self, fp32: bool):
        """FP32 (True) or FP64 (False) arithmetic inside the V-cycle."""
        check(self.lib.fl_amg_set_precision(self.handle, int(fp32)), "fl_amg_set_precision")

    def levels(self):
        """[(rows, nonzeros)] of every level, finest first."""
        cap = 16
        nl = C.c_int32()
        rows = (C.c_int64 * cap)()
        nnz = (C.c_int64 * cap)()
        check(self.lib.fl_amg_levels(self.handle, C.byref(nl), rows, nnz, cap), "fl_amg_levels")
        return [(int(rows[i]), int(nnz[i])) for i in range(nl.value)]

    def solve(self, x, rhs, options: SolverOpts, stream=None) -> dict:
        """CG preconditioned by the hierarchy: x holds the guess, receives the solution."""
        rep = SolveReport()
        check(self.lib.fl_amg_solve(self.handle, C.byref(options), _ptr(rhs), _ptr(x), C.byref(rep),
                                    _stream_ptr(stream)), "fl_amg_solve")
        return _report_dict(rep)

    def close(self):
        if self.handle:
            self.lib.fl_amg_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def projected_guess(mesh: Mesh, val, rhs, basis, inactive=None, out=None, stream=None):
    """Initial guess x0 = V a minimising the A-norm error over span(basis)
    (the projection method for successive right-hand sides, Fischer 1998) on
    the ghost-reduced system petsc_solve solves; device tensors.  Returns
    (x0, a)."""
    import torch
    k = len(basis)
    ptrs = (C.c_void_p * k)(*[b.data_ptr() for b in basis])
    coef = np.zeros(k)
    if out is None:
        out = torch.empty(mesh.N, dtype=torch.float64, device="cuda")
    check(mesh.lib.fl_dev_projected_guess(mesh.handle, _ptr(val), _ptr(inactive), _ptr(rhs), k, ptrs,
                                          _ptr(out), coef.ctypes.data, _stream_ptr(stream)),
          "fl_dev_projected_guess")
    return out, coef


def csr_mult(mesh: Mesh, val, x, y, stream=None):
    """y = A x (device tensors)."""
    check(mesh.lib.fl_dev_csr_mult(mesh.handle, _ptr(val), _ptr(x), _ptr(y), _stream_ptr(stream)),
          "fl_dev_csr_mult")


def solve_field_equation_cg(mesh: Mesh, t, params: AdvDifParams, options: SolverOpts, *,
                            bc_nodes, bc_values, velocity=None, source=None, absorption=None):
    """One solve of a CG scalar field in acceleration form (Advection_Diffusion_CG.F90:127-174).

    Assembles (M + theta dt (A + K)) delta_t = rhs, applies strong Dirichlet
    conditions in rate-of-change form, solves for delta_t with zero initial
    change and returns (t + dt * delta_t, solve report).  Host numpy arrays.
    """
    val, rhs = assemble_advection_diffusion_cg(mesh, params, t=t, velocity=velocity, source=source,
                                               absorption=absorption)
    inactive = np.zeros(mesh.N, dtype=np.uint8)
    apply_dirichlet_conditions(mesh, rhs, inactive, bc_nodes, bc_values, t=t, dt=params.dt)
    delta = np.zeros(mesh.N)
    rep = petsc_solve(mesh, delta, val, rhs, options, inactive=inactive)
    return t + params.dt * delta, rep


def solve_field_equation_cg_device(mesh: Mesh, t, params: AdvDifParams, options: SolverOpts, *, bc_nodes,
                                   bc_values, velocity=None, source=None, absorption=None, t_out=None,
                                   stream=None) -> tuple:
    """The device form of solve_field_equation_cg (device tensors): one
    fl_dev_solve_field_equation_cg call assembles, applies the strong
    Dirichlet conditions in rate-of-change form, solves for the change from
    zero and returns (t + dt * delta, solve report), with one error check
    for the whole step.  Scratch (val, rhs, inactive, delta) is kept on the
    mesh object between calls."""
    import torch
    sc = getattr(mesh, "_sfe_scratch", None)
    if sc is None or sc["val"].numel() != mesh.nnz:
        dev = t.device
        sc = {"val": torch.empty(mesh.nnz, dtype=torch.float64, device=dev),
              "rhs": torch.empty(mesh.N, dtype=torch.float64, device=dev),
              "inactive": torch.empty(mesh.N, dtype=torch.uint8, device=dev),
              "delta": torch.empty(mesh.N, dtype=torch.float64, device=dev)}
        mesh._sfe_scratch = sc
    out = t_out if t_out is not None else torch.empty_like(t)
    f = Fields(_ptr(t), _ptr(velocity), _ptr(source), _ptr(absorption))
    rep = SolveReport()
    check(mesh.lib.fl_dev_solve_field_equation_cg(
        mesh.handle, C.byref(params), C.byref(f), int(len(bc_nodes)), _ptr(bc_nodes), 0, _ptr(bc_values),
        C.byref(options), _ptr(sc["val"]), _ptr(sc["rhs"]), _ptr(sc["inactive"]), _ptr(sc["delta"]),
        _ptr(out), C.byref(rep), _stream_ptr(stream)), "fl_dev_solve_field_equation_cg")
    return out, _report_dict(rep)


def _report_dict(rep: SolveReport) -> dict:
    return {
        "iterations": rep.iterations, "reason": rep.reason,
        "reason_name": _lib.REASONS.get(rep.reason, str(rep.reason)),
        "final_rnorm": rep.final_rnorm, "rnorm0": rep.rnorm0,
        "true_rel_residual": rep.true_rel_residual, "outer_iterations": rep.outer_iterations,
    }


def autotune_assembly(mesh: Mesh, params: AdvDifParams, *, t=None, velocity=None, source=None,
                      absorption=None, val=None, rhs=None, stream=None):
    """Pick the fastest assembly tiles for this mesh (device tensors).

    Returns (val, rhs, tiles) with the assembled system and the chosen
    (element block, element blocks per SM, row tile); later assemblies on the
    mesh use the tiles.  Results do not depend on them.
    """
    import torch
    if val is None:
        val = torch.empty(mesh.nnz, dtype=torch.float64, device="cuda")
    if rhs is None:
        rhs = torch.empty(mesh.N, dtype=torch.float64, device="cuda")
    f = Fields(_ptr(t), _ptr(velocity), _ptr(source), _ptr(absorption))
    tiles = (C.c_int32 * 3)()
    check(mesh.lib.fl_dev_autotune_assembly(mesh.handle, C.byref(params), C.byref(f), _ptr(val),
                                            _ptr(rhs), _stream_ptr(stream), tiles),
          "fl_dev_autotune_assembly")
    return val, rhs, tuple(int(v) for v in tiles)


def set_assembly_tiles(mesh: Mesh, elem_block: int, elem_blocks_per_sm: int, row_tile: int):
    check(mesh.lib.fl_set_assembly_tiles(mesh.handle, elem_block, elem_blocks_per_sm, row_tile),
          "fl_set_assembly_tiles")


class Batch:
    """Many solve_field_equation_cg steps run as CUDA graphs (fl_batch_*).

    Each ``add`` registers one step on device tensors: assembly of ``params``
    with the given fields, strong Dirichlet conditions on ``bc_nodes`` in
    rate-of-change form, and a solve with ``options`` into ``x`` (the initial
    guess unless start_from_zero).  ``run`` executes every member and returns
    their solve reports; the tensors are read at run time, so a later ``run``
    sees their new contents.  The batch keeps references to every tensor.
    """

    def __init__(self):
        self.lib = _lib.load()
        h = C.c_void_p()
        check(self.lib.fl_batch_create(C.byref(h)), "fl_batch_create")
        self.handle = h.value
        self._keep = []
        self.members = []

    def add(self, mesh: Mesh, params: AdvDifParams, options: SolverOpts, *, bc_nodes, bc_values,
            t=None, velocity=None, source=None, absorption=None, x=None):
        import torch
        dev = torch.device("cuda")
        val = torch.empty(mesh.nnz, dtype=torch.float64, device=dev)
        rhs = torch.empty(mesh.N, dtype=torch.float64, device=dev)
        inactive = torch.zeros(mesh.N, dtype=torch.uint8, device=dev)
        if x is None:
            x = torch.zeros(mesh.N, dtype=torch.float64, device=dev)
        nodes = torch.as_tensor(bc_nodes, dtype=torch.int32, device=dev).contiguous()
        values = torch.as_tensor(bc_values, dtype=torch.float64, device=dev).contiguous()
        f = Fields(_ptr(t), _ptr(velocity), _ptr(source), _ptr(absorption))
        check(self.lib.fl_batch_add(self.handle, mesh.handle, C.byref(params), C.byref(f),
                                    int(nodes.numel()), _ptr(nodes), 0, _ptr(values),
                                    C.byref(options), _ptr(val), _ptr(rhs), _ptr(inactive), _ptr(x)),
              "fl_batch_add")
        m = {"mesh": mesh, "val": val, "rhs": rhs, "inactive": inactive, "x": x}
        self._keep.append((params, options, nodes, values, t, velocity, source, absorption))
        self.members.append(m)
        return m

    def run(self, stream=None) -> list[dict]:
        n = len(self.members)
        reps = (SolveReport * max(n, 1))()
        check(self.lib.fl_batch_run(self.handle, _stream_ptr(stream), reps), "fl_batch_run")
        return [_report_dict(reps[i]) for i in range(n)]

    def close(self):
        if self.handle:
            self.lib.fl_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kernel_launch_count() -> int:
    """Kernels this library launched in this process so far (all devices' counters)."""
    return int(_lib.load().fl_kernel_launch_count())
