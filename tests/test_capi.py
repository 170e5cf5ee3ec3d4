"""The C-ABI library builds for sm_103a, loads, and exports every symbol the
public header declares (no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re
import subprocess

import pytest

from fluidity_gb300 import _lib, build

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include",
                      "fluidity_gb300.h")


def declared_symbols():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fl_[A-Za-z0-9_]+)\s*\(", txt)))


def test_header_and_binding_agree():
    assert declared_symbols() == sorted(_lib.EXPORTS)


def test_library_exports_every_symbol():
    path = build.build()
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    for name in declared_symbols():
        assert re.search(rf"\bT {name}\b", out), name


def test_every_entry_point_has_a_full_ctypes_signature():
    """Pointers cross as c_void_p: a missing argtypes list would truncate 64-bit addresses."""
    lib = _lib.load()
    for name in declared_symbols():
        fn = getattr(lib, name)
        assert fn.argtypes is not None, name
        assert fn.restype is not None, name


# Entry points whose null call is not an error: queries without arguments,
# destroy of a null handle (a no-op, as free(NULL)), and the size of no batch.
_NULL_OK = {"fl_last_error", "fl_kernel_launch_count", "fl_gnn_num_params", "fl_gpu_mesh_destroy",
            "fl_batch_destroy", "fl_gnn_destroy", "fl_amg_destroy", "fl_batch_size"}


def test_null_arguments_are_usage_errors():
    """Every entry point given null pointers and zero sizes returns the usage
    error status (1, where the reference aborts with FLAbort) and a message,
    before any device work: no GPU is needed and nothing crashes."""
    lib = _lib.load()
    for name in declared_symbols():
        res, args = _lib._SIGNATURES[name]
        vals = [0 if a in (ctypes.c_int32, ctypes.c_int, ctypes.c_int64)
                else 0.0 if a in (ctypes.c_double, ctypes.c_float) else None for a in args]
        st = getattr(lib, name)(*vals)
        if name in _NULL_OK:
            continue
        assert st == 1, (name, st)
        assert lib.fl_last_error(), name


def _fortran_interfaces():
    """bind(c, name=...) functions of the Fortran shim with their argument names."""
    path = os.path.join(os.path.dirname(HEADER), "..", "fluidity_gb300", "fortran", "fl_gpu_bindings.F90")
    src = open(path).read()
    src = re.sub(r"&\s*\n\s*&?", " ", src)  # join continuation lines
    out = {}
    for m in re.finditer(r"function\s+(\w+)\s*\(([^)]*)\)\s*bind\(c,\s*name=\"(\w+)\"\)", src):
        args = [a.strip() for a in m.group(2).split(",") if a.strip()]
        out[m.group(3)] = (m.group(1), args)
    return out


def _header_arg_counts():
    txt = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    out = {}
    for m in re.finditer(r"\b(fl_[A-Za-z0-9_]+)\s*\(([^;{]*?)\)\s*;", txt):
        args = " ".join(m.group(2).split())
        out[m.group(1)] = 0 if args in ("", "void") else args.count(",") + 1
    return out


def test_fortran_shim_binds_every_export_with_its_arity():
    """Every bind(c) interface of the Fortran shim names a header export, has
    the header's argument count and keeps the C name as its Fortran name;
    every header export has an interface (no Fortran compiler here: this is
    the shim's structural check)."""
    fi = _fortran_interfaces()
    hc = _header_arg_counts()
    assert sorted(fi) == sorted(hc), set(fi) ^ set(hc)
    for name, (fname, args) in fi.items():
        assert fname == name, name
        assert len(args) == hc[name], (name, args, hc[name])


def test_fortran_structs_match_the_ctypes_layouts():
    """The bind(c) derived types list the fields of the C structs in order."""
    path = os.path.join(os.path.dirname(HEADER), "..", "fluidity_gb300", "fortran", "fl_gpu_bindings.F90")
    src = open(path).read()
    structs = {"fl_advdif_params": _lib.AdvDifParams, "fl_fields": _lib.Fields, "fl_face_bcs": _lib.FaceBcs,
               "fl_solver_opts": _lib.SolverOpts, "fl_solve_report": _lib.SolveReport,
               "fl_mesh_desc": _lib.MeshDesc, "fl_divergence_params": _lib.DivergenceParams}
    for fname, cstruct in structs.items():
        m = re.search(rf"type, bind\(c\) :: {fname}\n(.*?)end type {fname}", src, flags=re.S)
        assert m, fname
        names = []
        for line in m.group(1).splitlines():
            if "::" in line:
                decl = line.split("::", 1)[1]
                names += [re.sub(r"\(.*\)", "", v).strip() for v in decl.split(",")]
        assert names == [f[0] for f in cstruct._fields_], (fname, names)


def test_solver_options_schedule_field():
    """fl_solver_opts.schedule (the GMRES launch schedule) and the size limit
    of the automatic choice, as the header declares them."""
    from fluidity_gb300 import femtools as ft
    assert ft.solver_options(ksp="gmres").schedule == 0
    assert ft.solver_options(ksp="gmres", schedule="graph").schedule == 1
    assert ft.solver_options(ksp="gmres", schedule="persistent").schedule == 2
    with pytest.raises(KeyError):
        ft.solver_options(schedule="sometimes")
    src = open(HEADER).read()
    assert re.search(r"#define FL_PERSIST_MAX_ROWS \d+", src)
    assert [f[0] for f in _lib.SolverOpts._fields_][-1] == "schedule"
