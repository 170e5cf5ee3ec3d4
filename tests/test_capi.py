"""The C-ABI library builds for sm_103a, loads, and exports every symbol the
public header declares (no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re
import subprocess

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
