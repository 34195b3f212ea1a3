"""The C ABI library loads and exports every symbol include/synk.h declares
(CPU only: no compute call is made)."""
import ctypes
import os
import re

from synkrotomo_gb300 import _lib
from synkrotomo_gb300 import build as B

HEADER_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_symbols():
    names = set()
    for fn in os.listdir(HEADER_DIR):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(HEADER_DIR, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[\w\s\*]+?\b(synk_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_entry_points():
    names = declared_symbols()
    for n in ["synk_context_new", "synk_forwardprojection", "synk_backprojection", "synk_SIRT", "synk_SIRT3D",
              "synk_forwardprojection_sparse", "synk_backprojection_sparse", "synk_sirt_slices"]:
        assert n in names


def test_library_exports_every_declared_symbol():
    path = B.build()
    lib = ctypes.CDLL(path)
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    assert declared_symbols() <= set(_lib.SIGNATURES)


def test_version_string_without_gpu():
    lib = ctypes.CDLL(B.build())
    lib.synk_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.synk_version()
