"""The C ABI library loads and exports every function include/*.h declares
(no compute call: this runs without a GPU)."""
import ctypes
import glob
import os
import re

from snapy_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(sg_\w+)\s*\(",
                             text, flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_the_api():
    names = declared()
    assert {"sg_create", "sg_stage", "sg_max_dt", "sg_destroy"} <= names


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    for n in sorted(declared()):
        assert hasattr(L, n), n
    assert set(declared()) <= set(_lib.SIGNATURES), \
        set(declared()) - set(_lib.SIGNATURES)
    assert L.sg_version().decode().startswith("snapy_gb300")


def test_errors_are_reported_without_a_gpu():
    L = _lib.load()
    h = ctypes.c_void_p()
    rc = L.sg_create(None, None, 0, ctypes.byref(h))
    assert rc == 1
    assert "null" in L.sg_last_error().decode()
