"""The C-ABI library loads and exports every symbol include/nla3d_gpu.h
declares (no compute calls: this runs without a GPU)."""
import ctypes
import os
import re

from nla3d_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(nla3d_\w+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 20
    for n in sorted(names):
        assert hasattr(lib, n), n
    assert names == set(_lib.EXPORTS)


def test_library_is_the_in_tree_build():
    assert os.path.dirname(_lib.LIB_PATH) == os.path.join(ROOT, "nla3d_gb300")
    assert os.path.exists(_lib.LIB_PATH)
    ctypes.CDLL(_lib.LIB_PATH)
