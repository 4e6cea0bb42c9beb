"""The C-ABI library builds for sm_103a, loads without a GPU, and exports every
entry point include/*.h declares (no compute calls here)."""
import ctypes
import glob
import os
import re

from symmetrix_gb300 import _lib
from symmetrix_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names.update(re.findall(r"\b(smx_\w+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    path = build()
    lib = ctypes.CDLL(path)
    names = declared_functions()
    assert "smx_compute_node_energies_forces" in names
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_binding_covers_the_header():
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_functions()) <= bound


def declared_arity():
    """Parameter count of every smx_* declaration in include/*.h."""
    out = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for name, params in re.findall(r"\b(smx_\w+)\s*\(([^)]*)\)\s*;", text):
            params = params.strip()
            out[name] = 0 if params in ("", "void") else len(params.split(","))
    return out


def test_binding_argument_counts_match_the_header():
    arity = declared_arity()
    assert len(arity) == len(declared_functions())
    wrong = {n: (len(a), arity[n]) for n, _, a in _lib.SIGNATURES if n in arity and len(a) != arity[n]}
    assert not wrong, wrong
