"""The generated polynomial sources (symmetrix_gb300/csrc/poly_canon.h and
poly_canon_tables.h) are exactly what gen_poly.py writes: regenerating them from the
equivariant monomial sets reproduces the committed files byte for byte."""
import importlib.util
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "symmetrix_gb300", "csrc")


def test_generated_sources_are_current(tmp_path):
    spec = importlib.util.spec_from_file_location("gen_poly", os.path.join(CSRC, "gen_poly.py"))
    gen = importlib.util.module_from_spec(spec)
    keep, sys.dont_write_bytecode = sys.dont_write_bytecode, True  # no __pycache__ among the sources
    try:
        spec.loader.exec_module(gen)
    finally:
        sys.dont_write_bytecode = keep
    gen.main(out_dir=str(tmp_path))
    for name in ("poly_canon.h", "poly_canon_tables.h"):
        with open(os.path.join(CSRC, name)) as f, open(tmp_path / name) as g:
            assert f.read() == g.read(), name
