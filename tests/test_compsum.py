"""The compensated float64 sum of the GPU energy and virial reductions
(symmetrix_gb300/csrc/compsum.h), compiled for the host with g++: on sequences whose
plain float64 sum loses every significant digit it returns the exact sum (checked
against rational arithmetic), and on random data it is at least as close as the
plain sum."""
import os
import subprocess
from fractions import Fraction

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "symmetrix_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include "compsum.h"
int main() {
  smx::CompSum cs;
  double plain = 0.0, x;
  while (std::scanf("%lf", &x) == 1) { cs.add(x); plain += x; }
  std::printf("%.17g %.17g\n", cs.value(), plain);
  return 0;
}
"""


@pytest.fixture(scope="module")
def summer(tmp_path_factory):
    d = tmp_path_factory.mktemp("compsum")
    src, exe = d / "t.cpp", d / "t"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", SRC, str(src), "-o", str(exe)], check=True)

    def run(values):
        text = "\n".join(repr(float(v)) for v in values)
        out = subprocess.run([str(exe)], input=text, capture_output=True, text=True, check=True).stdout.split()
        return float(out[0]), float(out[1])
    return run


def exact(values):
    return float(sum(Fraction(float(v)) for v in values))


def test_cancellation_is_exact(summer):
    vals = [1e16, 1.0, -1e16] * 50 + [3.0, 1e-3, -3.0]
    comp, plain = summer(vals)
    assert comp == exact(vals) == 50.001
    assert plain != comp  # the plain sum loses the ones


def test_random_terms_no_worse_than_plain(summer):
    rng = np.random.default_rng(5)
    vals = rng.normal(size=5000) * 10.0 ** rng.integers(-6, 7, size=5000)
    comp, plain = summer(vals)
    ref = exact(vals)
    assert abs(comp - ref) <= abs(plain - ref)
    assert abs(comp - ref) <= 2 * np.spacing(abs(ref))
