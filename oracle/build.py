"""Build recipe for the oracle (test infrastructure only).

* `build_oracle()` compiles the float64 restatement oracle/mace_oracle.cpp into
  oracle/_build/liborc.so.  It builds anywhere g++ is present.
* `build_reference()` compiles the reference's own evaluator, unchanged, from the
  sources where they lie in the reference tree (libsymmetrix/source/*.cpp under
  $SMX_REFERENCE_ROOT, default the container's reference checkout) with the
  stand-in headers under oracle/shim, plus oracle/ref_capi.cpp, into
  oracle/_ref/libsmx_ref.so.  It is skipped when the reference tree is absent.

No -march=native (the binaries must also build on Arm hosts) and no -ffast-math
(the reference's own CMake adds it; the oracle must be plain IEEE float64).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference tree (read-only); SMX_REFERENCE_ROOT points elsewhere when it lives elsewhere
REF_ROOT = os.environ.get("SMX_REFERENCE_ROOT", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "libsymmetrix", "source")
REF_FILES = ["mace.cpp", "cubic_spline.cpp", "cubic_spline_set.cpp", "multivariate_polynomial.cpp",
             "multilayer_perceptron.cpp", "zbl.cpp", "tools.cpp", "spherical_harmonic.cpp"]

ORACLE_SO = os.path.join(HERE, "_build", "liborc.so")
REF_SO = os.path.join(HERE, "_ref", "libsmx_ref.so")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build_oracle(force=False):
    src = os.path.join(HERE, "mace_oracle.cpp")
    hdr = os.path.join(HERE, "shim", "include", "nlohmann", "json.hpp")
    if force or _stale(ORACLE_SO, [src, hdr]):
        os.makedirs(os.path.dirname(ORACLE_SO), exist_ok=True)
        _run(["g++", "-std=c++20", "-O3", "-fPIC", "-shared", "-pthread", "-I",
              os.path.join(HERE, "shim", "include"), src, "-o", ORACLE_SO])
    return ORACLE_SO


def build_reference(force=False):
    if not os.path.isdir(REF_SRC):
        return None
    srcs = [os.path.join(REF_SRC, f) for f in REF_FILES]
    ours = [os.path.join(HERE, "ref_capi.cpp"), os.path.join(HERE, "shim", "cblas_shim.c")]
    hdrs = [os.path.join(HERE, "shim", "include", "nlohmann", "json.hpp"),
            os.path.join(HERE, "shim", "include", "sphericart.hpp")]
    if not (force or _stale(REF_SO, srcs + ours + hdrs)):
        return REF_SO
    obj_dir = os.path.join(HERE, "_ref", "obj")
    os.makedirs(obj_dir, exist_ok=True)
    inc = ["-I", os.path.join(HERE, "shim", "include"), "-I", os.path.join(HERE, "shim"), "-I", REF_SRC]
    objs, procs = [], []
    for s in srcs + ours:
        o = os.path.join(obj_dir, os.path.basename(s) + ".o")
        objs.append(o)
        if s.endswith(".c"):
            cmd = ["gcc", "-O2", "-fPIC", "-c", s, "-o", o] + inc
        else:
            cmd = ["g++", "-std=c++20", "-O2", "-fPIC", "-c", s, "-o", o] + inc
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)))
    for cmd, p in procs:
        out, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("reference build failed:\n" + " ".join(cmd) + "\n" + out + err)
    _run(["g++", "-shared", "-o", REF_SO] + objs)
    return REF_SO


if __name__ == "__main__":
    print(build_oracle(force="--force" in sys.argv))
    print(build_reference(force="--force" in sys.argv))
