"""Generate poly_canon.h: straight-line CUDA for the symmetric-contraction polynomials.

The monomials of a MACE symmetric contraction (degree <= 3 in the 16 A-basis
components, l_max = 3) are fixed by the equivariance of each output component LM:
every species and channel uses the same monomial set, only the coefficients differ
(extract_mace_data.py:239-304 folds U tensors and weights into exactly these
coefficients).  This script writes those sets, in the order symmetrix_gb300.synth
emits them, as compile-time code: the A-basis values and the gradient live in
registers and each monomial costs one coalesced coefficient load plus a few FMAs.

    python symmetrix_gb300/csrc/gen_poly.py      # rewrites poly_canon.h next to it
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from symmetrix_gb300.synth.equivariant import equivariant_polynomial_basis  # noqa: E402

L_MAX = 2  # hidden irreps up to 0e + 1o + 2e: LM = 0..8 (an L_max = 1 model uses LM = 0..3)


def canonical(L, M):
    keys = []
    for d in (1, 2, 3):
        mono, U = equivariant_polynomial_basis(L, d, 3)
        for t, key in enumerate(mono):
            if (U[:, M, t] != 0.0).any():
                keys.append(tuple(key))
    return keys


def pack(m):
    idx = list(m) + [16] * (3 - len(m))
    return idx[0] | (idx[1] << 8) | (idx[2] << 16)


def term(m):
    return "*".join(f"x[{a}]" for a in m)


def value_fn(name, monos):
    # one sum: the layer-0 kernel evaluates several of these side by side (four partial
    # sums each measured slower there); the node tail's value_grad uses four
    out = [f"__device__ __forceinline__ float {name}(const float* x, const float* __restrict__ cf, int C) {{",
           "  float f = 0.0f;"]
    for t, m in enumerate(monos):
        out.append(f"  f = fmaf(__ldg(cf + {t} * C), {term(m)}, f);")
    out += ["  return f;", "}"]
    return "\n".join(out)


def grad_lines(monos, scaled):
    out = []
    for t, m in enumerate(monos):
        q = f"w * __ldg(cf + {t} * C)" if scaled else f"__ldg(cf + {t} * C)"
        out.append(f"  {{ const float q = {q};")
        if len(m) == 1:
            out.append(f"    g[{m[0]}] += q;")
        else:
            for i, a in enumerate(m):
                rest = [b for j, b in enumerate(m) if j != i]
                out.append(f"    g[{a}] = fmaf(q, {term(rest)}, g[{a}]);")
        out.append("  }")
    return out


def grad_fn(name, monos):
    out = [f"__device__ __forceinline__ void {name}(const float* x, float w, const float* __restrict__ cf, int C, "
           f"float* g) {{"]
    out += grad_lines(monos, True)
    out.append("}")
    return "\n".join(out)


def value_grad_fn(name, monos):
    out = [f"__device__ __forceinline__ float {name}(const float* x, const float* __restrict__ cf, int C, "
           f"float* g) {{", "  float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f, f3 = 0.0f;"]
    for t, m in enumerate(monos):
        out.append(f"  {{ const float q = __ldg(cf + {t} * C);")
        out.append(f"    f{t % 4} = fmaf(q, {term(m)}, f{t % 4});")
        if len(m) == 1:
            out.append(f"    g[{m[0]}] += q;")
        else:
            for i, a in enumerate(m):
                rest = [b for j, b in enumerate(m) if j != i]
                out.append(f"    g[{a}] = fmaf(q, {term(rest)}, g[{a}]);")
        out.append("  }")
    out += ["  return (f0 + f1) + (f2 + f3);", "}"]
    return "\n".join(out)


def main(out_dir=HERE):
    lists = []
    for L in range(L_MAX + 1):
        for M in range(2 * L + 1):
            lists.append(canonical(L, M))
    nLM = len(lists)
    flat = [pack(m) for lst in lists for m in lst]
    offs = [0]
    for lst in lists:
        offs.append(offs[-1] + len(lst))
    t = ["// Generated by gen_poly.py: canonical symmetric-contraction monomial tables (l_max 3,",
         "// degree <= 3), shared by host and device code.  Do not edit; rerun the script.",
         "#pragma once", "", "namespace smx {", "namespace poly {", "",
         f"constexpr int kNumLM = {nLM};  // LM = 0 .. (L_max + 1)^2 - 1 for L_max up to {L_MAX}",
         f"constexpr int kOffset[{nLM + 1}] = {{{', '.join(map(str, offs))}}};",
         "// packed a | b << 8 | c << 16, 16 = constant one; LM-major, canonical order",
         f"constexpr int kMono[{len(flat)}] = {{{', '.join(map(str, flat))}}};", "",
         "}  // namespace poly", "}  // namespace smx", ""]
    with open(os.path.join(out_dir, "poly_canon_tables.h"), "w") as f:
        f.write("\n".join(t))
    h = ["// Generated by gen_poly.py: canonical symmetric-contraction monomials (l_max 3,",
         "// degree <= 3) as straight-line code.  Do not edit; rerun the script.",
         "#pragma once", "", '#include "poly_canon_tables.h"', "", "namespace smx {", "namespace poly {", ""]
    for LM, lst in enumerate(lists):
        h.append(value_fn(f"value_LM{LM}", lst))
        h.append("")
        h.append(grad_fn(f"grad_LM{LM}", lst))
        h.append("")
    h.append("// the layer-1 contraction is the LM = 0 set")
    h.append(value_grad_fn("value_grad_M1", lists[0]))
    h += ["", "}  // namespace poly", "}  // namespace smx", ""]
    path = os.path.join(out_dir, "poly_canon.h")
    with open(path, "w") as f:
        f.write("\n".join(h))
    print(f"wrote {path}: {[len(x) for x in lists]} monomials")


if __name__ == "__main__":
    main()
