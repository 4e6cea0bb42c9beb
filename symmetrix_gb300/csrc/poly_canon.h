// Generated by gen_poly.py: canonical symmetric-contraction monomials (l_max 3,
// degree <= 3) as straight-line code.  Do not edit; rerun the script.
#pragma once

#include "poly_canon_tables.h"

namespace smx {
namespace poly {

__device__ __forceinline__ float value_LM0(const float* x, const float* __restrict__ cf, int C) {
  float f = 0.0f;
  f = fmaf(__ldg(cf + 0 * C), x[0], f);
  f = fmaf(__ldg(cf + 1 * C), x[0]*x[0], f);
  f = fmaf(__ldg(cf + 2 * C), x[1]*x[1], f);
  f = fmaf(__ldg(cf + 3 * C), x[2]*x[2], f);
  f = fmaf(__ldg(cf + 4 * C), x[3]*x[3], f);
  f = fmaf(__ldg(cf + 5 * C), x[4]*x[4], f);
  f = fmaf(__ldg(cf + 6 * C), x[5]*x[5], f);
  f = fmaf(__ldg(cf + 7 * C), x[6]*x[6], f);
  f = fmaf(__ldg(cf + 8 * C), x[7]*x[7], f);
  f = fmaf(__ldg(cf + 9 * C), x[8]*x[8], f);
  f = fmaf(__ldg(cf + 10 * C), x[9]*x[9], f);
  f = fmaf(__ldg(cf + 11 * C), x[10]*x[10], f);
  f = fmaf(__ldg(cf + 12 * C), x[11]*x[11], f);
  f = fmaf(__ldg(cf + 13 * C), x[12]*x[12], f);
  f = fmaf(__ldg(cf + 14 * C), x[13]*x[13], f);
  f = fmaf(__ldg(cf + 15 * C), x[14]*x[14], f);
  f = fmaf(__ldg(cf + 16 * C), x[15]*x[15], f);
  f = fmaf(__ldg(cf + 17 * C), x[0]*x[0]*x[0], f);
  f = fmaf(__ldg(cf + 18 * C), x[0]*x[1]*x[1], f);
  f = fmaf(__ldg(cf + 19 * C), x[0]*x[2]*x[2], f);
  f = fmaf(__ldg(cf + 20 * C), x[0]*x[3]*x[3], f);
  f = fmaf(__ldg(cf + 21 * C), x[0]*x[4]*x[4], f);
  f = fmaf(__ldg(cf + 22 * C), x[0]*x[5]*x[5], f);
  f = fmaf(__ldg(cf + 23 * C), x[0]*x[6]*x[6], f);
  f = fmaf(__ldg(cf + 24 * C), x[0]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 25 * C), x[0]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 26 * C), x[0]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 27 * C), x[0]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 28 * C), x[0]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 29 * C), x[0]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 30 * C), x[0]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 31 * C), x[0]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 32 * C), x[0]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 33 * C), x[1]*x[1]*x[6], f);
  f = fmaf(__ldg(cf + 34 * C), x[1]*x[1]*x[8], f);
  f = fmaf(__ldg(cf + 35 * C), x[1]*x[2]*x[5], f);
  f = fmaf(__ldg(cf + 36 * C), x[1]*x[3]*x[4], f);
  f = fmaf(__ldg(cf + 37 * C), x[1]*x[4]*x[13], f);
  f = fmaf(__ldg(cf + 38 * C), x[1]*x[4]*x[15], f);
  f = fmaf(__ldg(cf + 39 * C), x[1]*x[5]*x[12], f);
  f = fmaf(__ldg(cf + 40 * C), x[1]*x[5]*x[14], f);
  f = fmaf(__ldg(cf + 41 * C), x[1]*x[6]*x[11], f);
  f = fmaf(__ldg(cf + 42 * C), x[1]*x[7]*x[10], f);
  f = fmaf(__ldg(cf + 43 * C), x[1]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 44 * C), x[1]*x[8]*x[11], f);
  f = fmaf(__ldg(cf + 45 * C), x[2]*x[2]*x[6], f);
  f = fmaf(__ldg(cf + 46 * C), x[2]*x[3]*x[7], f);
  f = fmaf(__ldg(cf + 47 * C), x[2]*x[4]*x[10], f);
  f = fmaf(__ldg(cf + 48 * C), x[2]*x[5]*x[11], f);
  f = fmaf(__ldg(cf + 49 * C), x[2]*x[6]*x[12], f);
  f = fmaf(__ldg(cf + 50 * C), x[2]*x[7]*x[13], f);
  f = fmaf(__ldg(cf + 51 * C), x[2]*x[8]*x[14], f);
  f = fmaf(__ldg(cf + 52 * C), x[3]*x[3]*x[6], f);
  f = fmaf(__ldg(cf + 53 * C), x[3]*x[3]*x[8], f);
  f = fmaf(__ldg(cf + 54 * C), x[3]*x[4]*x[9], f);
  f = fmaf(__ldg(cf + 55 * C), x[3]*x[4]*x[11], f);
  f = fmaf(__ldg(cf + 56 * C), x[3]*x[5]*x[10], f);
  f = fmaf(__ldg(cf + 57 * C), x[3]*x[6]*x[13], f);
  f = fmaf(__ldg(cf + 58 * C), x[3]*x[7]*x[12], f);
  f = fmaf(__ldg(cf + 59 * C), x[3]*x[7]*x[14], f);
  f = fmaf(__ldg(cf + 60 * C), x[3]*x[8]*x[13], f);
  f = fmaf(__ldg(cf + 61 * C), x[3]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 62 * C), x[4]*x[4]*x[6], f);
  f = fmaf(__ldg(cf + 63 * C), x[4]*x[5]*x[7], f);
  f = fmaf(__ldg(cf + 64 * C), x[4]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 65 * C), x[4]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 66 * C), x[4]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 67 * C), x[4]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 68 * C), x[5]*x[5]*x[6], f);
  f = fmaf(__ldg(cf + 69 * C), x[5]*x[5]*x[8], f);
  f = fmaf(__ldg(cf + 70 * C), x[5]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 71 * C), x[5]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 72 * C), x[5]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 73 * C), x[5]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 74 * C), x[5]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 75 * C), x[6]*x[6]*x[6], f);
  f = fmaf(__ldg(cf + 76 * C), x[6]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 77 * C), x[6]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 78 * C), x[6]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 79 * C), x[6]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 80 * C), x[6]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 81 * C), x[6]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 82 * C), x[6]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 83 * C), x[7]*x[7]*x[8], f);
  f = fmaf(__ldg(cf + 84 * C), x[7]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 85 * C), x[7]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 86 * C), x[7]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 87 * C), x[7]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 88 * C), x[7]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 89 * C), x[8]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 90 * C), x[8]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 91 * C), x[8]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 92 * C), x[8]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 93 * C), x[8]*x[13]*x[15], f);
  return f;
}

__device__ __forceinline__ void grad_LM0(const float* x, float w, const float* __restrict__ cf, int C, float* g) {
  { const float q = w * __ldg(cf + 0 * C);
    g[0] += q;
  }
  { const float q = w * __ldg(cf + 1 * C);
    g[0] = fmaf(q, x[0], g[0]);
    g[0] = fmaf(q, x[0], g[0]);
  }
  { const float q = w * __ldg(cf + 2 * C);
    g[1] = fmaf(q, x[1], g[1]);
    g[1] = fmaf(q, x[1], g[1]);
  }
  { const float q = w * __ldg(cf + 3 * C);
    g[2] = fmaf(q, x[2], g[2]);
    g[2] = fmaf(q, x[2], g[2]);
  }
  { const float q = w * __ldg(cf + 4 * C);
    g[3] = fmaf(q, x[3], g[3]);
    g[3] = fmaf(q, x[3], g[3]);
  }
  { const float q = w * __ldg(cf + 5 * C);
    g[4] = fmaf(q, x[4], g[4]);
    g[4] = fmaf(q, x[4], g[4]);
  }
  { const float q = w * __ldg(cf + 6 * C);
    g[5] = fmaf(q, x[5], g[5]);
    g[5] = fmaf(q, x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 7 * C);
    g[6] = fmaf(q, x[6], g[6]);
    g[6] = fmaf(q, x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 8 * C);
    g[7] = fmaf(q, x[7], g[7]);
    g[7] = fmaf(q, x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 9 * C);
    g[8] = fmaf(q, x[8], g[8]);
    g[8] = fmaf(q, x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 10 * C);
    g[9] = fmaf(q, x[9], g[9]);
    g[9] = fmaf(q, x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 11 * C);
    g[10] = fmaf(q, x[10], g[10]);
    g[10] = fmaf(q, x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 12 * C);
    g[11] = fmaf(q, x[11], g[11]);
    g[11] = fmaf(q, x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 13 * C);
    g[12] = fmaf(q, x[12], g[12]);
    g[12] = fmaf(q, x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 14 * C);
    g[13] = fmaf(q, x[13], g[13]);
    g[13] = fmaf(q, x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 15 * C);
    g[14] = fmaf(q, x[14], g[14]);
    g[14] = fmaf(q, x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 16 * C);
    g[15] = fmaf(q, x[15], g[15]);
    g[15] = fmaf(q, x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 17 * C);
    g[0] = fmaf(q, x[0]*x[0], g[0]);
    g[0] = fmaf(q, x[0]*x[0], g[0]);
    g[0] = fmaf(q, x[0]*x[0], g[0]);
  }
  { const float q = w * __ldg(cf + 18 * C);
    g[0] = fmaf(q, x[1]*x[1], g[0]);
    g[1] = fmaf(q, x[0]*x[1], g[1]);
    g[1] = fmaf(q, x[0]*x[1], g[1]);
  }
  { const float q = w * __ldg(cf + 19 * C);
    g[0] = fmaf(q, x[2]*x[2], g[0]);
    g[2] = fmaf(q, x[0]*x[2], g[2]);
    g[2] = fmaf(q, x[0]*x[2], g[2]);
  }
  { const float q = w * __ldg(cf + 20 * C);
    g[0] = fmaf(q, x[3]*x[3], g[0]);
    g[3] = fmaf(q, x[0]*x[3], g[3]);
    g[3] = fmaf(q, x[0]*x[3], g[3]);
  }
  { const float q = w * __ldg(cf + 21 * C);
    g[0] = fmaf(q, x[4]*x[4], g[0]);
    g[4] = fmaf(q, x[0]*x[4], g[4]);
    g[4] = fmaf(q, x[0]*x[4], g[4]);
  }
  { const float q = w * __ldg(cf + 22 * C);
    g[0] = fmaf(q, x[5]*x[5], g[0]);
    g[5] = fmaf(q, x[0]*x[5], g[5]);
    g[5] = fmaf(q, x[0]*x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 23 * C);
    g[0] = fmaf(q, x[6]*x[6], g[0]);
    g[6] = fmaf(q, x[0]*x[6], g[6]);
    g[6] = fmaf(q, x[0]*x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 24 * C);
    g[0] = fmaf(q, x[7]*x[7], g[0]);
    g[7] = fmaf(q, x[0]*x[7], g[7]);
    g[7] = fmaf(q, x[0]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 25 * C);
    g[0] = fmaf(q, x[8]*x[8], g[0]);
    g[8] = fmaf(q, x[0]*x[8], g[8]);
    g[8] = fmaf(q, x[0]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 26 * C);
    g[0] = fmaf(q, x[9]*x[9], g[0]);
    g[9] = fmaf(q, x[0]*x[9], g[9]);
    g[9] = fmaf(q, x[0]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 27 * C);
    g[0] = fmaf(q, x[10]*x[10], g[0]);
    g[10] = fmaf(q, x[0]*x[10], g[10]);
    g[10] = fmaf(q, x[0]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 28 * C);
    g[0] = fmaf(q, x[11]*x[11], g[0]);
    g[11] = fmaf(q, x[0]*x[11], g[11]);
    g[11] = fmaf(q, x[0]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 29 * C);
    g[0] = fmaf(q, x[12]*x[12], g[0]);
    g[12] = fmaf(q, x[0]*x[12], g[12]);
    g[12] = fmaf(q, x[0]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 30 * C);
    g[0] = fmaf(q, x[13]*x[13], g[0]);
    g[13] = fmaf(q, x[0]*x[13], g[13]);
    g[13] = fmaf(q, x[0]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 31 * C);
    g[0] = fmaf(q, x[14]*x[14], g[0]);
    g[14] = fmaf(q, x[0]*x[14], g[14]);
    g[14] = fmaf(q, x[0]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 32 * C);
    g[0] = fmaf(q, x[15]*x[15], g[0]);
    g[15] = fmaf(q, x[0]*x[15], g[15]);
    g[15] = fmaf(q, x[0]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 33 * C);
    g[1] = fmaf(q, x[1]*x[6], g[1]);
    g[1] = fmaf(q, x[1]*x[6], g[1]);
    g[6] = fmaf(q, x[1]*x[1], g[6]);
  }
  { const float q = w * __ldg(cf + 34 * C);
    g[1] = fmaf(q, x[1]*x[8], g[1]);
    g[1] = fmaf(q, x[1]*x[8], g[1]);
    g[8] = fmaf(q, x[1]*x[1], g[8]);
  }
  { const float q = w * __ldg(cf + 35 * C);
    g[1] = fmaf(q, x[2]*x[5], g[1]);
    g[2] = fmaf(q, x[1]*x[5], g[2]);
    g[5] = fmaf(q, x[1]*x[2], g[5]);
  }
  { const float q = w * __ldg(cf + 36 * C);
    g[1] = fmaf(q, x[3]*x[4], g[1]);
    g[3] = fmaf(q, x[1]*x[4], g[3]);
    g[4] = fmaf(q, x[1]*x[3], g[4]);
  }
  { const float q = w * __ldg(cf + 37 * C);
    g[1] = fmaf(q, x[4]*x[13], g[1]);
    g[4] = fmaf(q, x[1]*x[13], g[4]);
    g[13] = fmaf(q, x[1]*x[4], g[13]);
  }
  { const float q = w * __ldg(cf + 38 * C);
    g[1] = fmaf(q, x[4]*x[15], g[1]);
    g[4] = fmaf(q, x[1]*x[15], g[4]);
    g[15] = fmaf(q, x[1]*x[4], g[15]);
  }
  { const float q = w * __ldg(cf + 39 * C);
    g[1] = fmaf(q, x[5]*x[12], g[1]);
    g[5] = fmaf(q, x[1]*x[12], g[5]);
    g[12] = fmaf(q, x[1]*x[5], g[12]);
  }
  { const float q = w * __ldg(cf + 40 * C);
    g[1] = fmaf(q, x[5]*x[14], g[1]);
    g[5] = fmaf(q, x[1]*x[14], g[5]);
    g[14] = fmaf(q, x[1]*x[5], g[14]);
  }
  { const float q = w * __ldg(cf + 41 * C);
    g[1] = fmaf(q, x[6]*x[11], g[1]);
    g[6] = fmaf(q, x[1]*x[11], g[6]);
    g[11] = fmaf(q, x[1]*x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 42 * C);
    g[1] = fmaf(q, x[7]*x[10], g[1]);
    g[7] = fmaf(q, x[1]*x[10], g[7]);
    g[10] = fmaf(q, x[1]*x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 43 * C);
    g[1] = fmaf(q, x[8]*x[9], g[1]);
    g[8] = fmaf(q, x[1]*x[9], g[8]);
    g[9] = fmaf(q, x[1]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 44 * C);
    g[1] = fmaf(q, x[8]*x[11], g[1]);
    g[8] = fmaf(q, x[1]*x[11], g[8]);
    g[11] = fmaf(q, x[1]*x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 45 * C);
    g[2] = fmaf(q, x[2]*x[6], g[2]);
    g[2] = fmaf(q, x[2]*x[6], g[2]);
    g[6] = fmaf(q, x[2]*x[2], g[6]);
  }
  { const float q = w * __ldg(cf + 46 * C);
    g[2] = fmaf(q, x[3]*x[7], g[2]);
    g[3] = fmaf(q, x[2]*x[7], g[3]);
    g[7] = fmaf(q, x[2]*x[3], g[7]);
  }
  { const float q = w * __ldg(cf + 47 * C);
    g[2] = fmaf(q, x[4]*x[10], g[2]);
    g[4] = fmaf(q, x[2]*x[10], g[4]);
    g[10] = fmaf(q, x[2]*x[4], g[10]);
  }
  { const float q = w * __ldg(cf + 48 * C);
    g[2] = fmaf(q, x[5]*x[11], g[2]);
    g[5] = fmaf(q, x[2]*x[11], g[5]);
    g[11] = fmaf(q, x[2]*x[5], g[11]);
  }
  { const float q = w * __ldg(cf + 49 * C);
    g[2] = fmaf(q, x[6]*x[12], g[2]);
    g[6] = fmaf(q, x[2]*x[12], g[6]);
    g[12] = fmaf(q, x[2]*x[6], g[12]);
  }
  { const float q = w * __ldg(cf + 50 * C);
    g[2] = fmaf(q, x[7]*x[13], g[2]);
    g[7] = fmaf(q, x[2]*x[13], g[7]);
    g[13] = fmaf(q, x[2]*x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 51 * C);
    g[2] = fmaf(q, x[8]*x[14], g[2]);
    g[8] = fmaf(q, x[2]*x[14], g[8]);
    g[14] = fmaf(q, x[2]*x[8], g[14]);
  }
  { const float q = w * __ldg(cf + 52 * C);
    g[3] = fmaf(q, x[3]*x[6], g[3]);
    g[3] = fmaf(q, x[3]*x[6], g[3]);
    g[6] = fmaf(q, x[3]*x[3], g[6]);
  }
  { const float q = w * __ldg(cf + 53 * C);
    g[3] = fmaf(q, x[3]*x[8], g[3]);
    g[3] = fmaf(q, x[3]*x[8], g[3]);
    g[8] = fmaf(q, x[3]*x[3], g[8]);
  }
  { const float q = w * __ldg(cf + 54 * C);
    g[3] = fmaf(q, x[4]*x[9], g[3]);
    g[4] = fmaf(q, x[3]*x[9], g[4]);
    g[9] = fmaf(q, x[3]*x[4], g[9]);
  }
  { const float q = w * __ldg(cf + 55 * C);
    g[3] = fmaf(q, x[4]*x[11], g[3]);
    g[4] = fmaf(q, x[3]*x[11], g[4]);
    g[11] = fmaf(q, x[3]*x[4], g[11]);
  }
  { const float q = w * __ldg(cf + 56 * C);
    g[3] = fmaf(q, x[5]*x[10], g[3]);
    g[5] = fmaf(q, x[3]*x[10], g[5]);
    g[10] = fmaf(q, x[3]*x[5], g[10]);
  }
  { const float q = w * __ldg(cf + 57 * C);
    g[3] = fmaf(q, x[6]*x[13], g[3]);
    g[6] = fmaf(q, x[3]*x[13], g[6]);
    g[13] = fmaf(q, x[3]*x[6], g[13]);
  }
  { const float q = w * __ldg(cf + 58 * C);
    g[3] = fmaf(q, x[7]*x[12], g[3]);
    g[7] = fmaf(q, x[3]*x[12], g[7]);
    g[12] = fmaf(q, x[3]*x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 59 * C);
    g[3] = fmaf(q, x[7]*x[14], g[3]);
    g[7] = fmaf(q, x[3]*x[14], g[7]);
    g[14] = fmaf(q, x[3]*x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 60 * C);
    g[3] = fmaf(q, x[8]*x[13], g[3]);
    g[8] = fmaf(q, x[3]*x[13], g[8]);
    g[13] = fmaf(q, x[3]*x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 61 * C);
    g[3] = fmaf(q, x[8]*x[15], g[3]);
    g[8] = fmaf(q, x[3]*x[15], g[8]);
    g[15] = fmaf(q, x[3]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 62 * C);
    g[4] = fmaf(q, x[4]*x[6], g[4]);
    g[4] = fmaf(q, x[4]*x[6], g[4]);
    g[6] = fmaf(q, x[4]*x[4], g[6]);
  }
  { const float q = w * __ldg(cf + 63 * C);
    g[4] = fmaf(q, x[5]*x[7], g[4]);
    g[5] = fmaf(q, x[4]*x[7], g[5]);
    g[7] = fmaf(q, x[4]*x[5], g[7]);
  }
  { const float q = w * __ldg(cf + 64 * C);
    g[4] = fmaf(q, x[9]*x[13], g[4]);
    g[9] = fmaf(q, x[4]*x[13], g[9]);
    g[13] = fmaf(q, x[4]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 65 * C);
    g[4] = fmaf(q, x[10]*x[12], g[4]);
    g[10] = fmaf(q, x[4]*x[12], g[10]);
    g[12] = fmaf(q, x[4]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 66 * C);
    g[4] = fmaf(q, x[11]*x[13], g[4]);
    g[11] = fmaf(q, x[4]*x[13], g[11]);
    g[13] = fmaf(q, x[4]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 67 * C);
    g[4] = fmaf(q, x[11]*x[15], g[4]);
    g[11] = fmaf(q, x[4]*x[15], g[11]);
    g[15] = fmaf(q, x[4]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 68 * C);
    g[5] = fmaf(q, x[5]*x[6], g[5]);
    g[5] = fmaf(q, x[5]*x[6], g[5]);
    g[6] = fmaf(q, x[5]*x[5], g[6]);
  }
  { const float q = w * __ldg(cf + 69 * C);
    g[5] = fmaf(q, x[5]*x[8], g[5]);
    g[5] = fmaf(q, x[5]*x[8], g[5]);
    g[8] = fmaf(q, x[5]*x[5], g[8]);
  }
  { const float q = w * __ldg(cf + 70 * C);
    g[5] = fmaf(q, x[9]*x[14], g[5]);
    g[9] = fmaf(q, x[5]*x[14], g[9]);
    g[14] = fmaf(q, x[5]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 71 * C);
    g[5] = fmaf(q, x[10]*x[13], g[5]);
    g[10] = fmaf(q, x[5]*x[13], g[10]);
    g[13] = fmaf(q, x[5]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 72 * C);
    g[5] = fmaf(q, x[10]*x[15], g[5]);
    g[10] = fmaf(q, x[5]*x[15], g[10]);
    g[15] = fmaf(q, x[5]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 73 * C);
    g[5] = fmaf(q, x[11]*x[12], g[5]);
    g[11] = fmaf(q, x[5]*x[12], g[11]);
    g[12] = fmaf(q, x[5]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 74 * C);
    g[5] = fmaf(q, x[11]*x[14], g[5]);
    g[11] = fmaf(q, x[5]*x[14], g[11]);
    g[14] = fmaf(q, x[5]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 75 * C);
    g[6] = fmaf(q, x[6]*x[6], g[6]);
    g[6] = fmaf(q, x[6]*x[6], g[6]);
    g[6] = fmaf(q, x[6]*x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 76 * C);
    g[6] = fmaf(q, x[7]*x[7], g[6]);
    g[7] = fmaf(q, x[6]*x[7], g[7]);
    g[7] = fmaf(q, x[6]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 77 * C);
    g[6] = fmaf(q, x[8]*x[8], g[6]);
    g[8] = fmaf(q, x[6]*x[8], g[8]);
    g[8] = fmaf(q, x[6]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 78 * C);
    g[6] = fmaf(q, x[9]*x[9], g[6]);
    g[9] = fmaf(q, x[6]*x[9], g[9]);
    g[9] = fmaf(q, x[6]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 79 * C);
    g[6] = fmaf(q, x[11]*x[11], g[6]);
    g[11] = fmaf(q, x[6]*x[11], g[11]);
    g[11] = fmaf(q, x[6]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 80 * C);
    g[6] = fmaf(q, x[12]*x[12], g[6]);
    g[12] = fmaf(q, x[6]*x[12], g[12]);
    g[12] = fmaf(q, x[6]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 81 * C);
    g[6] = fmaf(q, x[13]*x[13], g[6]);
    g[13] = fmaf(q, x[6]*x[13], g[13]);
    g[13] = fmaf(q, x[6]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 82 * C);
    g[6] = fmaf(q, x[15]*x[15], g[6]);
    g[15] = fmaf(q, x[6]*x[15], g[15]);
    g[15] = fmaf(q, x[6]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 83 * C);
    g[7] = fmaf(q, x[7]*x[8], g[7]);
    g[7] = fmaf(q, x[7]*x[8], g[7]);
    g[8] = fmaf(q, x[7]*x[7], g[8]);
  }
  { const float q = w * __ldg(cf + 84 * C);
    g[7] = fmaf(q, x[9]*x[10], g[7]);
    g[9] = fmaf(q, x[7]*x[10], g[9]);
    g[10] = fmaf(q, x[7]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 85 * C);
    g[7] = fmaf(q, x[10]*x[11], g[7]);
    g[10] = fmaf(q, x[7]*x[11], g[10]);
    g[11] = fmaf(q, x[7]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 86 * C);
    g[7] = fmaf(q, x[12]*x[13], g[7]);
    g[12] = fmaf(q, x[7]*x[13], g[12]);
    g[13] = fmaf(q, x[7]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 87 * C);
    g[7] = fmaf(q, x[13]*x[14], g[7]);
    g[13] = fmaf(q, x[7]*x[14], g[13]);
    g[14] = fmaf(q, x[7]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 88 * C);
    g[7] = fmaf(q, x[14]*x[15], g[7]);
    g[14] = fmaf(q, x[7]*x[15], g[14]);
    g[15] = fmaf(q, x[7]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 89 * C);
    g[8] = fmaf(q, x[9]*x[11], g[8]);
    g[9] = fmaf(q, x[8]*x[11], g[9]);
    g[11] = fmaf(q, x[8]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 90 * C);
    g[8] = fmaf(q, x[11]*x[11], g[8]);
    g[11] = fmaf(q, x[8]*x[11], g[11]);
    g[11] = fmaf(q, x[8]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 91 * C);
    g[8] = fmaf(q, x[12]*x[14], g[8]);
    g[12] = fmaf(q, x[8]*x[14], g[12]);
    g[14] = fmaf(q, x[8]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 92 * C);
    g[8] = fmaf(q, x[13]*x[13], g[8]);
    g[13] = fmaf(q, x[8]*x[13], g[13]);
    g[13] = fmaf(q, x[8]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 93 * C);
    g[8] = fmaf(q, x[13]*x[15], g[8]);
    g[13] = fmaf(q, x[8]*x[15], g[13]);
    g[15] = fmaf(q, x[8]*x[13], g[15]);
  }
}

__device__ __forceinline__ float value_LM1(const float* x, const float* __restrict__ cf, int C) {
  float f = 0.0f;
  f = fmaf(__ldg(cf + 0 * C), x[1], f);
  f = fmaf(__ldg(cf + 1 * C), x[0]*x[1], f);
  f = fmaf(__ldg(cf + 2 * C), x[1]*x[6], f);
  f = fmaf(__ldg(cf + 3 * C), x[1]*x[8], f);
  f = fmaf(__ldg(cf + 4 * C), x[2]*x[5], f);
  f = fmaf(__ldg(cf + 5 * C), x[3]*x[4], f);
  f = fmaf(__ldg(cf + 6 * C), x[4]*x[13], f);
  f = fmaf(__ldg(cf + 7 * C), x[4]*x[15], f);
  f = fmaf(__ldg(cf + 8 * C), x[5]*x[12], f);
  f = fmaf(__ldg(cf + 9 * C), x[5]*x[14], f);
  f = fmaf(__ldg(cf + 10 * C), x[6]*x[11], f);
  f = fmaf(__ldg(cf + 11 * C), x[7]*x[10], f);
  f = fmaf(__ldg(cf + 12 * C), x[8]*x[9], f);
  f = fmaf(__ldg(cf + 13 * C), x[8]*x[11], f);
  f = fmaf(__ldg(cf + 14 * C), x[0]*x[0]*x[1], f);
  f = fmaf(__ldg(cf + 15 * C), x[0]*x[1]*x[6], f);
  f = fmaf(__ldg(cf + 16 * C), x[0]*x[1]*x[8], f);
  f = fmaf(__ldg(cf + 17 * C), x[0]*x[2]*x[5], f);
  f = fmaf(__ldg(cf + 18 * C), x[0]*x[3]*x[4], f);
  f = fmaf(__ldg(cf + 19 * C), x[0]*x[4]*x[13], f);
  f = fmaf(__ldg(cf + 20 * C), x[0]*x[4]*x[15], f);
  f = fmaf(__ldg(cf + 21 * C), x[0]*x[5]*x[12], f);
  f = fmaf(__ldg(cf + 22 * C), x[0]*x[5]*x[14], f);
  f = fmaf(__ldg(cf + 23 * C), x[0]*x[6]*x[11], f);
  f = fmaf(__ldg(cf + 24 * C), x[0]*x[7]*x[10], f);
  f = fmaf(__ldg(cf + 25 * C), x[0]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 26 * C), x[0]*x[8]*x[11], f);
  f = fmaf(__ldg(cf + 27 * C), x[1]*x[1]*x[1], f);
  f = fmaf(__ldg(cf + 28 * C), x[1]*x[1]*x[9], f);
  f = fmaf(__ldg(cf + 29 * C), x[1]*x[1]*x[11], f);
  f = fmaf(__ldg(cf + 30 * C), x[1]*x[2]*x[2], f);
  f = fmaf(__ldg(cf + 31 * C), x[1]*x[2]*x[12], f);
  f = fmaf(__ldg(cf + 32 * C), x[1]*x[2]*x[14], f);
  f = fmaf(__ldg(cf + 33 * C), x[1]*x[3]*x[3], f);
  f = fmaf(__ldg(cf + 34 * C), x[1]*x[3]*x[13], f);
  f = fmaf(__ldg(cf + 35 * C), x[1]*x[3]*x[15], f);
  f = fmaf(__ldg(cf + 36 * C), x[1]*x[4]*x[4], f);
  f = fmaf(__ldg(cf + 37 * C), x[1]*x[5]*x[5], f);
  f = fmaf(__ldg(cf + 38 * C), x[1]*x[6]*x[6], f);
  f = fmaf(__ldg(cf + 39 * C), x[1]*x[6]*x[8], f);
  f = fmaf(__ldg(cf + 40 * C), x[1]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 41 * C), x[1]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 42 * C), x[1]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 43 * C), x[1]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 44 * C), x[1]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 45 * C), x[1]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 46 * C), x[1]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 47 * C), x[1]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 48 * C), x[1]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 49 * C), x[1]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 50 * C), x[1]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 51 * C), x[1]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 52 * C), x[2]*x[2]*x[11], f);
  f = fmaf(__ldg(cf + 53 * C), x[2]*x[3]*x[10], f);
  f = fmaf(__ldg(cf + 54 * C), x[2]*x[4]*x[7], f);
  f = fmaf(__ldg(cf + 55 * C), x[2]*x[5]*x[6], f);
  f = fmaf(__ldg(cf + 56 * C), x[2]*x[5]*x[8], f);
  f = fmaf(__ldg(cf + 57 * C), x[2]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 58 * C), x[2]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 59 * C), x[2]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 60 * C), x[2]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 61 * C), x[2]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 62 * C), x[3]*x[3]*x[9], f);
  f = fmaf(__ldg(cf + 63 * C), x[3]*x[3]*x[11], f);
  f = fmaf(__ldg(cf + 64 * C), x[3]*x[4]*x[6], f);
  f = fmaf(__ldg(cf + 65 * C), x[3]*x[5]*x[7], f);
  f = fmaf(__ldg(cf + 66 * C), x[3]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 67 * C), x[3]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 68 * C), x[3]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 69 * C), x[3]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 70 * C), x[4]*x[4]*x[9], f);
  f = fmaf(__ldg(cf + 71 * C), x[4]*x[4]*x[11], f);
  f = fmaf(__ldg(cf + 72 * C), x[4]*x[5]*x[10], f);
  f = fmaf(__ldg(cf + 73 * C), x[4]*x[6]*x[13], f);
  f = fmaf(__ldg(cf + 74 * C), x[4]*x[6]*x[15], f);
  f = fmaf(__ldg(cf + 75 * C), x[4]*x[7]*x[12], f);
  f = fmaf(__ldg(cf + 76 * C), x[4]*x[7]*x[14], f);
  f = fmaf(__ldg(cf + 77 * C), x[4]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 78 * C), x[5]*x[5]*x[9], f);
  f = fmaf(__ldg(cf + 79 * C), x[5]*x[5]*x[11], f);
  f = fmaf(__ldg(cf + 80 * C), x[5]*x[6]*x[12], f);
  f = fmaf(__ldg(cf + 81 * C), x[5]*x[6]*x[14], f);
  f = fmaf(__ldg(cf + 82 * C), x[5]*x[7]*x[13], f);
  f = fmaf(__ldg(cf + 83 * C), x[5]*x[7]*x[15], f);
  f = fmaf(__ldg(cf + 84 * C), x[5]*x[8]*x[12], f);
  f = fmaf(__ldg(cf + 85 * C), x[5]*x[8]*x[14], f);
  f = fmaf(__ldg(cf + 86 * C), x[6]*x[6]*x[11], f);
  f = fmaf(__ldg(cf + 87 * C), x[6]*x[7]*x[10], f);
  f = fmaf(__ldg(cf + 88 * C), x[6]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 89 * C), x[6]*x[8]*x[11], f);
  f = fmaf(__ldg(cf + 90 * C), x[7]*x[7]*x[9], f);
  f = fmaf(__ldg(cf + 91 * C), x[7]*x[7]*x[11], f);
  f = fmaf(__ldg(cf + 92 * C), x[7]*x[8]*x[10], f);
  f = fmaf(__ldg(cf + 93 * C), x[8]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 94 * C), x[8]*x[8]*x[11], f);
  f = fmaf(__ldg(cf + 95 * C), x[9]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 96 * C), x[9]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 97 * C), x[9]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 98 * C), x[9]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 99 * C), x[9]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 100 * C), x[9]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 101 * C), x[10]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 102 * C), x[10]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 103 * C), x[10]*x[12]*x[15], f);
  f = fmaf(__ldg(cf + 104 * C), x[10]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 105 * C), x[11]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 106 * C), x[11]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 107 * C), x[11]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 108 * C), x[11]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 109 * C), x[11]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 110 * C), x[11]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 111 * C), x[11]*x[15]*x[15], f);
  return f;
}

__device__ __forceinline__ void grad_LM1(const float* x, float w, const float* __restrict__ cf, int C, float* g) {
  { const float q = w * __ldg(cf + 0 * C);
    g[1] += q;
  }
  { const float q = w * __ldg(cf + 1 * C);
    g[0] = fmaf(q, x[1], g[0]);
    g[1] = fmaf(q, x[0], g[1]);
  }
  { const float q = w * __ldg(cf + 2 * C);
    g[1] = fmaf(q, x[6], g[1]);
    g[6] = fmaf(q, x[1], g[6]);
  }
  { const float q = w * __ldg(cf + 3 * C);
    g[1] = fmaf(q, x[8], g[1]);
    g[8] = fmaf(q, x[1], g[8]);
  }
  { const float q = w * __ldg(cf + 4 * C);
    g[2] = fmaf(q, x[5], g[2]);
    g[5] = fmaf(q, x[2], g[5]);
  }
  { const float q = w * __ldg(cf + 5 * C);
    g[3] = fmaf(q, x[4], g[3]);
    g[4] = fmaf(q, x[3], g[4]);
  }
  { const float q = w * __ldg(cf + 6 * C);
    g[4] = fmaf(q, x[13], g[4]);
    g[13] = fmaf(q, x[4], g[13]);
  }
  { const float q = w * __ldg(cf + 7 * C);
    g[4] = fmaf(q, x[15], g[4]);
    g[15] = fmaf(q, x[4], g[15]);
  }
  { const float q = w * __ldg(cf + 8 * C);
    g[5] = fmaf(q, x[12], g[5]);
    g[12] = fmaf(q, x[5], g[12]);
  }
  { const float q = w * __ldg(cf + 9 * C);
    g[5] = fmaf(q, x[14], g[5]);
    g[14] = fmaf(q, x[5], g[14]);
  }
  { const float q = w * __ldg(cf + 10 * C);
    g[6] = fmaf(q, x[11], g[6]);
    g[11] = fmaf(q, x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 11 * C);
    g[7] = fmaf(q, x[10], g[7]);
    g[10] = fmaf(q, x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 12 * C);
    g[8] = fmaf(q, x[9], g[8]);
    g[9] = fmaf(q, x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 13 * C);
    g[8] = fmaf(q, x[11], g[8]);
    g[11] = fmaf(q, x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 14 * C);
    g[0] = fmaf(q, x[0]*x[1], g[0]);
    g[0] = fmaf(q, x[0]*x[1], g[0]);
    g[1] = fmaf(q, x[0]*x[0], g[1]);
  }
  { const float q = w * __ldg(cf + 15 * C);
    g[0] = fmaf(q, x[1]*x[6], g[0]);
    g[1] = fmaf(q, x[0]*x[6], g[1]);
    g[6] = fmaf(q, x[0]*x[1], g[6]);
  }
  { const float q = w * __ldg(cf + 16 * C);
    g[0] = fmaf(q, x[1]*x[8], g[0]);
    g[1] = fmaf(q, x[0]*x[8], g[1]);
    g[8] = fmaf(q, x[0]*x[1], g[8]);
  }
  { const float q = w * __ldg(cf + 17 * C);
    g[0] = fmaf(q, x[2]*x[5], g[0]);
    g[2] = fmaf(q, x[0]*x[5], g[2]);
    g[5] = fmaf(q, x[0]*x[2], g[5]);
  }
  { const float q = w * __ldg(cf + 18 * C);
    g[0] = fmaf(q, x[3]*x[4], g[0]);
    g[3] = fmaf(q, x[0]*x[4], g[3]);
    g[4] = fmaf(q, x[0]*x[3], g[4]);
  }
  { const float q = w * __ldg(cf + 19 * C);
    g[0] = fmaf(q, x[4]*x[13], g[0]);
    g[4] = fmaf(q, x[0]*x[13], g[4]);
    g[13] = fmaf(q, x[0]*x[4], g[13]);
  }
  { const float q = w * __ldg(cf + 20 * C);
    g[0] = fmaf(q, x[4]*x[15], g[0]);
    g[4] = fmaf(q, x[0]*x[15], g[4]);
    g[15] = fmaf(q, x[0]*x[4], g[15]);
  }
  { const float q = w * __ldg(cf + 21 * C);
    g[0] = fmaf(q, x[5]*x[12], g[0]);
    g[5] = fmaf(q, x[0]*x[12], g[5]);
    g[12] = fmaf(q, x[0]*x[5], g[12]);
  }
  { const float q = w * __ldg(cf + 22 * C);
    g[0] = fmaf(q, x[5]*x[14], g[0]);
    g[5] = fmaf(q, x[0]*x[14], g[5]);
    g[14] = fmaf(q, x[0]*x[5], g[14]);
  }
  { const float q = w * __ldg(cf + 23 * C);
    g[0] = fmaf(q, x[6]*x[11], g[0]);
    g[6] = fmaf(q, x[0]*x[11], g[6]);
    g[11] = fmaf(q, x[0]*x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 24 * C);
    g[0] = fmaf(q, x[7]*x[10], g[0]);
    g[7] = fmaf(q, x[0]*x[10], g[7]);
    g[10] = fmaf(q, x[0]*x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 25 * C);
    g[0] = fmaf(q, x[8]*x[9], g[0]);
    g[8] = fmaf(q, x[0]*x[9], g[8]);
    g[9] = fmaf(q, x[0]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 26 * C);
    g[0] = fmaf(q, x[8]*x[11], g[0]);
    g[8] = fmaf(q, x[0]*x[11], g[8]);
    g[11] = fmaf(q, x[0]*x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 27 * C);
    g[1] = fmaf(q, x[1]*x[1], g[1]);
    g[1] = fmaf(q, x[1]*x[1], g[1]);
    g[1] = fmaf(q, x[1]*x[1], g[1]);
  }
  { const float q = w * __ldg(cf + 28 * C);
    g[1] = fmaf(q, x[1]*x[9], g[1]);
    g[1] = fmaf(q, x[1]*x[9], g[1]);
    g[9] = fmaf(q, x[1]*x[1], g[9]);
  }
  { const float q = w * __ldg(cf + 29 * C);
    g[1] = fmaf(q, x[1]*x[11], g[1]);
    g[1] = fmaf(q, x[1]*x[11], g[1]);
    g[11] = fmaf(q, x[1]*x[1], g[11]);
  }
  { const float q = w * __ldg(cf + 30 * C);
    g[1] = fmaf(q, x[2]*x[2], g[1]);
    g[2] = fmaf(q, x[1]*x[2], g[2]);
    g[2] = fmaf(q, x[1]*x[2], g[2]);
  }
  { const float q = w * __ldg(cf + 31 * C);
    g[1] = fmaf(q, x[2]*x[12], g[1]);
    g[2] = fmaf(q, x[1]*x[12], g[2]);
    g[12] = fmaf(q, x[1]*x[2], g[12]);
  }
  { const float q = w * __ldg(cf + 32 * C);
    g[1] = fmaf(q, x[2]*x[14], g[1]);
    g[2] = fmaf(q, x[1]*x[14], g[2]);
    g[14] = fmaf(q, x[1]*x[2], g[14]);
  }
  { const float q = w * __ldg(cf + 33 * C);
    g[1] = fmaf(q, x[3]*x[3], g[1]);
    g[3] = fmaf(q, x[1]*x[3], g[3]);
    g[3] = fmaf(q, x[1]*x[3], g[3]);
  }
  { const float q = w * __ldg(cf + 34 * C);
    g[1] = fmaf(q, x[3]*x[13], g[1]);
    g[3] = fmaf(q, x[1]*x[13], g[3]);
    g[13] = fmaf(q, x[1]*x[3], g[13]);
  }
  { const float q = w * __ldg(cf + 35 * C);
    g[1] = fmaf(q, x[3]*x[15], g[1]);
    g[3] = fmaf(q, x[1]*x[15], g[3]);
    g[15] = fmaf(q, x[1]*x[3], g[15]);
  }
  { const float q = w * __ldg(cf + 36 * C);
    g[1] = fmaf(q, x[4]*x[4], g[1]);
    g[4] = fmaf(q, x[1]*x[4], g[4]);
    g[4] = fmaf(q, x[1]*x[4], g[4]);
  }
  { const float q = w * __ldg(cf + 37 * C);
    g[1] = fmaf(q, x[5]*x[5], g[1]);
    g[5] = fmaf(q, x[1]*x[5], g[5]);
    g[5] = fmaf(q, x[1]*x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 38 * C);
    g[1] = fmaf(q, x[6]*x[6], g[1]);
    g[6] = fmaf(q, x[1]*x[6], g[6]);
    g[6] = fmaf(q, x[1]*x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 39 * C);
    g[1] = fmaf(q, x[6]*x[8], g[1]);
    g[6] = fmaf(q, x[1]*x[8], g[6]);
    g[8] = fmaf(q, x[1]*x[6], g[8]);
  }
  { const float q = w * __ldg(cf + 40 * C);
    g[1] = fmaf(q, x[7]*x[7], g[1]);
    g[7] = fmaf(q, x[1]*x[7], g[7]);
    g[7] = fmaf(q, x[1]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 41 * C);
    g[1] = fmaf(q, x[8]*x[8], g[1]);
    g[8] = fmaf(q, x[1]*x[8], g[8]);
    g[8] = fmaf(q, x[1]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 42 * C);
    g[1] = fmaf(q, x[9]*x[9], g[1]);
    g[9] = fmaf(q, x[1]*x[9], g[9]);
    g[9] = fmaf(q, x[1]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 43 * C);
    g[1] = fmaf(q, x[9]*x[11], g[1]);
    g[9] = fmaf(q, x[1]*x[11], g[9]);
    g[11] = fmaf(q, x[1]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 44 * C);
    g[1] = fmaf(q, x[10]*x[10], g[1]);
    g[10] = fmaf(q, x[1]*x[10], g[10]);
    g[10] = fmaf(q, x[1]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 45 * C);
    g[1] = fmaf(q, x[11]*x[11], g[1]);
    g[11] = fmaf(q, x[1]*x[11], g[11]);
    g[11] = fmaf(q, x[1]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 46 * C);
    g[1] = fmaf(q, x[12]*x[12], g[1]);
    g[12] = fmaf(q, x[1]*x[12], g[12]);
    g[12] = fmaf(q, x[1]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 47 * C);
    g[1] = fmaf(q, x[12]*x[14], g[1]);
    g[12] = fmaf(q, x[1]*x[14], g[12]);
    g[14] = fmaf(q, x[1]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 48 * C);
    g[1] = fmaf(q, x[13]*x[13], g[1]);
    g[13] = fmaf(q, x[1]*x[13], g[13]);
    g[13] = fmaf(q, x[1]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 49 * C);
    g[1] = fmaf(q, x[13]*x[15], g[1]);
    g[13] = fmaf(q, x[1]*x[15], g[13]);
    g[15] = fmaf(q, x[1]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 50 * C);
    g[1] = fmaf(q, x[14]*x[14], g[1]);
    g[14] = fmaf(q, x[1]*x[14], g[14]);
    g[14] = fmaf(q, x[1]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 51 * C);
    g[1] = fmaf(q, x[15]*x[15], g[1]);
    g[15] = fmaf(q, x[1]*x[15], g[15]);
    g[15] = fmaf(q, x[1]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 52 * C);
    g[2] = fmaf(q, x[2]*x[11], g[2]);
    g[2] = fmaf(q, x[2]*x[11], g[2]);
    g[11] = fmaf(q, x[2]*x[2], g[11]);
  }
  { const float q = w * __ldg(cf + 53 * C);
    g[2] = fmaf(q, x[3]*x[10], g[2]);
    g[3] = fmaf(q, x[2]*x[10], g[3]);
    g[10] = fmaf(q, x[2]*x[3], g[10]);
  }
  { const float q = w * __ldg(cf + 54 * C);
    g[2] = fmaf(q, x[4]*x[7], g[2]);
    g[4] = fmaf(q, x[2]*x[7], g[4]);
    g[7] = fmaf(q, x[2]*x[4], g[7]);
  }
  { const float q = w * __ldg(cf + 55 * C);
    g[2] = fmaf(q, x[5]*x[6], g[2]);
    g[5] = fmaf(q, x[2]*x[6], g[5]);
    g[6] = fmaf(q, x[2]*x[5], g[6]);
  }
  { const float q = w * __ldg(cf + 56 * C);
    g[2] = fmaf(q, x[5]*x[8], g[2]);
    g[5] = fmaf(q, x[2]*x[8], g[5]);
    g[8] = fmaf(q, x[2]*x[5], g[8]);
  }
  { const float q = w * __ldg(cf + 57 * C);
    g[2] = fmaf(q, x[9]*x[14], g[2]);
    g[9] = fmaf(q, x[2]*x[14], g[9]);
    g[14] = fmaf(q, x[2]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 58 * C);
    g[2] = fmaf(q, x[10]*x[13], g[2]);
    g[10] = fmaf(q, x[2]*x[13], g[10]);
    g[13] = fmaf(q, x[2]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 59 * C);
    g[2] = fmaf(q, x[10]*x[15], g[2]);
    g[10] = fmaf(q, x[2]*x[15], g[10]);
    g[15] = fmaf(q, x[2]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 60 * C);
    g[2] = fmaf(q, x[11]*x[12], g[2]);
    g[11] = fmaf(q, x[2]*x[12], g[11]);
    g[12] = fmaf(q, x[2]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 61 * C);
    g[2] = fmaf(q, x[11]*x[14], g[2]);
    g[11] = fmaf(q, x[2]*x[14], g[11]);
    g[14] = fmaf(q, x[2]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 62 * C);
    g[3] = fmaf(q, x[3]*x[9], g[3]);
    g[3] = fmaf(q, x[3]*x[9], g[3]);
    g[9] = fmaf(q, x[3]*x[3], g[9]);
  }
  { const float q = w * __ldg(cf + 63 * C);
    g[3] = fmaf(q, x[3]*x[11], g[3]);
    g[3] = fmaf(q, x[3]*x[11], g[3]);
    g[11] = fmaf(q, x[3]*x[3], g[11]);
  }
  { const float q = w * __ldg(cf + 64 * C);
    g[3] = fmaf(q, x[4]*x[6], g[3]);
    g[4] = fmaf(q, x[3]*x[6], g[4]);
    g[6] = fmaf(q, x[3]*x[4], g[6]);
  }
  { const float q = w * __ldg(cf + 65 * C);
    g[3] = fmaf(q, x[5]*x[7], g[3]);
    g[5] = fmaf(q, x[3]*x[7], g[5]);
    g[7] = fmaf(q, x[3]*x[5], g[7]);
  }
  { const float q = w * __ldg(cf + 66 * C);
    g[3] = fmaf(q, x[9]*x[13], g[3]);
    g[9] = fmaf(q, x[3]*x[13], g[9]);
    g[13] = fmaf(q, x[3]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 67 * C);
    g[3] = fmaf(q, x[10]*x[12], g[3]);
    g[10] = fmaf(q, x[3]*x[12], g[10]);
    g[12] = fmaf(q, x[3]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 68 * C);
    g[3] = fmaf(q, x[11]*x[13], g[3]);
    g[11] = fmaf(q, x[3]*x[13], g[11]);
    g[13] = fmaf(q, x[3]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 69 * C);
    g[3] = fmaf(q, x[11]*x[15], g[3]);
    g[11] = fmaf(q, x[3]*x[15], g[11]);
    g[15] = fmaf(q, x[3]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 70 * C);
    g[4] = fmaf(q, x[4]*x[9], g[4]);
    g[4] = fmaf(q, x[4]*x[9], g[4]);
    g[9] = fmaf(q, x[4]*x[4], g[9]);
  }
  { const float q = w * __ldg(cf + 71 * C);
    g[4] = fmaf(q, x[4]*x[11], g[4]);
    g[4] = fmaf(q, x[4]*x[11], g[4]);
    g[11] = fmaf(q, x[4]*x[4], g[11]);
  }
  { const float q = w * __ldg(cf + 72 * C);
    g[4] = fmaf(q, x[5]*x[10], g[4]);
    g[5] = fmaf(q, x[4]*x[10], g[5]);
    g[10] = fmaf(q, x[4]*x[5], g[10]);
  }
  { const float q = w * __ldg(cf + 73 * C);
    g[4] = fmaf(q, x[6]*x[13], g[4]);
    g[6] = fmaf(q, x[4]*x[13], g[6]);
    g[13] = fmaf(q, x[4]*x[6], g[13]);
  }
  { const float q = w * __ldg(cf + 74 * C);
    g[4] = fmaf(q, x[6]*x[15], g[4]);
    g[6] = fmaf(q, x[4]*x[15], g[6]);
    g[15] = fmaf(q, x[4]*x[6], g[15]);
  }
  { const float q = w * __ldg(cf + 75 * C);
    g[4] = fmaf(q, x[7]*x[12], g[4]);
    g[7] = fmaf(q, x[4]*x[12], g[7]);
    g[12] = fmaf(q, x[4]*x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 76 * C);
    g[4] = fmaf(q, x[7]*x[14], g[4]);
    g[7] = fmaf(q, x[4]*x[14], g[7]);
    g[14] = fmaf(q, x[4]*x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 77 * C);
    g[4] = fmaf(q, x[8]*x[15], g[4]);
    g[8] = fmaf(q, x[4]*x[15], g[8]);
    g[15] = fmaf(q, x[4]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 78 * C);
    g[5] = fmaf(q, x[5]*x[9], g[5]);
    g[5] = fmaf(q, x[5]*x[9], g[5]);
    g[9] = fmaf(q, x[5]*x[5], g[9]);
  }
  { const float q = w * __ldg(cf + 79 * C);
    g[5] = fmaf(q, x[5]*x[11], g[5]);
    g[5] = fmaf(q, x[5]*x[11], g[5]);
    g[11] = fmaf(q, x[5]*x[5], g[11]);
  }
  { const float q = w * __ldg(cf + 80 * C);
    g[5] = fmaf(q, x[6]*x[12], g[5]);
    g[6] = fmaf(q, x[5]*x[12], g[6]);
    g[12] = fmaf(q, x[5]*x[6], g[12]);
  }
  { const float q = w * __ldg(cf + 81 * C);
    g[5] = fmaf(q, x[6]*x[14], g[5]);
    g[6] = fmaf(q, x[5]*x[14], g[6]);
    g[14] = fmaf(q, x[5]*x[6], g[14]);
  }
  { const float q = w * __ldg(cf + 82 * C);
    g[5] = fmaf(q, x[7]*x[13], g[5]);
    g[7] = fmaf(q, x[5]*x[13], g[7]);
    g[13] = fmaf(q, x[5]*x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 83 * C);
    g[5] = fmaf(q, x[7]*x[15], g[5]);
    g[7] = fmaf(q, x[5]*x[15], g[7]);
    g[15] = fmaf(q, x[5]*x[7], g[15]);
  }
  { const float q = w * __ldg(cf + 84 * C);
    g[5] = fmaf(q, x[8]*x[12], g[5]);
    g[8] = fmaf(q, x[5]*x[12], g[8]);
    g[12] = fmaf(q, x[5]*x[8], g[12]);
  }
  { const float q = w * __ldg(cf + 85 * C);
    g[5] = fmaf(q, x[8]*x[14], g[5]);
    g[8] = fmaf(q, x[5]*x[14], g[8]);
    g[14] = fmaf(q, x[5]*x[8], g[14]);
  }
  { const float q = w * __ldg(cf + 86 * C);
    g[6] = fmaf(q, x[6]*x[11], g[6]);
    g[6] = fmaf(q, x[6]*x[11], g[6]);
    g[11] = fmaf(q, x[6]*x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 87 * C);
    g[6] = fmaf(q, x[7]*x[10], g[6]);
    g[7] = fmaf(q, x[6]*x[10], g[7]);
    g[10] = fmaf(q, x[6]*x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 88 * C);
    g[6] = fmaf(q, x[8]*x[9], g[6]);
    g[8] = fmaf(q, x[6]*x[9], g[8]);
    g[9] = fmaf(q, x[6]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 89 * C);
    g[6] = fmaf(q, x[8]*x[11], g[6]);
    g[8] = fmaf(q, x[6]*x[11], g[8]);
    g[11] = fmaf(q, x[6]*x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 90 * C);
    g[7] = fmaf(q, x[7]*x[9], g[7]);
    g[7] = fmaf(q, x[7]*x[9], g[7]);
    g[9] = fmaf(q, x[7]*x[7], g[9]);
  }
  { const float q = w * __ldg(cf + 91 * C);
    g[7] = fmaf(q, x[7]*x[11], g[7]);
    g[7] = fmaf(q, x[7]*x[11], g[7]);
    g[11] = fmaf(q, x[7]*x[7], g[11]);
  }
  { const float q = w * __ldg(cf + 92 * C);
    g[7] = fmaf(q, x[8]*x[10], g[7]);
    g[8] = fmaf(q, x[7]*x[10], g[8]);
    g[10] = fmaf(q, x[7]*x[8], g[10]);
  }
  { const float q = w * __ldg(cf + 93 * C);
    g[8] = fmaf(q, x[8]*x[9], g[8]);
    g[8] = fmaf(q, x[8]*x[9], g[8]);
    g[9] = fmaf(q, x[8]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 94 * C);
    g[8] = fmaf(q, x[8]*x[11], g[8]);
    g[8] = fmaf(q, x[8]*x[11], g[8]);
    g[11] = fmaf(q, x[8]*x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 95 * C);
    g[9] = fmaf(q, x[9]*x[11], g[9]);
    g[9] = fmaf(q, x[9]*x[11], g[9]);
    g[11] = fmaf(q, x[9]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 96 * C);
    g[9] = fmaf(q, x[10]*x[10], g[9]);
    g[10] = fmaf(q, x[9]*x[10], g[10]);
    g[10] = fmaf(q, x[9]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 97 * C);
    g[9] = fmaf(q, x[11]*x[11], g[9]);
    g[11] = fmaf(q, x[9]*x[11], g[11]);
    g[11] = fmaf(q, x[9]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 98 * C);
    g[9] = fmaf(q, x[12]*x[14], g[9]);
    g[12] = fmaf(q, x[9]*x[14], g[12]);
    g[14] = fmaf(q, x[9]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 99 * C);
    g[9] = fmaf(q, x[13]*x[13], g[9]);
    g[13] = fmaf(q, x[9]*x[13], g[13]);
    g[13] = fmaf(q, x[9]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 100 * C);
    g[9] = fmaf(q, x[14]*x[14], g[9]);
    g[14] = fmaf(q, x[9]*x[14], g[14]);
    g[14] = fmaf(q, x[9]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 101 * C);
    g[10] = fmaf(q, x[10]*x[11], g[10]);
    g[10] = fmaf(q, x[10]*x[11], g[10]);
    g[11] = fmaf(q, x[10]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 102 * C);
    g[10] = fmaf(q, x[12]*x[13], g[10]);
    g[12] = fmaf(q, x[10]*x[13], g[12]);
    g[13] = fmaf(q, x[10]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 103 * C);
    g[10] = fmaf(q, x[12]*x[15], g[10]);
    g[12] = fmaf(q, x[10]*x[15], g[12]);
    g[15] = fmaf(q, x[10]*x[12], g[15]);
  }
  { const float q = w * __ldg(cf + 104 * C);
    g[10] = fmaf(q, x[14]*x[15], g[10]);
    g[14] = fmaf(q, x[10]*x[15], g[14]);
    g[15] = fmaf(q, x[10]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 105 * C);
    g[11] = fmaf(q, x[11]*x[11], g[11]);
    g[11] = fmaf(q, x[11]*x[11], g[11]);
    g[11] = fmaf(q, x[11]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 106 * C);
    g[11] = fmaf(q, x[12]*x[12], g[11]);
    g[12] = fmaf(q, x[11]*x[12], g[12]);
    g[12] = fmaf(q, x[11]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 107 * C);
    g[11] = fmaf(q, x[12]*x[14], g[11]);
    g[12] = fmaf(q, x[11]*x[14], g[12]);
    g[14] = fmaf(q, x[11]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 108 * C);
    g[11] = fmaf(q, x[13]*x[13], g[11]);
    g[13] = fmaf(q, x[11]*x[13], g[13]);
    g[13] = fmaf(q, x[11]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 109 * C);
    g[11] = fmaf(q, x[13]*x[15], g[11]);
    g[13] = fmaf(q, x[11]*x[15], g[13]);
    g[15] = fmaf(q, x[11]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 110 * C);
    g[11] = fmaf(q, x[14]*x[14], g[11]);
    g[14] = fmaf(q, x[11]*x[14], g[14]);
    g[14] = fmaf(q, x[11]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 111 * C);
    g[11] = fmaf(q, x[15]*x[15], g[11]);
    g[15] = fmaf(q, x[11]*x[15], g[15]);
    g[15] = fmaf(q, x[11]*x[15], g[15]);
  }
}

__device__ __forceinline__ float value_LM2(const float* x, const float* __restrict__ cf, int C) {
  float f = 0.0f;
  f = fmaf(__ldg(cf + 0 * C), x[2], f);
  f = fmaf(__ldg(cf + 1 * C), x[0]*x[2], f);
  f = fmaf(__ldg(cf + 2 * C), x[1]*x[5], f);
  f = fmaf(__ldg(cf + 3 * C), x[2]*x[6], f);
  f = fmaf(__ldg(cf + 4 * C), x[3]*x[7], f);
  f = fmaf(__ldg(cf + 5 * C), x[4]*x[10], f);
  f = fmaf(__ldg(cf + 6 * C), x[5]*x[11], f);
  f = fmaf(__ldg(cf + 7 * C), x[6]*x[12], f);
  f = fmaf(__ldg(cf + 8 * C), x[7]*x[13], f);
  f = fmaf(__ldg(cf + 9 * C), x[8]*x[14], f);
  f = fmaf(__ldg(cf + 10 * C), x[0]*x[0]*x[2], f);
  f = fmaf(__ldg(cf + 11 * C), x[0]*x[1]*x[5], f);
  f = fmaf(__ldg(cf + 12 * C), x[0]*x[2]*x[6], f);
  f = fmaf(__ldg(cf + 13 * C), x[0]*x[3]*x[7], f);
  f = fmaf(__ldg(cf + 14 * C), x[0]*x[4]*x[10], f);
  f = fmaf(__ldg(cf + 15 * C), x[0]*x[5]*x[11], f);
  f = fmaf(__ldg(cf + 16 * C), x[0]*x[6]*x[12], f);
  f = fmaf(__ldg(cf + 17 * C), x[0]*x[7]*x[13], f);
  f = fmaf(__ldg(cf + 18 * C), x[0]*x[8]*x[14], f);
  f = fmaf(__ldg(cf + 19 * C), x[1]*x[1]*x[2], f);
  f = fmaf(__ldg(cf + 20 * C), x[1]*x[1]*x[12], f);
  f = fmaf(__ldg(cf + 21 * C), x[1]*x[1]*x[14], f);
  f = fmaf(__ldg(cf + 22 * C), x[1]*x[2]*x[11], f);
  f = fmaf(__ldg(cf + 23 * C), x[1]*x[3]*x[10], f);
  f = fmaf(__ldg(cf + 24 * C), x[1]*x[4]*x[7], f);
  f = fmaf(__ldg(cf + 25 * C), x[1]*x[5]*x[6], f);
  f = fmaf(__ldg(cf + 26 * C), x[1]*x[5]*x[8], f);
  f = fmaf(__ldg(cf + 27 * C), x[1]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 28 * C), x[1]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 29 * C), x[1]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 30 * C), x[1]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 31 * C), x[1]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 32 * C), x[2]*x[2]*x[2], f);
  f = fmaf(__ldg(cf + 33 * C), x[2]*x[2]*x[12], f);
  f = fmaf(__ldg(cf + 34 * C), x[2]*x[3]*x[3], f);
  f = fmaf(__ldg(cf + 35 * C), x[2]*x[3]*x[13], f);
  f = fmaf(__ldg(cf + 36 * C), x[2]*x[4]*x[4], f);
  f = fmaf(__ldg(cf + 37 * C), x[2]*x[5]*x[5], f);
  f = fmaf(__ldg(cf + 38 * C), x[2]*x[6]*x[6], f);
  f = fmaf(__ldg(cf + 39 * C), x[2]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 40 * C), x[2]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 41 * C), x[2]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 42 * C), x[2]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 43 * C), x[2]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 44 * C), x[2]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 45 * C), x[2]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 46 * C), x[2]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 47 * C), x[2]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 48 * C), x[3]*x[3]*x[12], f);
  f = fmaf(__ldg(cf + 49 * C), x[3]*x[3]*x[14], f);
  f = fmaf(__ldg(cf + 50 * C), x[3]*x[4]*x[5], f);
  f = fmaf(__ldg(cf + 51 * C), x[3]*x[6]*x[7], f);
  f = fmaf(__ldg(cf + 52 * C), x[3]*x[7]*x[8], f);
  f = fmaf(__ldg(cf + 53 * C), x[3]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 54 * C), x[3]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 55 * C), x[3]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 56 * C), x[3]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 57 * C), x[3]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 58 * C), x[4]*x[4]*x[12], f);
  f = fmaf(__ldg(cf + 59 * C), x[4]*x[5]*x[13], f);
  f = fmaf(__ldg(cf + 60 * C), x[4]*x[5]*x[15], f);
  f = fmaf(__ldg(cf + 61 * C), x[4]*x[6]*x[10], f);
  f = fmaf(__ldg(cf + 62 * C), x[4]*x[7]*x[9], f);
  f = fmaf(__ldg(cf + 63 * C), x[4]*x[7]*x[11], f);
  f = fmaf(__ldg(cf + 64 * C), x[5]*x[5]*x[12], f);
  f = fmaf(__ldg(cf + 65 * C), x[5]*x[5]*x[14], f);
  f = fmaf(__ldg(cf + 66 * C), x[5]*x[6]*x[11], f);
  f = fmaf(__ldg(cf + 67 * C), x[5]*x[7]*x[10], f);
  f = fmaf(__ldg(cf + 68 * C), x[5]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 69 * C), x[5]*x[8]*x[11], f);
  f = fmaf(__ldg(cf + 70 * C), x[6]*x[6]*x[12], f);
  f = fmaf(__ldg(cf + 71 * C), x[6]*x[7]*x[13], f);
  f = fmaf(__ldg(cf + 72 * C), x[6]*x[8]*x[14], f);
  f = fmaf(__ldg(cf + 73 * C), x[7]*x[7]*x[12], f);
  f = fmaf(__ldg(cf + 74 * C), x[7]*x[7]*x[14], f);
  f = fmaf(__ldg(cf + 75 * C), x[7]*x[8]*x[13], f);
  f = fmaf(__ldg(cf + 76 * C), x[7]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 77 * C), x[8]*x[8]*x[12], f);
  f = fmaf(__ldg(cf + 78 * C), x[9]*x[9]*x[12], f);
  f = fmaf(__ldg(cf + 79 * C), x[9]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 80 * C), x[9]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 81 * C), x[10]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 82 * C), x[10]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 83 * C), x[10]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 84 * C), x[11]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 85 * C), x[11]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 86 * C), x[12]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 87 * C), x[12]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 88 * C), x[12]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 89 * C), x[12]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 90 * C), x[13]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 91 * C), x[13]*x[14]*x[15], f);
  return f;
}

__device__ __forceinline__ void grad_LM2(const float* x, float w, const float* __restrict__ cf, int C, float* g) {
  { const float q = w * __ldg(cf + 0 * C);
    g[2] += q;
  }
  { const float q = w * __ldg(cf + 1 * C);
    g[0] = fmaf(q, x[2], g[0]);
    g[2] = fmaf(q, x[0], g[2]);
  }
  { const float q = w * __ldg(cf + 2 * C);
    g[1] = fmaf(q, x[5], g[1]);
    g[5] = fmaf(q, x[1], g[5]);
  }
  { const float q = w * __ldg(cf + 3 * C);
    g[2] = fmaf(q, x[6], g[2]);
    g[6] = fmaf(q, x[2], g[6]);
  }
  { const float q = w * __ldg(cf + 4 * C);
    g[3] = fmaf(q, x[7], g[3]);
    g[7] = fmaf(q, x[3], g[7]);
  }
  { const float q = w * __ldg(cf + 5 * C);
    g[4] = fmaf(q, x[10], g[4]);
    g[10] = fmaf(q, x[4], g[10]);
  }
  { const float q = w * __ldg(cf + 6 * C);
    g[5] = fmaf(q, x[11], g[5]);
    g[11] = fmaf(q, x[5], g[11]);
  }
  { const float q = w * __ldg(cf + 7 * C);
    g[6] = fmaf(q, x[12], g[6]);
    g[12] = fmaf(q, x[6], g[12]);
  }
  { const float q = w * __ldg(cf + 8 * C);
    g[7] = fmaf(q, x[13], g[7]);
    g[13] = fmaf(q, x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 9 * C);
    g[8] = fmaf(q, x[14], g[8]);
    g[14] = fmaf(q, x[8], g[14]);
  }
  { const float q = w * __ldg(cf + 10 * C);
    g[0] = fmaf(q, x[0]*x[2], g[0]);
    g[0] = fmaf(q, x[0]*x[2], g[0]);
    g[2] = fmaf(q, x[0]*x[0], g[2]);
  }
  { const float q = w * __ldg(cf + 11 * C);
    g[0] = fmaf(q, x[1]*x[5], g[0]);
    g[1] = fmaf(q, x[0]*x[5], g[1]);
    g[5] = fmaf(q, x[0]*x[1], g[5]);
  }
  { const float q = w * __ldg(cf + 12 * C);
    g[0] = fmaf(q, x[2]*x[6], g[0]);
    g[2] = fmaf(q, x[0]*x[6], g[2]);
    g[6] = fmaf(q, x[0]*x[2], g[6]);
  }
  { const float q = w * __ldg(cf + 13 * C);
    g[0] = fmaf(q, x[3]*x[7], g[0]);
    g[3] = fmaf(q, x[0]*x[7], g[3]);
    g[7] = fmaf(q, x[0]*x[3], g[7]);
  }
  { const float q = w * __ldg(cf + 14 * C);
    g[0] = fmaf(q, x[4]*x[10], g[0]);
    g[4] = fmaf(q, x[0]*x[10], g[4]);
    g[10] = fmaf(q, x[0]*x[4], g[10]);
  }
  { const float q = w * __ldg(cf + 15 * C);
    g[0] = fmaf(q, x[5]*x[11], g[0]);
    g[5] = fmaf(q, x[0]*x[11], g[5]);
    g[11] = fmaf(q, x[0]*x[5], g[11]);
  }
  { const float q = w * __ldg(cf + 16 * C);
    g[0] = fmaf(q, x[6]*x[12], g[0]);
    g[6] = fmaf(q, x[0]*x[12], g[6]);
    g[12] = fmaf(q, x[0]*x[6], g[12]);
  }
  { const float q = w * __ldg(cf + 17 * C);
    g[0] = fmaf(q, x[7]*x[13], g[0]);
    g[7] = fmaf(q, x[0]*x[13], g[7]);
    g[13] = fmaf(q, x[0]*x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 18 * C);
    g[0] = fmaf(q, x[8]*x[14], g[0]);
    g[8] = fmaf(q, x[0]*x[14], g[8]);
    g[14] = fmaf(q, x[0]*x[8], g[14]);
  }
  { const float q = w * __ldg(cf + 19 * C);
    g[1] = fmaf(q, x[1]*x[2], g[1]);
    g[1] = fmaf(q, x[1]*x[2], g[1]);
    g[2] = fmaf(q, x[1]*x[1], g[2]);
  }
  { const float q = w * __ldg(cf + 20 * C);
    g[1] = fmaf(q, x[1]*x[12], g[1]);
    g[1] = fmaf(q, x[1]*x[12], g[1]);
    g[12] = fmaf(q, x[1]*x[1], g[12]);
  }
  { const float q = w * __ldg(cf + 21 * C);
    g[1] = fmaf(q, x[1]*x[14], g[1]);
    g[1] = fmaf(q, x[1]*x[14], g[1]);
    g[14] = fmaf(q, x[1]*x[1], g[14]);
  }
  { const float q = w * __ldg(cf + 22 * C);
    g[1] = fmaf(q, x[2]*x[11], g[1]);
    g[2] = fmaf(q, x[1]*x[11], g[2]);
    g[11] = fmaf(q, x[1]*x[2], g[11]);
  }
  { const float q = w * __ldg(cf + 23 * C);
    g[1] = fmaf(q, x[3]*x[10], g[1]);
    g[3] = fmaf(q, x[1]*x[10], g[3]);
    g[10] = fmaf(q, x[1]*x[3], g[10]);
  }
  { const float q = w * __ldg(cf + 24 * C);
    g[1] = fmaf(q, x[4]*x[7], g[1]);
    g[4] = fmaf(q, x[1]*x[7], g[4]);
    g[7] = fmaf(q, x[1]*x[4], g[7]);
  }
  { const float q = w * __ldg(cf + 25 * C);
    g[1] = fmaf(q, x[5]*x[6], g[1]);
    g[5] = fmaf(q, x[1]*x[6], g[5]);
    g[6] = fmaf(q, x[1]*x[5], g[6]);
  }
  { const float q = w * __ldg(cf + 26 * C);
    g[1] = fmaf(q, x[5]*x[8], g[1]);
    g[5] = fmaf(q, x[1]*x[8], g[5]);
    g[8] = fmaf(q, x[1]*x[5], g[8]);
  }
  { const float q = w * __ldg(cf + 27 * C);
    g[1] = fmaf(q, x[9]*x[14], g[1]);
    g[9] = fmaf(q, x[1]*x[14], g[9]);
    g[14] = fmaf(q, x[1]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 28 * C);
    g[1] = fmaf(q, x[10]*x[13], g[1]);
    g[10] = fmaf(q, x[1]*x[13], g[10]);
    g[13] = fmaf(q, x[1]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 29 * C);
    g[1] = fmaf(q, x[10]*x[15], g[1]);
    g[10] = fmaf(q, x[1]*x[15], g[10]);
    g[15] = fmaf(q, x[1]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 30 * C);
    g[1] = fmaf(q, x[11]*x[12], g[1]);
    g[11] = fmaf(q, x[1]*x[12], g[11]);
    g[12] = fmaf(q, x[1]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 31 * C);
    g[1] = fmaf(q, x[11]*x[14], g[1]);
    g[11] = fmaf(q, x[1]*x[14], g[11]);
    g[14] = fmaf(q, x[1]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 32 * C);
    g[2] = fmaf(q, x[2]*x[2], g[2]);
    g[2] = fmaf(q, x[2]*x[2], g[2]);
    g[2] = fmaf(q, x[2]*x[2], g[2]);
  }
  { const float q = w * __ldg(cf + 33 * C);
    g[2] = fmaf(q, x[2]*x[12], g[2]);
    g[2] = fmaf(q, x[2]*x[12], g[2]);
    g[12] = fmaf(q, x[2]*x[2], g[12]);
  }
  { const float q = w * __ldg(cf + 34 * C);
    g[2] = fmaf(q, x[3]*x[3], g[2]);
    g[3] = fmaf(q, x[2]*x[3], g[3]);
    g[3] = fmaf(q, x[2]*x[3], g[3]);
  }
  { const float q = w * __ldg(cf + 35 * C);
    g[2] = fmaf(q, x[3]*x[13], g[2]);
    g[3] = fmaf(q, x[2]*x[13], g[3]);
    g[13] = fmaf(q, x[2]*x[3], g[13]);
  }
  { const float q = w * __ldg(cf + 36 * C);
    g[2] = fmaf(q, x[4]*x[4], g[2]);
    g[4] = fmaf(q, x[2]*x[4], g[4]);
    g[4] = fmaf(q, x[2]*x[4], g[4]);
  }
  { const float q = w * __ldg(cf + 37 * C);
    g[2] = fmaf(q, x[5]*x[5], g[2]);
    g[5] = fmaf(q, x[2]*x[5], g[5]);
    g[5] = fmaf(q, x[2]*x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 38 * C);
    g[2] = fmaf(q, x[6]*x[6], g[2]);
    g[6] = fmaf(q, x[2]*x[6], g[6]);
    g[6] = fmaf(q, x[2]*x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 39 * C);
    g[2] = fmaf(q, x[7]*x[7], g[2]);
    g[7] = fmaf(q, x[2]*x[7], g[7]);
    g[7] = fmaf(q, x[2]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 40 * C);
    g[2] = fmaf(q, x[8]*x[8], g[2]);
    g[8] = fmaf(q, x[2]*x[8], g[8]);
    g[8] = fmaf(q, x[2]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 41 * C);
    g[2] = fmaf(q, x[9]*x[9], g[2]);
    g[9] = fmaf(q, x[2]*x[9], g[9]);
    g[9] = fmaf(q, x[2]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 42 * C);
    g[2] = fmaf(q, x[10]*x[10], g[2]);
    g[10] = fmaf(q, x[2]*x[10], g[10]);
    g[10] = fmaf(q, x[2]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 43 * C);
    g[2] = fmaf(q, x[11]*x[11], g[2]);
    g[11] = fmaf(q, x[2]*x[11], g[11]);
    g[11] = fmaf(q, x[2]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 44 * C);
    g[2] = fmaf(q, x[12]*x[12], g[2]);
    g[12] = fmaf(q, x[2]*x[12], g[12]);
    g[12] = fmaf(q, x[2]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 45 * C);
    g[2] = fmaf(q, x[13]*x[13], g[2]);
    g[13] = fmaf(q, x[2]*x[13], g[13]);
    g[13] = fmaf(q, x[2]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 46 * C);
    g[2] = fmaf(q, x[14]*x[14], g[2]);
    g[14] = fmaf(q, x[2]*x[14], g[14]);
    g[14] = fmaf(q, x[2]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 47 * C);
    g[2] = fmaf(q, x[15]*x[15], g[2]);
    g[15] = fmaf(q, x[2]*x[15], g[15]);
    g[15] = fmaf(q, x[2]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 48 * C);
    g[3] = fmaf(q, x[3]*x[12], g[3]);
    g[3] = fmaf(q, x[3]*x[12], g[3]);
    g[12] = fmaf(q, x[3]*x[3], g[12]);
  }
  { const float q = w * __ldg(cf + 49 * C);
    g[3] = fmaf(q, x[3]*x[14], g[3]);
    g[3] = fmaf(q, x[3]*x[14], g[3]);
    g[14] = fmaf(q, x[3]*x[3], g[14]);
  }
  { const float q = w * __ldg(cf + 50 * C);
    g[3] = fmaf(q, x[4]*x[5], g[3]);
    g[4] = fmaf(q, x[3]*x[5], g[4]);
    g[5] = fmaf(q, x[3]*x[4], g[5]);
  }
  { const float q = w * __ldg(cf + 51 * C);
    g[3] = fmaf(q, x[6]*x[7], g[3]);
    g[6] = fmaf(q, x[3]*x[7], g[6]);
    g[7] = fmaf(q, x[3]*x[6], g[7]);
  }
  { const float q = w * __ldg(cf + 52 * C);
    g[3] = fmaf(q, x[7]*x[8], g[3]);
    g[7] = fmaf(q, x[3]*x[8], g[7]);
    g[8] = fmaf(q, x[3]*x[7], g[8]);
  }
  { const float q = w * __ldg(cf + 53 * C);
    g[3] = fmaf(q, x[9]*x[10], g[3]);
    g[9] = fmaf(q, x[3]*x[10], g[9]);
    g[10] = fmaf(q, x[3]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 54 * C);
    g[3] = fmaf(q, x[10]*x[11], g[3]);
    g[10] = fmaf(q, x[3]*x[11], g[10]);
    g[11] = fmaf(q, x[3]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 55 * C);
    g[3] = fmaf(q, x[12]*x[13], g[3]);
    g[12] = fmaf(q, x[3]*x[13], g[12]);
    g[13] = fmaf(q, x[3]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 56 * C);
    g[3] = fmaf(q, x[13]*x[14], g[3]);
    g[13] = fmaf(q, x[3]*x[14], g[13]);
    g[14] = fmaf(q, x[3]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 57 * C);
    g[3] = fmaf(q, x[14]*x[15], g[3]);
    g[14] = fmaf(q, x[3]*x[15], g[14]);
    g[15] = fmaf(q, x[3]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 58 * C);
    g[4] = fmaf(q, x[4]*x[12], g[4]);
    g[4] = fmaf(q, x[4]*x[12], g[4]);
    g[12] = fmaf(q, x[4]*x[4], g[12]);
  }
  { const float q = w * __ldg(cf + 59 * C);
    g[4] = fmaf(q, x[5]*x[13], g[4]);
    g[5] = fmaf(q, x[4]*x[13], g[5]);
    g[13] = fmaf(q, x[4]*x[5], g[13]);
  }
  { const float q = w * __ldg(cf + 60 * C);
    g[4] = fmaf(q, x[5]*x[15], g[4]);
    g[5] = fmaf(q, x[4]*x[15], g[5]);
    g[15] = fmaf(q, x[4]*x[5], g[15]);
  }
  { const float q = w * __ldg(cf + 61 * C);
    g[4] = fmaf(q, x[6]*x[10], g[4]);
    g[6] = fmaf(q, x[4]*x[10], g[6]);
    g[10] = fmaf(q, x[4]*x[6], g[10]);
  }
  { const float q = w * __ldg(cf + 62 * C);
    g[4] = fmaf(q, x[7]*x[9], g[4]);
    g[7] = fmaf(q, x[4]*x[9], g[7]);
    g[9] = fmaf(q, x[4]*x[7], g[9]);
  }
  { const float q = w * __ldg(cf + 63 * C);
    g[4] = fmaf(q, x[7]*x[11], g[4]);
    g[7] = fmaf(q, x[4]*x[11], g[7]);
    g[11] = fmaf(q, x[4]*x[7], g[11]);
  }
  { const float q = w * __ldg(cf + 64 * C);
    g[5] = fmaf(q, x[5]*x[12], g[5]);
    g[5] = fmaf(q, x[5]*x[12], g[5]);
    g[12] = fmaf(q, x[5]*x[5], g[12]);
  }
  { const float q = w * __ldg(cf + 65 * C);
    g[5] = fmaf(q, x[5]*x[14], g[5]);
    g[5] = fmaf(q, x[5]*x[14], g[5]);
    g[14] = fmaf(q, x[5]*x[5], g[14]);
  }
  { const float q = w * __ldg(cf + 66 * C);
    g[5] = fmaf(q, x[6]*x[11], g[5]);
    g[6] = fmaf(q, x[5]*x[11], g[6]);
    g[11] = fmaf(q, x[5]*x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 67 * C);
    g[5] = fmaf(q, x[7]*x[10], g[5]);
    g[7] = fmaf(q, x[5]*x[10], g[7]);
    g[10] = fmaf(q, x[5]*x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 68 * C);
    g[5] = fmaf(q, x[8]*x[9], g[5]);
    g[8] = fmaf(q, x[5]*x[9], g[8]);
    g[9] = fmaf(q, x[5]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 69 * C);
    g[5] = fmaf(q, x[8]*x[11], g[5]);
    g[8] = fmaf(q, x[5]*x[11], g[8]);
    g[11] = fmaf(q, x[5]*x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 70 * C);
    g[6] = fmaf(q, x[6]*x[12], g[6]);
    g[6] = fmaf(q, x[6]*x[12], g[6]);
    g[12] = fmaf(q, x[6]*x[6], g[12]);
  }
  { const float q = w * __ldg(cf + 71 * C);
    g[6] = fmaf(q, x[7]*x[13], g[6]);
    g[7] = fmaf(q, x[6]*x[13], g[7]);
    g[13] = fmaf(q, x[6]*x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 72 * C);
    g[6] = fmaf(q, x[8]*x[14], g[6]);
    g[8] = fmaf(q, x[6]*x[14], g[8]);
    g[14] = fmaf(q, x[6]*x[8], g[14]);
  }
  { const float q = w * __ldg(cf + 73 * C);
    g[7] = fmaf(q, x[7]*x[12], g[7]);
    g[7] = fmaf(q, x[7]*x[12], g[7]);
    g[12] = fmaf(q, x[7]*x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 74 * C);
    g[7] = fmaf(q, x[7]*x[14], g[7]);
    g[7] = fmaf(q, x[7]*x[14], g[7]);
    g[14] = fmaf(q, x[7]*x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 75 * C);
    g[7] = fmaf(q, x[8]*x[13], g[7]);
    g[8] = fmaf(q, x[7]*x[13], g[8]);
    g[13] = fmaf(q, x[7]*x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 76 * C);
    g[7] = fmaf(q, x[8]*x[15], g[7]);
    g[8] = fmaf(q, x[7]*x[15], g[8]);
    g[15] = fmaf(q, x[7]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 77 * C);
    g[8] = fmaf(q, x[8]*x[12], g[8]);
    g[8] = fmaf(q, x[8]*x[12], g[8]);
    g[12] = fmaf(q, x[8]*x[8], g[12]);
  }
  { const float q = w * __ldg(cf + 78 * C);
    g[9] = fmaf(q, x[9]*x[12], g[9]);
    g[9] = fmaf(q, x[9]*x[12], g[9]);
    g[12] = fmaf(q, x[9]*x[9], g[12]);
  }
  { const float q = w * __ldg(cf + 79 * C);
    g[9] = fmaf(q, x[10]*x[13], g[9]);
    g[10] = fmaf(q, x[9]*x[13], g[10]);
    g[13] = fmaf(q, x[9]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 80 * C);
    g[9] = fmaf(q, x[11]*x[14], g[9]);
    g[11] = fmaf(q, x[9]*x[14], g[11]);
    g[14] = fmaf(q, x[9]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 81 * C);
    g[10] = fmaf(q, x[10]*x[12], g[10]);
    g[10] = fmaf(q, x[10]*x[12], g[10]);
    g[12] = fmaf(q, x[10]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 82 * C);
    g[10] = fmaf(q, x[11]*x[13], g[10]);
    g[11] = fmaf(q, x[10]*x[13], g[11]);
    g[13] = fmaf(q, x[10]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 83 * C);
    g[10] = fmaf(q, x[11]*x[15], g[10]);
    g[11] = fmaf(q, x[10]*x[15], g[11]);
    g[15] = fmaf(q, x[10]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 84 * C);
    g[11] = fmaf(q, x[11]*x[12], g[11]);
    g[11] = fmaf(q, x[11]*x[12], g[11]);
    g[12] = fmaf(q, x[11]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 85 * C);
    g[11] = fmaf(q, x[11]*x[14], g[11]);
    g[11] = fmaf(q, x[11]*x[14], g[11]);
    g[14] = fmaf(q, x[11]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 86 * C);
    g[12] = fmaf(q, x[12]*x[12], g[12]);
    g[12] = fmaf(q, x[12]*x[12], g[12]);
    g[12] = fmaf(q, x[12]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 87 * C);
    g[12] = fmaf(q, x[13]*x[13], g[12]);
    g[13] = fmaf(q, x[12]*x[13], g[13]);
    g[13] = fmaf(q, x[12]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 88 * C);
    g[12] = fmaf(q, x[14]*x[14], g[12]);
    g[14] = fmaf(q, x[12]*x[14], g[14]);
    g[14] = fmaf(q, x[12]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 89 * C);
    g[12] = fmaf(q, x[15]*x[15], g[12]);
    g[15] = fmaf(q, x[12]*x[15], g[15]);
    g[15] = fmaf(q, x[12]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 90 * C);
    g[13] = fmaf(q, x[13]*x[14], g[13]);
    g[13] = fmaf(q, x[13]*x[14], g[13]);
    g[14] = fmaf(q, x[13]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 91 * C);
    g[13] = fmaf(q, x[14]*x[15], g[13]);
    g[14] = fmaf(q, x[13]*x[15], g[14]);
    g[15] = fmaf(q, x[13]*x[14], g[15]);
  }
}

__device__ __forceinline__ float value_LM3(const float* x, const float* __restrict__ cf, int C) {
  float f = 0.0f;
  f = fmaf(__ldg(cf + 0 * C), x[3], f);
  f = fmaf(__ldg(cf + 1 * C), x[0]*x[3], f);
  f = fmaf(__ldg(cf + 2 * C), x[1]*x[4], f);
  f = fmaf(__ldg(cf + 3 * C), x[2]*x[7], f);
  f = fmaf(__ldg(cf + 4 * C), x[3]*x[6], f);
  f = fmaf(__ldg(cf + 5 * C), x[3]*x[8], f);
  f = fmaf(__ldg(cf + 6 * C), x[4]*x[9], f);
  f = fmaf(__ldg(cf + 7 * C), x[4]*x[11], f);
  f = fmaf(__ldg(cf + 8 * C), x[5]*x[10], f);
  f = fmaf(__ldg(cf + 9 * C), x[6]*x[13], f);
  f = fmaf(__ldg(cf + 10 * C), x[7]*x[12], f);
  f = fmaf(__ldg(cf + 11 * C), x[7]*x[14], f);
  f = fmaf(__ldg(cf + 12 * C), x[8]*x[13], f);
  f = fmaf(__ldg(cf + 13 * C), x[8]*x[15], f);
  f = fmaf(__ldg(cf + 14 * C), x[0]*x[0]*x[3], f);
  f = fmaf(__ldg(cf + 15 * C), x[0]*x[1]*x[4], f);
  f = fmaf(__ldg(cf + 16 * C), x[0]*x[2]*x[7], f);
  f = fmaf(__ldg(cf + 17 * C), x[0]*x[3]*x[6], f);
  f = fmaf(__ldg(cf + 18 * C), x[0]*x[3]*x[8], f);
  f = fmaf(__ldg(cf + 19 * C), x[0]*x[4]*x[9], f);
  f = fmaf(__ldg(cf + 20 * C), x[0]*x[4]*x[11], f);
  f = fmaf(__ldg(cf + 21 * C), x[0]*x[5]*x[10], f);
  f = fmaf(__ldg(cf + 22 * C), x[0]*x[6]*x[13], f);
  f = fmaf(__ldg(cf + 23 * C), x[0]*x[7]*x[12], f);
  f = fmaf(__ldg(cf + 24 * C), x[0]*x[7]*x[14], f);
  f = fmaf(__ldg(cf + 25 * C), x[0]*x[8]*x[13], f);
  f = fmaf(__ldg(cf + 26 * C), x[0]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 27 * C), x[1]*x[1]*x[3], f);
  f = fmaf(__ldg(cf + 28 * C), x[1]*x[1]*x[13], f);
  f = fmaf(__ldg(cf + 29 * C), x[1]*x[1]*x[15], f);
  f = fmaf(__ldg(cf + 30 * C), x[1]*x[2]*x[10], f);
  f = fmaf(__ldg(cf + 31 * C), x[1]*x[3]*x[9], f);
  f = fmaf(__ldg(cf + 32 * C), x[1]*x[3]*x[11], f);
  f = fmaf(__ldg(cf + 33 * C), x[1]*x[4]*x[6], f);
  f = fmaf(__ldg(cf + 34 * C), x[1]*x[5]*x[7], f);
  f = fmaf(__ldg(cf + 35 * C), x[1]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 36 * C), x[1]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 37 * C), x[1]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 38 * C), x[1]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 39 * C), x[2]*x[2]*x[3], f);
  f = fmaf(__ldg(cf + 40 * C), x[2]*x[2]*x[13], f);
  f = fmaf(__ldg(cf + 41 * C), x[2]*x[3]*x[12], f);
  f = fmaf(__ldg(cf + 42 * C), x[2]*x[3]*x[14], f);
  f = fmaf(__ldg(cf + 43 * C), x[2]*x[4]*x[5], f);
  f = fmaf(__ldg(cf + 44 * C), x[2]*x[6]*x[7], f);
  f = fmaf(__ldg(cf + 45 * C), x[2]*x[7]*x[8], f);
  f = fmaf(__ldg(cf + 46 * C), x[2]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 47 * C), x[2]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 48 * C), x[2]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 49 * C), x[2]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 50 * C), x[2]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 51 * C), x[3]*x[3]*x[3], f);
  f = fmaf(__ldg(cf + 52 * C), x[3]*x[3]*x[13], f);
  f = fmaf(__ldg(cf + 53 * C), x[3]*x[3]*x[15], f);
  f = fmaf(__ldg(cf + 54 * C), x[3]*x[4]*x[4], f);
  f = fmaf(__ldg(cf + 55 * C), x[3]*x[5]*x[5], f);
  f = fmaf(__ldg(cf + 56 * C), x[3]*x[6]*x[6], f);
  f = fmaf(__ldg(cf + 57 * C), x[3]*x[6]*x[8], f);
  f = fmaf(__ldg(cf + 58 * C), x[3]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 59 * C), x[3]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 60 * C), x[3]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 61 * C), x[3]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 62 * C), x[3]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 63 * C), x[3]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 64 * C), x[3]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 65 * C), x[3]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 66 * C), x[3]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 67 * C), x[3]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 68 * C), x[3]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 69 * C), x[3]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 70 * C), x[4]*x[4]*x[13], f);
  f = fmaf(__ldg(cf + 71 * C), x[4]*x[4]*x[15], f);
  f = fmaf(__ldg(cf + 72 * C), x[4]*x[5]*x[12], f);
  f = fmaf(__ldg(cf + 73 * C), x[4]*x[5]*x[14], f);
  f = fmaf(__ldg(cf + 74 * C), x[4]*x[6]*x[9], f);
  f = fmaf(__ldg(cf + 75 * C), x[4]*x[6]*x[11], f);
  f = fmaf(__ldg(cf + 76 * C), x[4]*x[7]*x[10], f);
  f = fmaf(__ldg(cf + 77 * C), x[4]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 78 * C), x[5]*x[5]*x[13], f);
  f = fmaf(__ldg(cf + 79 * C), x[5]*x[5]*x[15], f);
  f = fmaf(__ldg(cf + 80 * C), x[5]*x[6]*x[10], f);
  f = fmaf(__ldg(cf + 81 * C), x[5]*x[7]*x[9], f);
  f = fmaf(__ldg(cf + 82 * C), x[5]*x[7]*x[11], f);
  f = fmaf(__ldg(cf + 83 * C), x[5]*x[8]*x[10], f);
  f = fmaf(__ldg(cf + 84 * C), x[6]*x[6]*x[13], f);
  f = fmaf(__ldg(cf + 85 * C), x[6]*x[7]*x[12], f);
  f = fmaf(__ldg(cf + 86 * C), x[6]*x[7]*x[14], f);
  f = fmaf(__ldg(cf + 87 * C), x[6]*x[8]*x[13], f);
  f = fmaf(__ldg(cf + 88 * C), x[6]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 89 * C), x[7]*x[7]*x[13], f);
  f = fmaf(__ldg(cf + 90 * C), x[7]*x[7]*x[15], f);
  f = fmaf(__ldg(cf + 91 * C), x[7]*x[8]*x[12], f);
  f = fmaf(__ldg(cf + 92 * C), x[7]*x[8]*x[14], f);
  f = fmaf(__ldg(cf + 93 * C), x[8]*x[8]*x[13], f);
  f = fmaf(__ldg(cf + 94 * C), x[8]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 95 * C), x[9]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 96 * C), x[9]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 97 * C), x[9]*x[10]*x[14], f);
  f = fmaf(__ldg(cf + 98 * C), x[9]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 99 * C), x[10]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 100 * C), x[10]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 101 * C), x[10]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 102 * C), x[11]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 103 * C), x[11]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 104 * C), x[12]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 105 * C), x[12]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 106 * C), x[12]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 107 * C), x[13]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 108 * C), x[13]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 109 * C), x[13]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 110 * C), x[13]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 111 * C), x[14]*x[14]*x[15], f);
  return f;
}

__device__ __forceinline__ void grad_LM3(const float* x, float w, const float* __restrict__ cf, int C, float* g) {
  { const float q = w * __ldg(cf + 0 * C);
    g[3] += q;
  }
  { const float q = w * __ldg(cf + 1 * C);
    g[0] = fmaf(q, x[3], g[0]);
    g[3] = fmaf(q, x[0], g[3]);
  }
  { const float q = w * __ldg(cf + 2 * C);
    g[1] = fmaf(q, x[4], g[1]);
    g[4] = fmaf(q, x[1], g[4]);
  }
  { const float q = w * __ldg(cf + 3 * C);
    g[2] = fmaf(q, x[7], g[2]);
    g[7] = fmaf(q, x[2], g[7]);
  }
  { const float q = w * __ldg(cf + 4 * C);
    g[3] = fmaf(q, x[6], g[3]);
    g[6] = fmaf(q, x[3], g[6]);
  }
  { const float q = w * __ldg(cf + 5 * C);
    g[3] = fmaf(q, x[8], g[3]);
    g[8] = fmaf(q, x[3], g[8]);
  }
  { const float q = w * __ldg(cf + 6 * C);
    g[4] = fmaf(q, x[9], g[4]);
    g[9] = fmaf(q, x[4], g[9]);
  }
  { const float q = w * __ldg(cf + 7 * C);
    g[4] = fmaf(q, x[11], g[4]);
    g[11] = fmaf(q, x[4], g[11]);
  }
  { const float q = w * __ldg(cf + 8 * C);
    g[5] = fmaf(q, x[10], g[5]);
    g[10] = fmaf(q, x[5], g[10]);
  }
  { const float q = w * __ldg(cf + 9 * C);
    g[6] = fmaf(q, x[13], g[6]);
    g[13] = fmaf(q, x[6], g[13]);
  }
  { const float q = w * __ldg(cf + 10 * C);
    g[7] = fmaf(q, x[12], g[7]);
    g[12] = fmaf(q, x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 11 * C);
    g[7] = fmaf(q, x[14], g[7]);
    g[14] = fmaf(q, x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 12 * C);
    g[8] = fmaf(q, x[13], g[8]);
    g[13] = fmaf(q, x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 13 * C);
    g[8] = fmaf(q, x[15], g[8]);
    g[15] = fmaf(q, x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 14 * C);
    g[0] = fmaf(q, x[0]*x[3], g[0]);
    g[0] = fmaf(q, x[0]*x[3], g[0]);
    g[3] = fmaf(q, x[0]*x[0], g[3]);
  }
  { const float q = w * __ldg(cf + 15 * C);
    g[0] = fmaf(q, x[1]*x[4], g[0]);
    g[1] = fmaf(q, x[0]*x[4], g[1]);
    g[4] = fmaf(q, x[0]*x[1], g[4]);
  }
  { const float q = w * __ldg(cf + 16 * C);
    g[0] = fmaf(q, x[2]*x[7], g[0]);
    g[2] = fmaf(q, x[0]*x[7], g[2]);
    g[7] = fmaf(q, x[0]*x[2], g[7]);
  }
  { const float q = w * __ldg(cf + 17 * C);
    g[0] = fmaf(q, x[3]*x[6], g[0]);
    g[3] = fmaf(q, x[0]*x[6], g[3]);
    g[6] = fmaf(q, x[0]*x[3], g[6]);
  }
  { const float q = w * __ldg(cf + 18 * C);
    g[0] = fmaf(q, x[3]*x[8], g[0]);
    g[3] = fmaf(q, x[0]*x[8], g[3]);
    g[8] = fmaf(q, x[0]*x[3], g[8]);
  }
  { const float q = w * __ldg(cf + 19 * C);
    g[0] = fmaf(q, x[4]*x[9], g[0]);
    g[4] = fmaf(q, x[0]*x[9], g[4]);
    g[9] = fmaf(q, x[0]*x[4], g[9]);
  }
  { const float q = w * __ldg(cf + 20 * C);
    g[0] = fmaf(q, x[4]*x[11], g[0]);
    g[4] = fmaf(q, x[0]*x[11], g[4]);
    g[11] = fmaf(q, x[0]*x[4], g[11]);
  }
  { const float q = w * __ldg(cf + 21 * C);
    g[0] = fmaf(q, x[5]*x[10], g[0]);
    g[5] = fmaf(q, x[0]*x[10], g[5]);
    g[10] = fmaf(q, x[0]*x[5], g[10]);
  }
  { const float q = w * __ldg(cf + 22 * C);
    g[0] = fmaf(q, x[6]*x[13], g[0]);
    g[6] = fmaf(q, x[0]*x[13], g[6]);
    g[13] = fmaf(q, x[0]*x[6], g[13]);
  }
  { const float q = w * __ldg(cf + 23 * C);
    g[0] = fmaf(q, x[7]*x[12], g[0]);
    g[7] = fmaf(q, x[0]*x[12], g[7]);
    g[12] = fmaf(q, x[0]*x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 24 * C);
    g[0] = fmaf(q, x[7]*x[14], g[0]);
    g[7] = fmaf(q, x[0]*x[14], g[7]);
    g[14] = fmaf(q, x[0]*x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 25 * C);
    g[0] = fmaf(q, x[8]*x[13], g[0]);
    g[8] = fmaf(q, x[0]*x[13], g[8]);
    g[13] = fmaf(q, x[0]*x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 26 * C);
    g[0] = fmaf(q, x[8]*x[15], g[0]);
    g[8] = fmaf(q, x[0]*x[15], g[8]);
    g[15] = fmaf(q, x[0]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 27 * C);
    g[1] = fmaf(q, x[1]*x[3], g[1]);
    g[1] = fmaf(q, x[1]*x[3], g[1]);
    g[3] = fmaf(q, x[1]*x[1], g[3]);
  }
  { const float q = w * __ldg(cf + 28 * C);
    g[1] = fmaf(q, x[1]*x[13], g[1]);
    g[1] = fmaf(q, x[1]*x[13], g[1]);
    g[13] = fmaf(q, x[1]*x[1], g[13]);
  }
  { const float q = w * __ldg(cf + 29 * C);
    g[1] = fmaf(q, x[1]*x[15], g[1]);
    g[1] = fmaf(q, x[1]*x[15], g[1]);
    g[15] = fmaf(q, x[1]*x[1], g[15]);
  }
  { const float q = w * __ldg(cf + 30 * C);
    g[1] = fmaf(q, x[2]*x[10], g[1]);
    g[2] = fmaf(q, x[1]*x[10], g[2]);
    g[10] = fmaf(q, x[1]*x[2], g[10]);
  }
  { const float q = w * __ldg(cf + 31 * C);
    g[1] = fmaf(q, x[3]*x[9], g[1]);
    g[3] = fmaf(q, x[1]*x[9], g[3]);
    g[9] = fmaf(q, x[1]*x[3], g[9]);
  }
  { const float q = w * __ldg(cf + 32 * C);
    g[1] = fmaf(q, x[3]*x[11], g[1]);
    g[3] = fmaf(q, x[1]*x[11], g[3]);
    g[11] = fmaf(q, x[1]*x[3], g[11]);
  }
  { const float q = w * __ldg(cf + 33 * C);
    g[1] = fmaf(q, x[4]*x[6], g[1]);
    g[4] = fmaf(q, x[1]*x[6], g[4]);
    g[6] = fmaf(q, x[1]*x[4], g[6]);
  }
  { const float q = w * __ldg(cf + 34 * C);
    g[1] = fmaf(q, x[5]*x[7], g[1]);
    g[5] = fmaf(q, x[1]*x[7], g[5]);
    g[7] = fmaf(q, x[1]*x[5], g[7]);
  }
  { const float q = w * __ldg(cf + 35 * C);
    g[1] = fmaf(q, x[9]*x[13], g[1]);
    g[9] = fmaf(q, x[1]*x[13], g[9]);
    g[13] = fmaf(q, x[1]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 36 * C);
    g[1] = fmaf(q, x[10]*x[12], g[1]);
    g[10] = fmaf(q, x[1]*x[12], g[10]);
    g[12] = fmaf(q, x[1]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 37 * C);
    g[1] = fmaf(q, x[11]*x[13], g[1]);
    g[11] = fmaf(q, x[1]*x[13], g[11]);
    g[13] = fmaf(q, x[1]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 38 * C);
    g[1] = fmaf(q, x[11]*x[15], g[1]);
    g[11] = fmaf(q, x[1]*x[15], g[11]);
    g[15] = fmaf(q, x[1]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 39 * C);
    g[2] = fmaf(q, x[2]*x[3], g[2]);
    g[2] = fmaf(q, x[2]*x[3], g[2]);
    g[3] = fmaf(q, x[2]*x[2], g[3]);
  }
  { const float q = w * __ldg(cf + 40 * C);
    g[2] = fmaf(q, x[2]*x[13], g[2]);
    g[2] = fmaf(q, x[2]*x[13], g[2]);
    g[13] = fmaf(q, x[2]*x[2], g[13]);
  }
  { const float q = w * __ldg(cf + 41 * C);
    g[2] = fmaf(q, x[3]*x[12], g[2]);
    g[3] = fmaf(q, x[2]*x[12], g[3]);
    g[12] = fmaf(q, x[2]*x[3], g[12]);
  }
  { const float q = w * __ldg(cf + 42 * C);
    g[2] = fmaf(q, x[3]*x[14], g[2]);
    g[3] = fmaf(q, x[2]*x[14], g[3]);
    g[14] = fmaf(q, x[2]*x[3], g[14]);
  }
  { const float q = w * __ldg(cf + 43 * C);
    g[2] = fmaf(q, x[4]*x[5], g[2]);
    g[4] = fmaf(q, x[2]*x[5], g[4]);
    g[5] = fmaf(q, x[2]*x[4], g[5]);
  }
  { const float q = w * __ldg(cf + 44 * C);
    g[2] = fmaf(q, x[6]*x[7], g[2]);
    g[6] = fmaf(q, x[2]*x[7], g[6]);
    g[7] = fmaf(q, x[2]*x[6], g[7]);
  }
  { const float q = w * __ldg(cf + 45 * C);
    g[2] = fmaf(q, x[7]*x[8], g[2]);
    g[7] = fmaf(q, x[2]*x[8], g[7]);
    g[8] = fmaf(q, x[2]*x[7], g[8]);
  }
  { const float q = w * __ldg(cf + 46 * C);
    g[2] = fmaf(q, x[9]*x[10], g[2]);
    g[9] = fmaf(q, x[2]*x[10], g[9]);
    g[10] = fmaf(q, x[2]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 47 * C);
    g[2] = fmaf(q, x[10]*x[11], g[2]);
    g[10] = fmaf(q, x[2]*x[11], g[10]);
    g[11] = fmaf(q, x[2]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 48 * C);
    g[2] = fmaf(q, x[12]*x[13], g[2]);
    g[12] = fmaf(q, x[2]*x[13], g[12]);
    g[13] = fmaf(q, x[2]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 49 * C);
    g[2] = fmaf(q, x[13]*x[14], g[2]);
    g[13] = fmaf(q, x[2]*x[14], g[13]);
    g[14] = fmaf(q, x[2]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 50 * C);
    g[2] = fmaf(q, x[14]*x[15], g[2]);
    g[14] = fmaf(q, x[2]*x[15], g[14]);
    g[15] = fmaf(q, x[2]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 51 * C);
    g[3] = fmaf(q, x[3]*x[3], g[3]);
    g[3] = fmaf(q, x[3]*x[3], g[3]);
    g[3] = fmaf(q, x[3]*x[3], g[3]);
  }
  { const float q = w * __ldg(cf + 52 * C);
    g[3] = fmaf(q, x[3]*x[13], g[3]);
    g[3] = fmaf(q, x[3]*x[13], g[3]);
    g[13] = fmaf(q, x[3]*x[3], g[13]);
  }
  { const float q = w * __ldg(cf + 53 * C);
    g[3] = fmaf(q, x[3]*x[15], g[3]);
    g[3] = fmaf(q, x[3]*x[15], g[3]);
    g[15] = fmaf(q, x[3]*x[3], g[15]);
  }
  { const float q = w * __ldg(cf + 54 * C);
    g[3] = fmaf(q, x[4]*x[4], g[3]);
    g[4] = fmaf(q, x[3]*x[4], g[4]);
    g[4] = fmaf(q, x[3]*x[4], g[4]);
  }
  { const float q = w * __ldg(cf + 55 * C);
    g[3] = fmaf(q, x[5]*x[5], g[3]);
    g[5] = fmaf(q, x[3]*x[5], g[5]);
    g[5] = fmaf(q, x[3]*x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 56 * C);
    g[3] = fmaf(q, x[6]*x[6], g[3]);
    g[6] = fmaf(q, x[3]*x[6], g[6]);
    g[6] = fmaf(q, x[3]*x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 57 * C);
    g[3] = fmaf(q, x[6]*x[8], g[3]);
    g[6] = fmaf(q, x[3]*x[8], g[6]);
    g[8] = fmaf(q, x[3]*x[6], g[8]);
  }
  { const float q = w * __ldg(cf + 58 * C);
    g[3] = fmaf(q, x[7]*x[7], g[3]);
    g[7] = fmaf(q, x[3]*x[7], g[7]);
    g[7] = fmaf(q, x[3]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 59 * C);
    g[3] = fmaf(q, x[8]*x[8], g[3]);
    g[8] = fmaf(q, x[3]*x[8], g[8]);
    g[8] = fmaf(q, x[3]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 60 * C);
    g[3] = fmaf(q, x[9]*x[9], g[3]);
    g[9] = fmaf(q, x[3]*x[9], g[9]);
    g[9] = fmaf(q, x[3]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 61 * C);
    g[3] = fmaf(q, x[9]*x[11], g[3]);
    g[9] = fmaf(q, x[3]*x[11], g[9]);
    g[11] = fmaf(q, x[3]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 62 * C);
    g[3] = fmaf(q, x[10]*x[10], g[3]);
    g[10] = fmaf(q, x[3]*x[10], g[10]);
    g[10] = fmaf(q, x[3]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 63 * C);
    g[3] = fmaf(q, x[11]*x[11], g[3]);
    g[11] = fmaf(q, x[3]*x[11], g[11]);
    g[11] = fmaf(q, x[3]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 64 * C);
    g[3] = fmaf(q, x[12]*x[12], g[3]);
    g[12] = fmaf(q, x[3]*x[12], g[12]);
    g[12] = fmaf(q, x[3]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 65 * C);
    g[3] = fmaf(q, x[12]*x[14], g[3]);
    g[12] = fmaf(q, x[3]*x[14], g[12]);
    g[14] = fmaf(q, x[3]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 66 * C);
    g[3] = fmaf(q, x[13]*x[13], g[3]);
    g[13] = fmaf(q, x[3]*x[13], g[13]);
    g[13] = fmaf(q, x[3]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 67 * C);
    g[3] = fmaf(q, x[13]*x[15], g[3]);
    g[13] = fmaf(q, x[3]*x[15], g[13]);
    g[15] = fmaf(q, x[3]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 68 * C);
    g[3] = fmaf(q, x[14]*x[14], g[3]);
    g[14] = fmaf(q, x[3]*x[14], g[14]);
    g[14] = fmaf(q, x[3]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 69 * C);
    g[3] = fmaf(q, x[15]*x[15], g[3]);
    g[15] = fmaf(q, x[3]*x[15], g[15]);
    g[15] = fmaf(q, x[3]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 70 * C);
    g[4] = fmaf(q, x[4]*x[13], g[4]);
    g[4] = fmaf(q, x[4]*x[13], g[4]);
    g[13] = fmaf(q, x[4]*x[4], g[13]);
  }
  { const float q = w * __ldg(cf + 71 * C);
    g[4] = fmaf(q, x[4]*x[15], g[4]);
    g[4] = fmaf(q, x[4]*x[15], g[4]);
    g[15] = fmaf(q, x[4]*x[4], g[15]);
  }
  { const float q = w * __ldg(cf + 72 * C);
    g[4] = fmaf(q, x[5]*x[12], g[4]);
    g[5] = fmaf(q, x[4]*x[12], g[5]);
    g[12] = fmaf(q, x[4]*x[5], g[12]);
  }
  { const float q = w * __ldg(cf + 73 * C);
    g[4] = fmaf(q, x[5]*x[14], g[4]);
    g[5] = fmaf(q, x[4]*x[14], g[5]);
    g[14] = fmaf(q, x[4]*x[5], g[14]);
  }
  { const float q = w * __ldg(cf + 74 * C);
    g[4] = fmaf(q, x[6]*x[9], g[4]);
    g[6] = fmaf(q, x[4]*x[9], g[6]);
    g[9] = fmaf(q, x[4]*x[6], g[9]);
  }
  { const float q = w * __ldg(cf + 75 * C);
    g[4] = fmaf(q, x[6]*x[11], g[4]);
    g[6] = fmaf(q, x[4]*x[11], g[6]);
    g[11] = fmaf(q, x[4]*x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 76 * C);
    g[4] = fmaf(q, x[7]*x[10], g[4]);
    g[7] = fmaf(q, x[4]*x[10], g[7]);
    g[10] = fmaf(q, x[4]*x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 77 * C);
    g[4] = fmaf(q, x[8]*x[9], g[4]);
    g[8] = fmaf(q, x[4]*x[9], g[8]);
    g[9] = fmaf(q, x[4]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 78 * C);
    g[5] = fmaf(q, x[5]*x[13], g[5]);
    g[5] = fmaf(q, x[5]*x[13], g[5]);
    g[13] = fmaf(q, x[5]*x[5], g[13]);
  }
  { const float q = w * __ldg(cf + 79 * C);
    g[5] = fmaf(q, x[5]*x[15], g[5]);
    g[5] = fmaf(q, x[5]*x[15], g[5]);
    g[15] = fmaf(q, x[5]*x[5], g[15]);
  }
  { const float q = w * __ldg(cf + 80 * C);
    g[5] = fmaf(q, x[6]*x[10], g[5]);
    g[6] = fmaf(q, x[5]*x[10], g[6]);
    g[10] = fmaf(q, x[5]*x[6], g[10]);
  }
  { const float q = w * __ldg(cf + 81 * C);
    g[5] = fmaf(q, x[7]*x[9], g[5]);
    g[7] = fmaf(q, x[5]*x[9], g[7]);
    g[9] = fmaf(q, x[5]*x[7], g[9]);
  }
  { const float q = w * __ldg(cf + 82 * C);
    g[5] = fmaf(q, x[7]*x[11], g[5]);
    g[7] = fmaf(q, x[5]*x[11], g[7]);
    g[11] = fmaf(q, x[5]*x[7], g[11]);
  }
  { const float q = w * __ldg(cf + 83 * C);
    g[5] = fmaf(q, x[8]*x[10], g[5]);
    g[8] = fmaf(q, x[5]*x[10], g[8]);
    g[10] = fmaf(q, x[5]*x[8], g[10]);
  }
  { const float q = w * __ldg(cf + 84 * C);
    g[6] = fmaf(q, x[6]*x[13], g[6]);
    g[6] = fmaf(q, x[6]*x[13], g[6]);
    g[13] = fmaf(q, x[6]*x[6], g[13]);
  }
  { const float q = w * __ldg(cf + 85 * C);
    g[6] = fmaf(q, x[7]*x[12], g[6]);
    g[7] = fmaf(q, x[6]*x[12], g[7]);
    g[12] = fmaf(q, x[6]*x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 86 * C);
    g[6] = fmaf(q, x[7]*x[14], g[6]);
    g[7] = fmaf(q, x[6]*x[14], g[7]);
    g[14] = fmaf(q, x[6]*x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 87 * C);
    g[6] = fmaf(q, x[8]*x[13], g[6]);
    g[8] = fmaf(q, x[6]*x[13], g[8]);
    g[13] = fmaf(q, x[6]*x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 88 * C);
    g[6] = fmaf(q, x[8]*x[15], g[6]);
    g[8] = fmaf(q, x[6]*x[15], g[8]);
    g[15] = fmaf(q, x[6]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 89 * C);
    g[7] = fmaf(q, x[7]*x[13], g[7]);
    g[7] = fmaf(q, x[7]*x[13], g[7]);
    g[13] = fmaf(q, x[7]*x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 90 * C);
    g[7] = fmaf(q, x[7]*x[15], g[7]);
    g[7] = fmaf(q, x[7]*x[15], g[7]);
    g[15] = fmaf(q, x[7]*x[7], g[15]);
  }
  { const float q = w * __ldg(cf + 91 * C);
    g[7] = fmaf(q, x[8]*x[12], g[7]);
    g[8] = fmaf(q, x[7]*x[12], g[8]);
    g[12] = fmaf(q, x[7]*x[8], g[12]);
  }
  { const float q = w * __ldg(cf + 92 * C);
    g[7] = fmaf(q, x[8]*x[14], g[7]);
    g[8] = fmaf(q, x[7]*x[14], g[8]);
    g[14] = fmaf(q, x[7]*x[8], g[14]);
  }
  { const float q = w * __ldg(cf + 93 * C);
    g[8] = fmaf(q, x[8]*x[13], g[8]);
    g[8] = fmaf(q, x[8]*x[13], g[8]);
    g[13] = fmaf(q, x[8]*x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 94 * C);
    g[8] = fmaf(q, x[8]*x[15], g[8]);
    g[8] = fmaf(q, x[8]*x[15], g[8]);
    g[15] = fmaf(q, x[8]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 95 * C);
    g[9] = fmaf(q, x[9]*x[13], g[9]);
    g[9] = fmaf(q, x[9]*x[13], g[9]);
    g[13] = fmaf(q, x[9]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 96 * C);
    g[9] = fmaf(q, x[10]*x[12], g[9]);
    g[10] = fmaf(q, x[9]*x[12], g[10]);
    g[12] = fmaf(q, x[9]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 97 * C);
    g[9] = fmaf(q, x[10]*x[14], g[9]);
    g[10] = fmaf(q, x[9]*x[14], g[10]);
    g[14] = fmaf(q, x[9]*x[10], g[14]);
  }
  { const float q = w * __ldg(cf + 98 * C);
    g[9] = fmaf(q, x[11]*x[13], g[9]);
    g[11] = fmaf(q, x[9]*x[13], g[11]);
    g[13] = fmaf(q, x[9]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 99 * C);
    g[10] = fmaf(q, x[10]*x[13], g[10]);
    g[10] = fmaf(q, x[10]*x[13], g[10]);
    g[13] = fmaf(q, x[10]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 100 * C);
    g[10] = fmaf(q, x[10]*x[15], g[10]);
    g[10] = fmaf(q, x[10]*x[15], g[10]);
    g[15] = fmaf(q, x[10]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 101 * C);
    g[10] = fmaf(q, x[11]*x[12], g[10]);
    g[11] = fmaf(q, x[10]*x[12], g[11]);
    g[12] = fmaf(q, x[10]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 102 * C);
    g[11] = fmaf(q, x[11]*x[13], g[11]);
    g[11] = fmaf(q, x[11]*x[13], g[11]);
    g[13] = fmaf(q, x[11]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 103 * C);
    g[11] = fmaf(q, x[11]*x[15], g[11]);
    g[11] = fmaf(q, x[11]*x[15], g[11]);
    g[15] = fmaf(q, x[11]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 104 * C);
    g[12] = fmaf(q, x[12]*x[13], g[12]);
    g[12] = fmaf(q, x[12]*x[13], g[12]);
    g[13] = fmaf(q, x[12]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 105 * C);
    g[12] = fmaf(q, x[13]*x[14], g[12]);
    g[13] = fmaf(q, x[12]*x[14], g[13]);
    g[14] = fmaf(q, x[12]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 106 * C);
    g[12] = fmaf(q, x[14]*x[15], g[12]);
    g[14] = fmaf(q, x[12]*x[15], g[14]);
    g[15] = fmaf(q, x[12]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 107 * C);
    g[13] = fmaf(q, x[13]*x[13], g[13]);
    g[13] = fmaf(q, x[13]*x[13], g[13]);
    g[13] = fmaf(q, x[13]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 108 * C);
    g[13] = fmaf(q, x[13]*x[15], g[13]);
    g[13] = fmaf(q, x[13]*x[15], g[13]);
    g[15] = fmaf(q, x[13]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 109 * C);
    g[13] = fmaf(q, x[14]*x[14], g[13]);
    g[14] = fmaf(q, x[13]*x[14], g[14]);
    g[14] = fmaf(q, x[13]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 110 * C);
    g[13] = fmaf(q, x[15]*x[15], g[13]);
    g[15] = fmaf(q, x[13]*x[15], g[15]);
    g[15] = fmaf(q, x[13]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 111 * C);
    g[14] = fmaf(q, x[14]*x[15], g[14]);
    g[14] = fmaf(q, x[14]*x[15], g[14]);
    g[15] = fmaf(q, x[14]*x[14], g[15]);
  }
}

__device__ __forceinline__ float value_LM4(const float* x, const float* __restrict__ cf, int C) {
  float f = 0.0f;
  f = fmaf(__ldg(cf + 0 * C), x[4], f);
  f = fmaf(__ldg(cf + 1 * C), x[0]*x[4], f);
  f = fmaf(__ldg(cf + 2 * C), x[1]*x[3], f);
  f = fmaf(__ldg(cf + 3 * C), x[1]*x[13], f);
  f = fmaf(__ldg(cf + 4 * C), x[1]*x[15], f);
  f = fmaf(__ldg(cf + 5 * C), x[2]*x[10], f);
  f = fmaf(__ldg(cf + 6 * C), x[3]*x[9], f);
  f = fmaf(__ldg(cf + 7 * C), x[3]*x[11], f);
  f = fmaf(__ldg(cf + 8 * C), x[4]*x[6], f);
  f = fmaf(__ldg(cf + 9 * C), x[5]*x[7], f);
  f = fmaf(__ldg(cf + 10 * C), x[9]*x[13], f);
  f = fmaf(__ldg(cf + 11 * C), x[10]*x[12], f);
  f = fmaf(__ldg(cf + 12 * C), x[11]*x[13], f);
  f = fmaf(__ldg(cf + 13 * C), x[11]*x[15], f);
  f = fmaf(__ldg(cf + 14 * C), x[0]*x[0]*x[4], f);
  f = fmaf(__ldg(cf + 15 * C), x[0]*x[1]*x[3], f);
  f = fmaf(__ldg(cf + 16 * C), x[0]*x[1]*x[13], f);
  f = fmaf(__ldg(cf + 17 * C), x[0]*x[1]*x[15], f);
  f = fmaf(__ldg(cf + 18 * C), x[0]*x[2]*x[10], f);
  f = fmaf(__ldg(cf + 19 * C), x[0]*x[3]*x[9], f);
  f = fmaf(__ldg(cf + 20 * C), x[0]*x[3]*x[11], f);
  f = fmaf(__ldg(cf + 21 * C), x[0]*x[4]*x[6], f);
  f = fmaf(__ldg(cf + 22 * C), x[0]*x[5]*x[7], f);
  f = fmaf(__ldg(cf + 23 * C), x[0]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 24 * C), x[0]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 25 * C), x[0]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 26 * C), x[0]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 27 * C), x[1]*x[1]*x[4], f);
  f = fmaf(__ldg(cf + 28 * C), x[1]*x[2]*x[7], f);
  f = fmaf(__ldg(cf + 29 * C), x[1]*x[3]*x[6], f);
  f = fmaf(__ldg(cf + 30 * C), x[1]*x[4]*x[9], f);
  f = fmaf(__ldg(cf + 31 * C), x[1]*x[4]*x[11], f);
  f = fmaf(__ldg(cf + 32 * C), x[1]*x[5]*x[10], f);
  f = fmaf(__ldg(cf + 33 * C), x[1]*x[6]*x[13], f);
  f = fmaf(__ldg(cf + 34 * C), x[1]*x[6]*x[15], f);
  f = fmaf(__ldg(cf + 35 * C), x[1]*x[7]*x[12], f);
  f = fmaf(__ldg(cf + 36 * C), x[1]*x[7]*x[14], f);
  f = fmaf(__ldg(cf + 37 * C), x[1]*x[8]*x[13], f);
  f = fmaf(__ldg(cf + 38 * C), x[1]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 39 * C), x[2]*x[2]*x[4], f);
  f = fmaf(__ldg(cf + 40 * C), x[2]*x[3]*x[5], f);
  f = fmaf(__ldg(cf + 41 * C), x[2]*x[4]*x[12], f);
  f = fmaf(__ldg(cf + 42 * C), x[2]*x[5]*x[13], f);
  f = fmaf(__ldg(cf + 43 * C), x[2]*x[5]*x[15], f);
  f = fmaf(__ldg(cf + 44 * C), x[2]*x[6]*x[10], f);
  f = fmaf(__ldg(cf + 45 * C), x[2]*x[7]*x[9], f);
  f = fmaf(__ldg(cf + 46 * C), x[2]*x[7]*x[11], f);
  f = fmaf(__ldg(cf + 47 * C), x[3]*x[3]*x[4], f);
  f = fmaf(__ldg(cf + 48 * C), x[3]*x[4]*x[13], f);
  f = fmaf(__ldg(cf + 49 * C), x[3]*x[4]*x[15], f);
  f = fmaf(__ldg(cf + 50 * C), x[3]*x[5]*x[12], f);
  f = fmaf(__ldg(cf + 51 * C), x[3]*x[5]*x[14], f);
  f = fmaf(__ldg(cf + 52 * C), x[3]*x[6]*x[9], f);
  f = fmaf(__ldg(cf + 53 * C), x[3]*x[6]*x[11], f);
  f = fmaf(__ldg(cf + 54 * C), x[3]*x[7]*x[10], f);
  f = fmaf(__ldg(cf + 55 * C), x[3]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 56 * C), x[3]*x[8]*x[11], f);
  f = fmaf(__ldg(cf + 57 * C), x[4]*x[4]*x[4], f);
  f = fmaf(__ldg(cf + 58 * C), x[4]*x[5]*x[5], f);
  f = fmaf(__ldg(cf + 59 * C), x[4]*x[6]*x[6], f);
  f = fmaf(__ldg(cf + 60 * C), x[4]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 61 * C), x[4]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 62 * C), x[4]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 63 * C), x[4]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 64 * C), x[4]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 65 * C), x[4]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 66 * C), x[4]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 67 * C), x[4]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 68 * C), x[4]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 69 * C), x[4]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 70 * C), x[4]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 71 * C), x[5]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 72 * C), x[5]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 73 * C), x[5]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 74 * C), x[5]*x[12]*x[15], f);
  f = fmaf(__ldg(cf + 75 * C), x[5]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 76 * C), x[5]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 77 * C), x[6]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 78 * C), x[6]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 79 * C), x[6]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 80 * C), x[6]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 81 * C), x[7]*x[9]*x[12], f);
  f = fmaf(__ldg(cf + 82 * C), x[7]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 83 * C), x[7]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 84 * C), x[7]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 85 * C), x[7]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 86 * C), x[7]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 87 * C), x[8]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 88 * C), x[8]*x[10]*x[14], f);
  f = fmaf(__ldg(cf + 89 * C), x[8]*x[11]*x[15], f);
  return f;
}

__device__ __forceinline__ void grad_LM4(const float* x, float w, const float* __restrict__ cf, int C, float* g) {
  { const float q = w * __ldg(cf + 0 * C);
    g[4] += q;
  }
  { const float q = w * __ldg(cf + 1 * C);
    g[0] = fmaf(q, x[4], g[0]);
    g[4] = fmaf(q, x[0], g[4]);
  }
  { const float q = w * __ldg(cf + 2 * C);
    g[1] = fmaf(q, x[3], g[1]);
    g[3] = fmaf(q, x[1], g[3]);
  }
  { const float q = w * __ldg(cf + 3 * C);
    g[1] = fmaf(q, x[13], g[1]);
    g[13] = fmaf(q, x[1], g[13]);
  }
  { const float q = w * __ldg(cf + 4 * C);
    g[1] = fmaf(q, x[15], g[1]);
    g[15] = fmaf(q, x[1], g[15]);
  }
  { const float q = w * __ldg(cf + 5 * C);
    g[2] = fmaf(q, x[10], g[2]);
    g[10] = fmaf(q, x[2], g[10]);
  }
  { const float q = w * __ldg(cf + 6 * C);
    g[3] = fmaf(q, x[9], g[3]);
    g[9] = fmaf(q, x[3], g[9]);
  }
  { const float q = w * __ldg(cf + 7 * C);
    g[3] = fmaf(q, x[11], g[3]);
    g[11] = fmaf(q, x[3], g[11]);
  }
  { const float q = w * __ldg(cf + 8 * C);
    g[4] = fmaf(q, x[6], g[4]);
    g[6] = fmaf(q, x[4], g[6]);
  }
  { const float q = w * __ldg(cf + 9 * C);
    g[5] = fmaf(q, x[7], g[5]);
    g[7] = fmaf(q, x[5], g[7]);
  }
  { const float q = w * __ldg(cf + 10 * C);
    g[9] = fmaf(q, x[13], g[9]);
    g[13] = fmaf(q, x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 11 * C);
    g[10] = fmaf(q, x[12], g[10]);
    g[12] = fmaf(q, x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 12 * C);
    g[11] = fmaf(q, x[13], g[11]);
    g[13] = fmaf(q, x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 13 * C);
    g[11] = fmaf(q, x[15], g[11]);
    g[15] = fmaf(q, x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 14 * C);
    g[0] = fmaf(q, x[0]*x[4], g[0]);
    g[0] = fmaf(q, x[0]*x[4], g[0]);
    g[4] = fmaf(q, x[0]*x[0], g[4]);
  }
  { const float q = w * __ldg(cf + 15 * C);
    g[0] = fmaf(q, x[1]*x[3], g[0]);
    g[1] = fmaf(q, x[0]*x[3], g[1]);
    g[3] = fmaf(q, x[0]*x[1], g[3]);
  }
  { const float q = w * __ldg(cf + 16 * C);
    g[0] = fmaf(q, x[1]*x[13], g[0]);
    g[1] = fmaf(q, x[0]*x[13], g[1]);
    g[13] = fmaf(q, x[0]*x[1], g[13]);
  }
  { const float q = w * __ldg(cf + 17 * C);
    g[0] = fmaf(q, x[1]*x[15], g[0]);
    g[1] = fmaf(q, x[0]*x[15], g[1]);
    g[15] = fmaf(q, x[0]*x[1], g[15]);
  }
  { const float q = w * __ldg(cf + 18 * C);
    g[0] = fmaf(q, x[2]*x[10], g[0]);
    g[2] = fmaf(q, x[0]*x[10], g[2]);
    g[10] = fmaf(q, x[0]*x[2], g[10]);
  }
  { const float q = w * __ldg(cf + 19 * C);
    g[0] = fmaf(q, x[3]*x[9], g[0]);
    g[3] = fmaf(q, x[0]*x[9], g[3]);
    g[9] = fmaf(q, x[0]*x[3], g[9]);
  }
  { const float q = w * __ldg(cf + 20 * C);
    g[0] = fmaf(q, x[3]*x[11], g[0]);
    g[3] = fmaf(q, x[0]*x[11], g[3]);
    g[11] = fmaf(q, x[0]*x[3], g[11]);
  }
  { const float q = w * __ldg(cf + 21 * C);
    g[0] = fmaf(q, x[4]*x[6], g[0]);
    g[4] = fmaf(q, x[0]*x[6], g[4]);
    g[6] = fmaf(q, x[0]*x[4], g[6]);
  }
  { const float q = w * __ldg(cf + 22 * C);
    g[0] = fmaf(q, x[5]*x[7], g[0]);
    g[5] = fmaf(q, x[0]*x[7], g[5]);
    g[7] = fmaf(q, x[0]*x[5], g[7]);
  }
  { const float q = w * __ldg(cf + 23 * C);
    g[0] = fmaf(q, x[9]*x[13], g[0]);
    g[9] = fmaf(q, x[0]*x[13], g[9]);
    g[13] = fmaf(q, x[0]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 24 * C);
    g[0] = fmaf(q, x[10]*x[12], g[0]);
    g[10] = fmaf(q, x[0]*x[12], g[10]);
    g[12] = fmaf(q, x[0]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 25 * C);
    g[0] = fmaf(q, x[11]*x[13], g[0]);
    g[11] = fmaf(q, x[0]*x[13], g[11]);
    g[13] = fmaf(q, x[0]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 26 * C);
    g[0] = fmaf(q, x[11]*x[15], g[0]);
    g[11] = fmaf(q, x[0]*x[15], g[11]);
    g[15] = fmaf(q, x[0]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 27 * C);
    g[1] = fmaf(q, x[1]*x[4], g[1]);
    g[1] = fmaf(q, x[1]*x[4], g[1]);
    g[4] = fmaf(q, x[1]*x[1], g[4]);
  }
  { const float q = w * __ldg(cf + 28 * C);
    g[1] = fmaf(q, x[2]*x[7], g[1]);
    g[2] = fmaf(q, x[1]*x[7], g[2]);
    g[7] = fmaf(q, x[1]*x[2], g[7]);
  }
  { const float q = w * __ldg(cf + 29 * C);
    g[1] = fmaf(q, x[3]*x[6], g[1]);
    g[3] = fmaf(q, x[1]*x[6], g[3]);
    g[6] = fmaf(q, x[1]*x[3], g[6]);
  }
  { const float q = w * __ldg(cf + 30 * C);
    g[1] = fmaf(q, x[4]*x[9], g[1]);
    g[4] = fmaf(q, x[1]*x[9], g[4]);
    g[9] = fmaf(q, x[1]*x[4], g[9]);
  }
  { const float q = w * __ldg(cf + 31 * C);
    g[1] = fmaf(q, x[4]*x[11], g[1]);
    g[4] = fmaf(q, x[1]*x[11], g[4]);
    g[11] = fmaf(q, x[1]*x[4], g[11]);
  }
  { const float q = w * __ldg(cf + 32 * C);
    g[1] = fmaf(q, x[5]*x[10], g[1]);
    g[5] = fmaf(q, x[1]*x[10], g[5]);
    g[10] = fmaf(q, x[1]*x[5], g[10]);
  }
  { const float q = w * __ldg(cf + 33 * C);
    g[1] = fmaf(q, x[6]*x[13], g[1]);
    g[6] = fmaf(q, x[1]*x[13], g[6]);
    g[13] = fmaf(q, x[1]*x[6], g[13]);
  }
  { const float q = w * __ldg(cf + 34 * C);
    g[1] = fmaf(q, x[6]*x[15], g[1]);
    g[6] = fmaf(q, x[1]*x[15], g[6]);
    g[15] = fmaf(q, x[1]*x[6], g[15]);
  }
  { const float q = w * __ldg(cf + 35 * C);
    g[1] = fmaf(q, x[7]*x[12], g[1]);
    g[7] = fmaf(q, x[1]*x[12], g[7]);
    g[12] = fmaf(q, x[1]*x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 36 * C);
    g[1] = fmaf(q, x[7]*x[14], g[1]);
    g[7] = fmaf(q, x[1]*x[14], g[7]);
    g[14] = fmaf(q, x[1]*x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 37 * C);
    g[1] = fmaf(q, x[8]*x[13], g[1]);
    g[8] = fmaf(q, x[1]*x[13], g[8]);
    g[13] = fmaf(q, x[1]*x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 38 * C);
    g[1] = fmaf(q, x[8]*x[15], g[1]);
    g[8] = fmaf(q, x[1]*x[15], g[8]);
    g[15] = fmaf(q, x[1]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 39 * C);
    g[2] = fmaf(q, x[2]*x[4], g[2]);
    g[2] = fmaf(q, x[2]*x[4], g[2]);
    g[4] = fmaf(q, x[2]*x[2], g[4]);
  }
  { const float q = w * __ldg(cf + 40 * C);
    g[2] = fmaf(q, x[3]*x[5], g[2]);
    g[3] = fmaf(q, x[2]*x[5], g[3]);
    g[5] = fmaf(q, x[2]*x[3], g[5]);
  }
  { const float q = w * __ldg(cf + 41 * C);
    g[2] = fmaf(q, x[4]*x[12], g[2]);
    g[4] = fmaf(q, x[2]*x[12], g[4]);
    g[12] = fmaf(q, x[2]*x[4], g[12]);
  }
  { const float q = w * __ldg(cf + 42 * C);
    g[2] = fmaf(q, x[5]*x[13], g[2]);
    g[5] = fmaf(q, x[2]*x[13], g[5]);
    g[13] = fmaf(q, x[2]*x[5], g[13]);
  }
  { const float q = w * __ldg(cf + 43 * C);
    g[2] = fmaf(q, x[5]*x[15], g[2]);
    g[5] = fmaf(q, x[2]*x[15], g[5]);
    g[15] = fmaf(q, x[2]*x[5], g[15]);
  }
  { const float q = w * __ldg(cf + 44 * C);
    g[2] = fmaf(q, x[6]*x[10], g[2]);
    g[6] = fmaf(q, x[2]*x[10], g[6]);
    g[10] = fmaf(q, x[2]*x[6], g[10]);
  }
  { const float q = w * __ldg(cf + 45 * C);
    g[2] = fmaf(q, x[7]*x[9], g[2]);
    g[7] = fmaf(q, x[2]*x[9], g[7]);
    g[9] = fmaf(q, x[2]*x[7], g[9]);
  }
  { const float q = w * __ldg(cf + 46 * C);
    g[2] = fmaf(q, x[7]*x[11], g[2]);
    g[7] = fmaf(q, x[2]*x[11], g[7]);
    g[11] = fmaf(q, x[2]*x[7], g[11]);
  }
  { const float q = w * __ldg(cf + 47 * C);
    g[3] = fmaf(q, x[3]*x[4], g[3]);
    g[3] = fmaf(q, x[3]*x[4], g[3]);
    g[4] = fmaf(q, x[3]*x[3], g[4]);
  }
  { const float q = w * __ldg(cf + 48 * C);
    g[3] = fmaf(q, x[4]*x[13], g[3]);
    g[4] = fmaf(q, x[3]*x[13], g[4]);
    g[13] = fmaf(q, x[3]*x[4], g[13]);
  }
  { const float q = w * __ldg(cf + 49 * C);
    g[3] = fmaf(q, x[4]*x[15], g[3]);
    g[4] = fmaf(q, x[3]*x[15], g[4]);
    g[15] = fmaf(q, x[3]*x[4], g[15]);
  }
  { const float q = w * __ldg(cf + 50 * C);
    g[3] = fmaf(q, x[5]*x[12], g[3]);
    g[5] = fmaf(q, x[3]*x[12], g[5]);
    g[12] = fmaf(q, x[3]*x[5], g[12]);
  }
  { const float q = w * __ldg(cf + 51 * C);
    g[3] = fmaf(q, x[5]*x[14], g[3]);
    g[5] = fmaf(q, x[3]*x[14], g[5]);
    g[14] = fmaf(q, x[3]*x[5], g[14]);
  }
  { const float q = w * __ldg(cf + 52 * C);
    g[3] = fmaf(q, x[6]*x[9], g[3]);
    g[6] = fmaf(q, x[3]*x[9], g[6]);
    g[9] = fmaf(q, x[3]*x[6], g[9]);
  }
  { const float q = w * __ldg(cf + 53 * C);
    g[3] = fmaf(q, x[6]*x[11], g[3]);
    g[6] = fmaf(q, x[3]*x[11], g[6]);
    g[11] = fmaf(q, x[3]*x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 54 * C);
    g[3] = fmaf(q, x[7]*x[10], g[3]);
    g[7] = fmaf(q, x[3]*x[10], g[7]);
    g[10] = fmaf(q, x[3]*x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 55 * C);
    g[3] = fmaf(q, x[8]*x[9], g[3]);
    g[8] = fmaf(q, x[3]*x[9], g[8]);
    g[9] = fmaf(q, x[3]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 56 * C);
    g[3] = fmaf(q, x[8]*x[11], g[3]);
    g[8] = fmaf(q, x[3]*x[11], g[8]);
    g[11] = fmaf(q, x[3]*x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 57 * C);
    g[4] = fmaf(q, x[4]*x[4], g[4]);
    g[4] = fmaf(q, x[4]*x[4], g[4]);
    g[4] = fmaf(q, x[4]*x[4], g[4]);
  }
  { const float q = w * __ldg(cf + 58 * C);
    g[4] = fmaf(q, x[5]*x[5], g[4]);
    g[5] = fmaf(q, x[4]*x[5], g[5]);
    g[5] = fmaf(q, x[4]*x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 59 * C);
    g[4] = fmaf(q, x[6]*x[6], g[4]);
    g[6] = fmaf(q, x[4]*x[6], g[6]);
    g[6] = fmaf(q, x[4]*x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 60 * C);
    g[4] = fmaf(q, x[7]*x[7], g[4]);
    g[7] = fmaf(q, x[4]*x[7], g[7]);
    g[7] = fmaf(q, x[4]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 61 * C);
    g[4] = fmaf(q, x[8]*x[8], g[4]);
    g[8] = fmaf(q, x[4]*x[8], g[8]);
    g[8] = fmaf(q, x[4]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 62 * C);
    g[4] = fmaf(q, x[9]*x[9], g[4]);
    g[9] = fmaf(q, x[4]*x[9], g[9]);
    g[9] = fmaf(q, x[4]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 63 * C);
    g[4] = fmaf(q, x[9]*x[11], g[4]);
    g[9] = fmaf(q, x[4]*x[11], g[9]);
    g[11] = fmaf(q, x[4]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 64 * C);
    g[4] = fmaf(q, x[10]*x[10], g[4]);
    g[10] = fmaf(q, x[4]*x[10], g[10]);
    g[10] = fmaf(q, x[4]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 65 * C);
    g[4] = fmaf(q, x[11]*x[11], g[4]);
    g[11] = fmaf(q, x[4]*x[11], g[11]);
    g[11] = fmaf(q, x[4]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 66 * C);
    g[4] = fmaf(q, x[12]*x[12], g[4]);
    g[12] = fmaf(q, x[4]*x[12], g[12]);
    g[12] = fmaf(q, x[4]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 67 * C);
    g[4] = fmaf(q, x[13]*x[13], g[4]);
    g[13] = fmaf(q, x[4]*x[13], g[13]);
    g[13] = fmaf(q, x[4]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 68 * C);
    g[4] = fmaf(q, x[13]*x[15], g[4]);
    g[13] = fmaf(q, x[4]*x[15], g[13]);
    g[15] = fmaf(q, x[4]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 69 * C);
    g[4] = fmaf(q, x[14]*x[14], g[4]);
    g[14] = fmaf(q, x[4]*x[14], g[14]);
    g[14] = fmaf(q, x[4]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 70 * C);
    g[4] = fmaf(q, x[15]*x[15], g[4]);
    g[15] = fmaf(q, x[4]*x[15], g[15]);
    g[15] = fmaf(q, x[4]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 71 * C);
    g[5] = fmaf(q, x[9]*x[10], g[5]);
    g[9] = fmaf(q, x[5]*x[10], g[9]);
    g[10] = fmaf(q, x[5]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 72 * C);
    g[5] = fmaf(q, x[10]*x[11], g[5]);
    g[10] = fmaf(q, x[5]*x[11], g[10]);
    g[11] = fmaf(q, x[5]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 73 * C);
    g[5] = fmaf(q, x[12]*x[13], g[5]);
    g[12] = fmaf(q, x[5]*x[13], g[12]);
    g[13] = fmaf(q, x[5]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 74 * C);
    g[5] = fmaf(q, x[12]*x[15], g[5]);
    g[12] = fmaf(q, x[5]*x[15], g[12]);
    g[15] = fmaf(q, x[5]*x[12], g[15]);
  }
  { const float q = w * __ldg(cf + 75 * C);
    g[5] = fmaf(q, x[13]*x[14], g[5]);
    g[13] = fmaf(q, x[5]*x[14], g[13]);
    g[14] = fmaf(q, x[5]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 76 * C);
    g[5] = fmaf(q, x[14]*x[15], g[5]);
    g[14] = fmaf(q, x[5]*x[15], g[14]);
    g[15] = fmaf(q, x[5]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 77 * C);
    g[6] = fmaf(q, x[9]*x[13], g[6]);
    g[9] = fmaf(q, x[6]*x[13], g[9]);
    g[13] = fmaf(q, x[6]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 78 * C);
    g[6] = fmaf(q, x[10]*x[12], g[6]);
    g[10] = fmaf(q, x[6]*x[12], g[10]);
    g[12] = fmaf(q, x[6]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 79 * C);
    g[6] = fmaf(q, x[11]*x[13], g[6]);
    g[11] = fmaf(q, x[6]*x[13], g[11]);
    g[13] = fmaf(q, x[6]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 80 * C);
    g[6] = fmaf(q, x[11]*x[15], g[6]);
    g[11] = fmaf(q, x[6]*x[15], g[11]);
    g[15] = fmaf(q, x[6]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 81 * C);
    g[7] = fmaf(q, x[9]*x[12], g[7]);
    g[9] = fmaf(q, x[7]*x[12], g[9]);
    g[12] = fmaf(q, x[7]*x[9], g[12]);
  }
  { const float q = w * __ldg(cf + 82 * C);
    g[7] = fmaf(q, x[9]*x[14], g[7]);
    g[9] = fmaf(q, x[7]*x[14], g[9]);
    g[14] = fmaf(q, x[7]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 83 * C);
    g[7] = fmaf(q, x[10]*x[13], g[7]);
    g[10] = fmaf(q, x[7]*x[13], g[10]);
    g[13] = fmaf(q, x[7]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 84 * C);
    g[7] = fmaf(q, x[10]*x[15], g[7]);
    g[10] = fmaf(q, x[7]*x[15], g[10]);
    g[15] = fmaf(q, x[7]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 85 * C);
    g[7] = fmaf(q, x[11]*x[12], g[7]);
    g[11] = fmaf(q, x[7]*x[12], g[11]);
    g[12] = fmaf(q, x[7]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 86 * C);
    g[7] = fmaf(q, x[11]*x[14], g[7]);
    g[11] = fmaf(q, x[7]*x[14], g[11]);
    g[14] = fmaf(q, x[7]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 87 * C);
    g[8] = fmaf(q, x[9]*x[13], g[8]);
    g[9] = fmaf(q, x[8]*x[13], g[9]);
    g[13] = fmaf(q, x[8]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 88 * C);
    g[8] = fmaf(q, x[10]*x[14], g[8]);
    g[10] = fmaf(q, x[8]*x[14], g[10]);
    g[14] = fmaf(q, x[8]*x[10], g[14]);
  }
  { const float q = w * __ldg(cf + 89 * C);
    g[8] = fmaf(q, x[11]*x[15], g[8]);
    g[11] = fmaf(q, x[8]*x[15], g[11]);
    g[15] = fmaf(q, x[8]*x[11], g[15]);
  }
}

__device__ __forceinline__ float value_LM5(const float* x, const float* __restrict__ cf, int C) {
  float f = 0.0f;
  f = fmaf(__ldg(cf + 0 * C), x[5], f);
  f = fmaf(__ldg(cf + 1 * C), x[0]*x[5], f);
  f = fmaf(__ldg(cf + 2 * C), x[1]*x[2], f);
  f = fmaf(__ldg(cf + 3 * C), x[1]*x[12], f);
  f = fmaf(__ldg(cf + 4 * C), x[1]*x[14], f);
  f = fmaf(__ldg(cf + 5 * C), x[2]*x[11], f);
  f = fmaf(__ldg(cf + 6 * C), x[3]*x[10], f);
  f = fmaf(__ldg(cf + 7 * C), x[4]*x[7], f);
  f = fmaf(__ldg(cf + 8 * C), x[5]*x[6], f);
  f = fmaf(__ldg(cf + 9 * C), x[5]*x[8], f);
  f = fmaf(__ldg(cf + 10 * C), x[9]*x[14], f);
  f = fmaf(__ldg(cf + 11 * C), x[10]*x[13], f);
  f = fmaf(__ldg(cf + 12 * C), x[10]*x[15], f);
  f = fmaf(__ldg(cf + 13 * C), x[11]*x[12], f);
  f = fmaf(__ldg(cf + 14 * C), x[11]*x[14], f);
  f = fmaf(__ldg(cf + 15 * C), x[0]*x[0]*x[5], f);
  f = fmaf(__ldg(cf + 16 * C), x[0]*x[1]*x[2], f);
  f = fmaf(__ldg(cf + 17 * C), x[0]*x[1]*x[12], f);
  f = fmaf(__ldg(cf + 18 * C), x[0]*x[1]*x[14], f);
  f = fmaf(__ldg(cf + 19 * C), x[0]*x[2]*x[11], f);
  f = fmaf(__ldg(cf + 20 * C), x[0]*x[3]*x[10], f);
  f = fmaf(__ldg(cf + 21 * C), x[0]*x[4]*x[7], f);
  f = fmaf(__ldg(cf + 22 * C), x[0]*x[5]*x[6], f);
  f = fmaf(__ldg(cf + 23 * C), x[0]*x[5]*x[8], f);
  f = fmaf(__ldg(cf + 24 * C), x[0]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 25 * C), x[0]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 26 * C), x[0]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 27 * C), x[0]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 28 * C), x[0]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 29 * C), x[1]*x[1]*x[5], f);
  f = fmaf(__ldg(cf + 30 * C), x[1]*x[2]*x[6], f);
  f = fmaf(__ldg(cf + 31 * C), x[1]*x[2]*x[8], f);
  f = fmaf(__ldg(cf + 32 * C), x[1]*x[3]*x[7], f);
  f = fmaf(__ldg(cf + 33 * C), x[1]*x[4]*x[10], f);
  f = fmaf(__ldg(cf + 34 * C), x[1]*x[5]*x[9], f);
  f = fmaf(__ldg(cf + 35 * C), x[1]*x[5]*x[11], f);
  f = fmaf(__ldg(cf + 36 * C), x[1]*x[6]*x[12], f);
  f = fmaf(__ldg(cf + 37 * C), x[1]*x[6]*x[14], f);
  f = fmaf(__ldg(cf + 38 * C), x[1]*x[7]*x[13], f);
  f = fmaf(__ldg(cf + 39 * C), x[1]*x[7]*x[15], f);
  f = fmaf(__ldg(cf + 40 * C), x[1]*x[8]*x[12], f);
  f = fmaf(__ldg(cf + 41 * C), x[1]*x[8]*x[14], f);
  f = fmaf(__ldg(cf + 42 * C), x[2]*x[2]*x[5], f);
  f = fmaf(__ldg(cf + 43 * C), x[2]*x[3]*x[4], f);
  f = fmaf(__ldg(cf + 44 * C), x[2]*x[4]*x[13], f);
  f = fmaf(__ldg(cf + 45 * C), x[2]*x[4]*x[15], f);
  f = fmaf(__ldg(cf + 46 * C), x[2]*x[5]*x[12], f);
  f = fmaf(__ldg(cf + 47 * C), x[2]*x[5]*x[14], f);
  f = fmaf(__ldg(cf + 48 * C), x[2]*x[6]*x[11], f);
  f = fmaf(__ldg(cf + 49 * C), x[2]*x[7]*x[10], f);
  f = fmaf(__ldg(cf + 50 * C), x[2]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 51 * C), x[2]*x[8]*x[11], f);
  f = fmaf(__ldg(cf + 52 * C), x[3]*x[3]*x[5], f);
  f = fmaf(__ldg(cf + 53 * C), x[3]*x[4]*x[12], f);
  f = fmaf(__ldg(cf + 54 * C), x[3]*x[4]*x[14], f);
  f = fmaf(__ldg(cf + 55 * C), x[3]*x[5]*x[13], f);
  f = fmaf(__ldg(cf + 56 * C), x[3]*x[5]*x[15], f);
  f = fmaf(__ldg(cf + 57 * C), x[3]*x[6]*x[10], f);
  f = fmaf(__ldg(cf + 58 * C), x[3]*x[7]*x[9], f);
  f = fmaf(__ldg(cf + 59 * C), x[3]*x[7]*x[11], f);
  f = fmaf(__ldg(cf + 60 * C), x[3]*x[8]*x[10], f);
  f = fmaf(__ldg(cf + 61 * C), x[4]*x[4]*x[5], f);
  f = fmaf(__ldg(cf + 62 * C), x[4]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 63 * C), x[4]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 64 * C), x[4]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 65 * C), x[4]*x[12]*x[15], f);
  f = fmaf(__ldg(cf + 66 * C), x[4]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 67 * C), x[4]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 68 * C), x[5]*x[5]*x[5], f);
  f = fmaf(__ldg(cf + 69 * C), x[5]*x[6]*x[6], f);
  f = fmaf(__ldg(cf + 70 * C), x[5]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 71 * C), x[5]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 72 * C), x[5]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 73 * C), x[5]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 74 * C), x[5]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 75 * C), x[5]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 76 * C), x[5]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 77 * C), x[5]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 78 * C), x[5]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 79 * C), x[5]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 80 * C), x[5]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 81 * C), x[5]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 82 * C), x[6]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 83 * C), x[6]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 84 * C), x[6]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 85 * C), x[6]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 86 * C), x[6]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 87 * C), x[7]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 88 * C), x[7]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 89 * C), x[7]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 90 * C), x[7]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 91 * C), x[8]*x[9]*x[12], f);
  f = fmaf(__ldg(cf + 92 * C), x[8]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 93 * C), x[8]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 94 * C), x[8]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 95 * C), x[8]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 96 * C), x[8]*x[11]*x[14], f);
  return f;
}

__device__ __forceinline__ void grad_LM5(const float* x, float w, const float* __restrict__ cf, int C, float* g) {
  { const float q = w * __ldg(cf + 0 * C);
    g[5] += q;
  }
  { const float q = w * __ldg(cf + 1 * C);
    g[0] = fmaf(q, x[5], g[0]);
    g[5] = fmaf(q, x[0], g[5]);
  }
  { const float q = w * __ldg(cf + 2 * C);
    g[1] = fmaf(q, x[2], g[1]);
    g[2] = fmaf(q, x[1], g[2]);
  }
  { const float q = w * __ldg(cf + 3 * C);
    g[1] = fmaf(q, x[12], g[1]);
    g[12] = fmaf(q, x[1], g[12]);
  }
  { const float q = w * __ldg(cf + 4 * C);
    g[1] = fmaf(q, x[14], g[1]);
    g[14] = fmaf(q, x[1], g[14]);
  }
  { const float q = w * __ldg(cf + 5 * C);
    g[2] = fmaf(q, x[11], g[2]);
    g[11] = fmaf(q, x[2], g[11]);
  }
  { const float q = w * __ldg(cf + 6 * C);
    g[3] = fmaf(q, x[10], g[3]);
    g[10] = fmaf(q, x[3], g[10]);
  }
  { const float q = w * __ldg(cf + 7 * C);
    g[4] = fmaf(q, x[7], g[4]);
    g[7] = fmaf(q, x[4], g[7]);
  }
  { const float q = w * __ldg(cf + 8 * C);
    g[5] = fmaf(q, x[6], g[5]);
    g[6] = fmaf(q, x[5], g[6]);
  }
  { const float q = w * __ldg(cf + 9 * C);
    g[5] = fmaf(q, x[8], g[5]);
    g[8] = fmaf(q, x[5], g[8]);
  }
  { const float q = w * __ldg(cf + 10 * C);
    g[9] = fmaf(q, x[14], g[9]);
    g[14] = fmaf(q, x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 11 * C);
    g[10] = fmaf(q, x[13], g[10]);
    g[13] = fmaf(q, x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 12 * C);
    g[10] = fmaf(q, x[15], g[10]);
    g[15] = fmaf(q, x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 13 * C);
    g[11] = fmaf(q, x[12], g[11]);
    g[12] = fmaf(q, x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 14 * C);
    g[11] = fmaf(q, x[14], g[11]);
    g[14] = fmaf(q, x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 15 * C);
    g[0] = fmaf(q, x[0]*x[5], g[0]);
    g[0] = fmaf(q, x[0]*x[5], g[0]);
    g[5] = fmaf(q, x[0]*x[0], g[5]);
  }
  { const float q = w * __ldg(cf + 16 * C);
    g[0] = fmaf(q, x[1]*x[2], g[0]);
    g[1] = fmaf(q, x[0]*x[2], g[1]);
    g[2] = fmaf(q, x[0]*x[1], g[2]);
  }
  { const float q = w * __ldg(cf + 17 * C);
    g[0] = fmaf(q, x[1]*x[12], g[0]);
    g[1] = fmaf(q, x[0]*x[12], g[1]);
    g[12] = fmaf(q, x[0]*x[1], g[12]);
  }
  { const float q = w * __ldg(cf + 18 * C);
    g[0] = fmaf(q, x[1]*x[14], g[0]);
    g[1] = fmaf(q, x[0]*x[14], g[1]);
    g[14] = fmaf(q, x[0]*x[1], g[14]);
  }
  { const float q = w * __ldg(cf + 19 * C);
    g[0] = fmaf(q, x[2]*x[11], g[0]);
    g[2] = fmaf(q, x[0]*x[11], g[2]);
    g[11] = fmaf(q, x[0]*x[2], g[11]);
  }
  { const float q = w * __ldg(cf + 20 * C);
    g[0] = fmaf(q, x[3]*x[10], g[0]);
    g[3] = fmaf(q, x[0]*x[10], g[3]);
    g[10] = fmaf(q, x[0]*x[3], g[10]);
  }
  { const float q = w * __ldg(cf + 21 * C);
    g[0] = fmaf(q, x[4]*x[7], g[0]);
    g[4] = fmaf(q, x[0]*x[7], g[4]);
    g[7] = fmaf(q, x[0]*x[4], g[7]);
  }
  { const float q = w * __ldg(cf + 22 * C);
    g[0] = fmaf(q, x[5]*x[6], g[0]);
    g[5] = fmaf(q, x[0]*x[6], g[5]);
    g[6] = fmaf(q, x[0]*x[5], g[6]);
  }
  { const float q = w * __ldg(cf + 23 * C);
    g[0] = fmaf(q, x[5]*x[8], g[0]);
    g[5] = fmaf(q, x[0]*x[8], g[5]);
    g[8] = fmaf(q, x[0]*x[5], g[8]);
  }
  { const float q = w * __ldg(cf + 24 * C);
    g[0] = fmaf(q, x[9]*x[14], g[0]);
    g[9] = fmaf(q, x[0]*x[14], g[9]);
    g[14] = fmaf(q, x[0]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 25 * C);
    g[0] = fmaf(q, x[10]*x[13], g[0]);
    g[10] = fmaf(q, x[0]*x[13], g[10]);
    g[13] = fmaf(q, x[0]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 26 * C);
    g[0] = fmaf(q, x[10]*x[15], g[0]);
    g[10] = fmaf(q, x[0]*x[15], g[10]);
    g[15] = fmaf(q, x[0]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 27 * C);
    g[0] = fmaf(q, x[11]*x[12], g[0]);
    g[11] = fmaf(q, x[0]*x[12], g[11]);
    g[12] = fmaf(q, x[0]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 28 * C);
    g[0] = fmaf(q, x[11]*x[14], g[0]);
    g[11] = fmaf(q, x[0]*x[14], g[11]);
    g[14] = fmaf(q, x[0]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 29 * C);
    g[1] = fmaf(q, x[1]*x[5], g[1]);
    g[1] = fmaf(q, x[1]*x[5], g[1]);
    g[5] = fmaf(q, x[1]*x[1], g[5]);
  }
  { const float q = w * __ldg(cf + 30 * C);
    g[1] = fmaf(q, x[2]*x[6], g[1]);
    g[2] = fmaf(q, x[1]*x[6], g[2]);
    g[6] = fmaf(q, x[1]*x[2], g[6]);
  }
  { const float q = w * __ldg(cf + 31 * C);
    g[1] = fmaf(q, x[2]*x[8], g[1]);
    g[2] = fmaf(q, x[1]*x[8], g[2]);
    g[8] = fmaf(q, x[1]*x[2], g[8]);
  }
  { const float q = w * __ldg(cf + 32 * C);
    g[1] = fmaf(q, x[3]*x[7], g[1]);
    g[3] = fmaf(q, x[1]*x[7], g[3]);
    g[7] = fmaf(q, x[1]*x[3], g[7]);
  }
  { const float q = w * __ldg(cf + 33 * C);
    g[1] = fmaf(q, x[4]*x[10], g[1]);
    g[4] = fmaf(q, x[1]*x[10], g[4]);
    g[10] = fmaf(q, x[1]*x[4], g[10]);
  }
  { const float q = w * __ldg(cf + 34 * C);
    g[1] = fmaf(q, x[5]*x[9], g[1]);
    g[5] = fmaf(q, x[1]*x[9], g[5]);
    g[9] = fmaf(q, x[1]*x[5], g[9]);
  }
  { const float q = w * __ldg(cf + 35 * C);
    g[1] = fmaf(q, x[5]*x[11], g[1]);
    g[5] = fmaf(q, x[1]*x[11], g[5]);
    g[11] = fmaf(q, x[1]*x[5], g[11]);
  }
  { const float q = w * __ldg(cf + 36 * C);
    g[1] = fmaf(q, x[6]*x[12], g[1]);
    g[6] = fmaf(q, x[1]*x[12], g[6]);
    g[12] = fmaf(q, x[1]*x[6], g[12]);
  }
  { const float q = w * __ldg(cf + 37 * C);
    g[1] = fmaf(q, x[6]*x[14], g[1]);
    g[6] = fmaf(q, x[1]*x[14], g[6]);
    g[14] = fmaf(q, x[1]*x[6], g[14]);
  }
  { const float q = w * __ldg(cf + 38 * C);
    g[1] = fmaf(q, x[7]*x[13], g[1]);
    g[7] = fmaf(q, x[1]*x[13], g[7]);
    g[13] = fmaf(q, x[1]*x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 39 * C);
    g[1] = fmaf(q, x[7]*x[15], g[1]);
    g[7] = fmaf(q, x[1]*x[15], g[7]);
    g[15] = fmaf(q, x[1]*x[7], g[15]);
  }
  { const float q = w * __ldg(cf + 40 * C);
    g[1] = fmaf(q, x[8]*x[12], g[1]);
    g[8] = fmaf(q, x[1]*x[12], g[8]);
    g[12] = fmaf(q, x[1]*x[8], g[12]);
  }
  { const float q = w * __ldg(cf + 41 * C);
    g[1] = fmaf(q, x[8]*x[14], g[1]);
    g[8] = fmaf(q, x[1]*x[14], g[8]);
    g[14] = fmaf(q, x[1]*x[8], g[14]);
  }
  { const float q = w * __ldg(cf + 42 * C);
    g[2] = fmaf(q, x[2]*x[5], g[2]);
    g[2] = fmaf(q, x[2]*x[5], g[2]);
    g[5] = fmaf(q, x[2]*x[2], g[5]);
  }
  { const float q = w * __ldg(cf + 43 * C);
    g[2] = fmaf(q, x[3]*x[4], g[2]);
    g[3] = fmaf(q, x[2]*x[4], g[3]);
    g[4] = fmaf(q, x[2]*x[3], g[4]);
  }
  { const float q = w * __ldg(cf + 44 * C);
    g[2] = fmaf(q, x[4]*x[13], g[2]);
    g[4] = fmaf(q, x[2]*x[13], g[4]);
    g[13] = fmaf(q, x[2]*x[4], g[13]);
  }
  { const float q = w * __ldg(cf + 45 * C);
    g[2] = fmaf(q, x[4]*x[15], g[2]);
    g[4] = fmaf(q, x[2]*x[15], g[4]);
    g[15] = fmaf(q, x[2]*x[4], g[15]);
  }
  { const float q = w * __ldg(cf + 46 * C);
    g[2] = fmaf(q, x[5]*x[12], g[2]);
    g[5] = fmaf(q, x[2]*x[12], g[5]);
    g[12] = fmaf(q, x[2]*x[5], g[12]);
  }
  { const float q = w * __ldg(cf + 47 * C);
    g[2] = fmaf(q, x[5]*x[14], g[2]);
    g[5] = fmaf(q, x[2]*x[14], g[5]);
    g[14] = fmaf(q, x[2]*x[5], g[14]);
  }
  { const float q = w * __ldg(cf + 48 * C);
    g[2] = fmaf(q, x[6]*x[11], g[2]);
    g[6] = fmaf(q, x[2]*x[11], g[6]);
    g[11] = fmaf(q, x[2]*x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 49 * C);
    g[2] = fmaf(q, x[7]*x[10], g[2]);
    g[7] = fmaf(q, x[2]*x[10], g[7]);
    g[10] = fmaf(q, x[2]*x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 50 * C);
    g[2] = fmaf(q, x[8]*x[9], g[2]);
    g[8] = fmaf(q, x[2]*x[9], g[8]);
    g[9] = fmaf(q, x[2]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 51 * C);
    g[2] = fmaf(q, x[8]*x[11], g[2]);
    g[8] = fmaf(q, x[2]*x[11], g[8]);
    g[11] = fmaf(q, x[2]*x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 52 * C);
    g[3] = fmaf(q, x[3]*x[5], g[3]);
    g[3] = fmaf(q, x[3]*x[5], g[3]);
    g[5] = fmaf(q, x[3]*x[3], g[5]);
  }
  { const float q = w * __ldg(cf + 53 * C);
    g[3] = fmaf(q, x[4]*x[12], g[3]);
    g[4] = fmaf(q, x[3]*x[12], g[4]);
    g[12] = fmaf(q, x[3]*x[4], g[12]);
  }
  { const float q = w * __ldg(cf + 54 * C);
    g[3] = fmaf(q, x[4]*x[14], g[3]);
    g[4] = fmaf(q, x[3]*x[14], g[4]);
    g[14] = fmaf(q, x[3]*x[4], g[14]);
  }
  { const float q = w * __ldg(cf + 55 * C);
    g[3] = fmaf(q, x[5]*x[13], g[3]);
    g[5] = fmaf(q, x[3]*x[13], g[5]);
    g[13] = fmaf(q, x[3]*x[5], g[13]);
  }
  { const float q = w * __ldg(cf + 56 * C);
    g[3] = fmaf(q, x[5]*x[15], g[3]);
    g[5] = fmaf(q, x[3]*x[15], g[5]);
    g[15] = fmaf(q, x[3]*x[5], g[15]);
  }
  { const float q = w * __ldg(cf + 57 * C);
    g[3] = fmaf(q, x[6]*x[10], g[3]);
    g[6] = fmaf(q, x[3]*x[10], g[6]);
    g[10] = fmaf(q, x[3]*x[6], g[10]);
  }
  { const float q = w * __ldg(cf + 58 * C);
    g[3] = fmaf(q, x[7]*x[9], g[3]);
    g[7] = fmaf(q, x[3]*x[9], g[7]);
    g[9] = fmaf(q, x[3]*x[7], g[9]);
  }
  { const float q = w * __ldg(cf + 59 * C);
    g[3] = fmaf(q, x[7]*x[11], g[3]);
    g[7] = fmaf(q, x[3]*x[11], g[7]);
    g[11] = fmaf(q, x[3]*x[7], g[11]);
  }
  { const float q = w * __ldg(cf + 60 * C);
    g[3] = fmaf(q, x[8]*x[10], g[3]);
    g[8] = fmaf(q, x[3]*x[10], g[8]);
    g[10] = fmaf(q, x[3]*x[8], g[10]);
  }
  { const float q = w * __ldg(cf + 61 * C);
    g[4] = fmaf(q, x[4]*x[5], g[4]);
    g[4] = fmaf(q, x[4]*x[5], g[4]);
    g[5] = fmaf(q, x[4]*x[4], g[5]);
  }
  { const float q = w * __ldg(cf + 62 * C);
    g[4] = fmaf(q, x[9]*x[10], g[4]);
    g[9] = fmaf(q, x[4]*x[10], g[9]);
    g[10] = fmaf(q, x[4]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 63 * C);
    g[4] = fmaf(q, x[10]*x[11], g[4]);
    g[10] = fmaf(q, x[4]*x[11], g[10]);
    g[11] = fmaf(q, x[4]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 64 * C);
    g[4] = fmaf(q, x[12]*x[13], g[4]);
    g[12] = fmaf(q, x[4]*x[13], g[12]);
    g[13] = fmaf(q, x[4]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 65 * C);
    g[4] = fmaf(q, x[12]*x[15], g[4]);
    g[12] = fmaf(q, x[4]*x[15], g[12]);
    g[15] = fmaf(q, x[4]*x[12], g[15]);
  }
  { const float q = w * __ldg(cf + 66 * C);
    g[4] = fmaf(q, x[13]*x[14], g[4]);
    g[13] = fmaf(q, x[4]*x[14], g[13]);
    g[14] = fmaf(q, x[4]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 67 * C);
    g[4] = fmaf(q, x[14]*x[15], g[4]);
    g[14] = fmaf(q, x[4]*x[15], g[14]);
    g[15] = fmaf(q, x[4]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 68 * C);
    g[5] = fmaf(q, x[5]*x[5], g[5]);
    g[5] = fmaf(q, x[5]*x[5], g[5]);
    g[5] = fmaf(q, x[5]*x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 69 * C);
    g[5] = fmaf(q, x[6]*x[6], g[5]);
    g[6] = fmaf(q, x[5]*x[6], g[6]);
    g[6] = fmaf(q, x[5]*x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 70 * C);
    g[5] = fmaf(q, x[7]*x[7], g[5]);
    g[7] = fmaf(q, x[5]*x[7], g[7]);
    g[7] = fmaf(q, x[5]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 71 * C);
    g[5] = fmaf(q, x[8]*x[8], g[5]);
    g[8] = fmaf(q, x[5]*x[8], g[8]);
    g[8] = fmaf(q, x[5]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 72 * C);
    g[5] = fmaf(q, x[9]*x[9], g[5]);
    g[9] = fmaf(q, x[5]*x[9], g[9]);
    g[9] = fmaf(q, x[5]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 73 * C);
    g[5] = fmaf(q, x[9]*x[11], g[5]);
    g[9] = fmaf(q, x[5]*x[11], g[9]);
    g[11] = fmaf(q, x[5]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 74 * C);
    g[5] = fmaf(q, x[10]*x[10], g[5]);
    g[10] = fmaf(q, x[5]*x[10], g[10]);
    g[10] = fmaf(q, x[5]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 75 * C);
    g[5] = fmaf(q, x[11]*x[11], g[5]);
    g[11] = fmaf(q, x[5]*x[11], g[11]);
    g[11] = fmaf(q, x[5]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 76 * C);
    g[5] = fmaf(q, x[12]*x[12], g[5]);
    g[12] = fmaf(q, x[5]*x[12], g[12]);
    g[12] = fmaf(q, x[5]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 77 * C);
    g[5] = fmaf(q, x[12]*x[14], g[5]);
    g[12] = fmaf(q, x[5]*x[14], g[12]);
    g[14] = fmaf(q, x[5]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 78 * C);
    g[5] = fmaf(q, x[13]*x[13], g[5]);
    g[13] = fmaf(q, x[5]*x[13], g[13]);
    g[13] = fmaf(q, x[5]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 79 * C);
    g[5] = fmaf(q, x[13]*x[15], g[5]);
    g[13] = fmaf(q, x[5]*x[15], g[13]);
    g[15] = fmaf(q, x[5]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 80 * C);
    g[5] = fmaf(q, x[14]*x[14], g[5]);
    g[14] = fmaf(q, x[5]*x[14], g[14]);
    g[14] = fmaf(q, x[5]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 81 * C);
    g[5] = fmaf(q, x[15]*x[15], g[5]);
    g[15] = fmaf(q, x[5]*x[15], g[15]);
    g[15] = fmaf(q, x[5]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 82 * C);
    g[6] = fmaf(q, x[9]*x[14], g[6]);
    g[9] = fmaf(q, x[6]*x[14], g[9]);
    g[14] = fmaf(q, x[6]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 83 * C);
    g[6] = fmaf(q, x[10]*x[13], g[6]);
    g[10] = fmaf(q, x[6]*x[13], g[10]);
    g[13] = fmaf(q, x[6]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 84 * C);
    g[6] = fmaf(q, x[10]*x[15], g[6]);
    g[10] = fmaf(q, x[6]*x[15], g[10]);
    g[15] = fmaf(q, x[6]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 85 * C);
    g[6] = fmaf(q, x[11]*x[12], g[6]);
    g[11] = fmaf(q, x[6]*x[12], g[11]);
    g[12] = fmaf(q, x[6]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 86 * C);
    g[6] = fmaf(q, x[11]*x[14], g[6]);
    g[11] = fmaf(q, x[6]*x[14], g[11]);
    g[14] = fmaf(q, x[6]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 87 * C);
    g[7] = fmaf(q, x[9]*x[13], g[7]);
    g[9] = fmaf(q, x[7]*x[13], g[9]);
    g[13] = fmaf(q, x[7]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 88 * C);
    g[7] = fmaf(q, x[10]*x[12], g[7]);
    g[10] = fmaf(q, x[7]*x[12], g[10]);
    g[12] = fmaf(q, x[7]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 89 * C);
    g[7] = fmaf(q, x[11]*x[13], g[7]);
    g[11] = fmaf(q, x[7]*x[13], g[11]);
    g[13] = fmaf(q, x[7]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 90 * C);
    g[7] = fmaf(q, x[11]*x[15], g[7]);
    g[11] = fmaf(q, x[7]*x[15], g[11]);
    g[15] = fmaf(q, x[7]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 91 * C);
    g[8] = fmaf(q, x[9]*x[12], g[8]);
    g[9] = fmaf(q, x[8]*x[12], g[9]);
    g[12] = fmaf(q, x[8]*x[9], g[12]);
  }
  { const float q = w * __ldg(cf + 92 * C);
    g[8] = fmaf(q, x[9]*x[14], g[8]);
    g[9] = fmaf(q, x[8]*x[14], g[9]);
    g[14] = fmaf(q, x[8]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 93 * C);
    g[8] = fmaf(q, x[10]*x[13], g[8]);
    g[10] = fmaf(q, x[8]*x[13], g[10]);
    g[13] = fmaf(q, x[8]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 94 * C);
    g[8] = fmaf(q, x[10]*x[15], g[8]);
    g[10] = fmaf(q, x[8]*x[15], g[10]);
    g[15] = fmaf(q, x[8]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 95 * C);
    g[8] = fmaf(q, x[11]*x[12], g[8]);
    g[11] = fmaf(q, x[8]*x[12], g[11]);
    g[12] = fmaf(q, x[8]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 96 * C);
    g[8] = fmaf(q, x[11]*x[14], g[8]);
    g[11] = fmaf(q, x[8]*x[14], g[11]);
    g[14] = fmaf(q, x[8]*x[11], g[14]);
  }
}

__device__ __forceinline__ float value_LM6(const float* x, const float* __restrict__ cf, int C) {
  float f = 0.0f;
  f = fmaf(__ldg(cf + 0 * C), x[6], f);
  f = fmaf(__ldg(cf + 1 * C), x[0]*x[6], f);
  f = fmaf(__ldg(cf + 2 * C), x[1]*x[1], f);
  f = fmaf(__ldg(cf + 3 * C), x[1]*x[11], f);
  f = fmaf(__ldg(cf + 4 * C), x[2]*x[2], f);
  f = fmaf(__ldg(cf + 5 * C), x[2]*x[12], f);
  f = fmaf(__ldg(cf + 6 * C), x[3]*x[3], f);
  f = fmaf(__ldg(cf + 7 * C), x[3]*x[13], f);
  f = fmaf(__ldg(cf + 8 * C), x[4]*x[4], f);
  f = fmaf(__ldg(cf + 9 * C), x[5]*x[5], f);
  f = fmaf(__ldg(cf + 10 * C), x[6]*x[6], f);
  f = fmaf(__ldg(cf + 11 * C), x[7]*x[7], f);
  f = fmaf(__ldg(cf + 12 * C), x[8]*x[8], f);
  f = fmaf(__ldg(cf + 13 * C), x[9]*x[9], f);
  f = fmaf(__ldg(cf + 14 * C), x[11]*x[11], f);
  f = fmaf(__ldg(cf + 15 * C), x[12]*x[12], f);
  f = fmaf(__ldg(cf + 16 * C), x[13]*x[13], f);
  f = fmaf(__ldg(cf + 17 * C), x[15]*x[15], f);
  f = fmaf(__ldg(cf + 18 * C), x[0]*x[0]*x[6], f);
  f = fmaf(__ldg(cf + 19 * C), x[0]*x[1]*x[1], f);
  f = fmaf(__ldg(cf + 20 * C), x[0]*x[1]*x[11], f);
  f = fmaf(__ldg(cf + 21 * C), x[0]*x[2]*x[2], f);
  f = fmaf(__ldg(cf + 22 * C), x[0]*x[2]*x[12], f);
  f = fmaf(__ldg(cf + 23 * C), x[0]*x[3]*x[3], f);
  f = fmaf(__ldg(cf + 24 * C), x[0]*x[3]*x[13], f);
  f = fmaf(__ldg(cf + 25 * C), x[0]*x[4]*x[4], f);
  f = fmaf(__ldg(cf + 26 * C), x[0]*x[5]*x[5], f);
  f = fmaf(__ldg(cf + 27 * C), x[0]*x[6]*x[6], f);
  f = fmaf(__ldg(cf + 28 * C), x[0]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 29 * C), x[0]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 30 * C), x[0]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 31 * C), x[0]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 32 * C), x[0]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 33 * C), x[0]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 34 * C), x[0]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 35 * C), x[1]*x[1]*x[6], f);
  f = fmaf(__ldg(cf + 36 * C), x[1]*x[1]*x[8], f);
  f = fmaf(__ldg(cf + 37 * C), x[1]*x[2]*x[5], f);
  f = fmaf(__ldg(cf + 38 * C), x[1]*x[3]*x[4], f);
  f = fmaf(__ldg(cf + 39 * C), x[1]*x[4]*x[13], f);
  f = fmaf(__ldg(cf + 40 * C), x[1]*x[4]*x[15], f);
  f = fmaf(__ldg(cf + 41 * C), x[1]*x[5]*x[12], f);
  f = fmaf(__ldg(cf + 42 * C), x[1]*x[5]*x[14], f);
  f = fmaf(__ldg(cf + 43 * C), x[1]*x[6]*x[11], f);
  f = fmaf(__ldg(cf + 44 * C), x[1]*x[7]*x[10], f);
  f = fmaf(__ldg(cf + 45 * C), x[1]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 46 * C), x[1]*x[8]*x[11], f);
  f = fmaf(__ldg(cf + 47 * C), x[2]*x[2]*x[6], f);
  f = fmaf(__ldg(cf + 48 * C), x[2]*x[3]*x[7], f);
  f = fmaf(__ldg(cf + 49 * C), x[2]*x[4]*x[10], f);
  f = fmaf(__ldg(cf + 50 * C), x[2]*x[5]*x[11], f);
  f = fmaf(__ldg(cf + 51 * C), x[2]*x[6]*x[12], f);
  f = fmaf(__ldg(cf + 52 * C), x[2]*x[7]*x[13], f);
  f = fmaf(__ldg(cf + 53 * C), x[2]*x[8]*x[14], f);
  f = fmaf(__ldg(cf + 54 * C), x[3]*x[3]*x[6], f);
  f = fmaf(__ldg(cf + 55 * C), x[3]*x[3]*x[8], f);
  f = fmaf(__ldg(cf + 56 * C), x[3]*x[4]*x[9], f);
  f = fmaf(__ldg(cf + 57 * C), x[3]*x[4]*x[11], f);
  f = fmaf(__ldg(cf + 58 * C), x[3]*x[5]*x[10], f);
  f = fmaf(__ldg(cf + 59 * C), x[3]*x[6]*x[13], f);
  f = fmaf(__ldg(cf + 60 * C), x[3]*x[7]*x[12], f);
  f = fmaf(__ldg(cf + 61 * C), x[3]*x[7]*x[14], f);
  f = fmaf(__ldg(cf + 62 * C), x[3]*x[8]*x[13], f);
  f = fmaf(__ldg(cf + 63 * C), x[3]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 64 * C), x[4]*x[4]*x[6], f);
  f = fmaf(__ldg(cf + 65 * C), x[4]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 66 * C), x[4]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 67 * C), x[4]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 68 * C), x[4]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 69 * C), x[5]*x[5]*x[6], f);
  f = fmaf(__ldg(cf + 70 * C), x[5]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 71 * C), x[5]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 72 * C), x[5]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 73 * C), x[5]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 74 * C), x[5]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 75 * C), x[6]*x[6]*x[6], f);
  f = fmaf(__ldg(cf + 76 * C), x[6]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 77 * C), x[6]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 78 * C), x[6]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 79 * C), x[6]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 80 * C), x[6]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 81 * C), x[6]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 82 * C), x[6]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 83 * C), x[6]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 84 * C), x[6]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 85 * C), x[7]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 86 * C), x[7]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 87 * C), x[7]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 88 * C), x[7]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 89 * C), x[7]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 90 * C), x[8]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 91 * C), x[8]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 92 * C), x[8]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 93 * C), x[8]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 94 * C), x[8]*x[13]*x[15], f);
  return f;
}

__device__ __forceinline__ void grad_LM6(const float* x, float w, const float* __restrict__ cf, int C, float* g) {
  { const float q = w * __ldg(cf + 0 * C);
    g[6] += q;
  }
  { const float q = w * __ldg(cf + 1 * C);
    g[0] = fmaf(q, x[6], g[0]);
    g[6] = fmaf(q, x[0], g[6]);
  }
  { const float q = w * __ldg(cf + 2 * C);
    g[1] = fmaf(q, x[1], g[1]);
    g[1] = fmaf(q, x[1], g[1]);
  }
  { const float q = w * __ldg(cf + 3 * C);
    g[1] = fmaf(q, x[11], g[1]);
    g[11] = fmaf(q, x[1], g[11]);
  }
  { const float q = w * __ldg(cf + 4 * C);
    g[2] = fmaf(q, x[2], g[2]);
    g[2] = fmaf(q, x[2], g[2]);
  }
  { const float q = w * __ldg(cf + 5 * C);
    g[2] = fmaf(q, x[12], g[2]);
    g[12] = fmaf(q, x[2], g[12]);
  }
  { const float q = w * __ldg(cf + 6 * C);
    g[3] = fmaf(q, x[3], g[3]);
    g[3] = fmaf(q, x[3], g[3]);
  }
  { const float q = w * __ldg(cf + 7 * C);
    g[3] = fmaf(q, x[13], g[3]);
    g[13] = fmaf(q, x[3], g[13]);
  }
  { const float q = w * __ldg(cf + 8 * C);
    g[4] = fmaf(q, x[4], g[4]);
    g[4] = fmaf(q, x[4], g[4]);
  }
  { const float q = w * __ldg(cf + 9 * C);
    g[5] = fmaf(q, x[5], g[5]);
    g[5] = fmaf(q, x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 10 * C);
    g[6] = fmaf(q, x[6], g[6]);
    g[6] = fmaf(q, x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 11 * C);
    g[7] = fmaf(q, x[7], g[7]);
    g[7] = fmaf(q, x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 12 * C);
    g[8] = fmaf(q, x[8], g[8]);
    g[8] = fmaf(q, x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 13 * C);
    g[9] = fmaf(q, x[9], g[9]);
    g[9] = fmaf(q, x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 14 * C);
    g[11] = fmaf(q, x[11], g[11]);
    g[11] = fmaf(q, x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 15 * C);
    g[12] = fmaf(q, x[12], g[12]);
    g[12] = fmaf(q, x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 16 * C);
    g[13] = fmaf(q, x[13], g[13]);
    g[13] = fmaf(q, x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 17 * C);
    g[15] = fmaf(q, x[15], g[15]);
    g[15] = fmaf(q, x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 18 * C);
    g[0] = fmaf(q, x[0]*x[6], g[0]);
    g[0] = fmaf(q, x[0]*x[6], g[0]);
    g[6] = fmaf(q, x[0]*x[0], g[6]);
  }
  { const float q = w * __ldg(cf + 19 * C);
    g[0] = fmaf(q, x[1]*x[1], g[0]);
    g[1] = fmaf(q, x[0]*x[1], g[1]);
    g[1] = fmaf(q, x[0]*x[1], g[1]);
  }
  { const float q = w * __ldg(cf + 20 * C);
    g[0] = fmaf(q, x[1]*x[11], g[0]);
    g[1] = fmaf(q, x[0]*x[11], g[1]);
    g[11] = fmaf(q, x[0]*x[1], g[11]);
  }
  { const float q = w * __ldg(cf + 21 * C);
    g[0] = fmaf(q, x[2]*x[2], g[0]);
    g[2] = fmaf(q, x[0]*x[2], g[2]);
    g[2] = fmaf(q, x[0]*x[2], g[2]);
  }
  { const float q = w * __ldg(cf + 22 * C);
    g[0] = fmaf(q, x[2]*x[12], g[0]);
    g[2] = fmaf(q, x[0]*x[12], g[2]);
    g[12] = fmaf(q, x[0]*x[2], g[12]);
  }
  { const float q = w * __ldg(cf + 23 * C);
    g[0] = fmaf(q, x[3]*x[3], g[0]);
    g[3] = fmaf(q, x[0]*x[3], g[3]);
    g[3] = fmaf(q, x[0]*x[3], g[3]);
  }
  { const float q = w * __ldg(cf + 24 * C);
    g[0] = fmaf(q, x[3]*x[13], g[0]);
    g[3] = fmaf(q, x[0]*x[13], g[3]);
    g[13] = fmaf(q, x[0]*x[3], g[13]);
  }
  { const float q = w * __ldg(cf + 25 * C);
    g[0] = fmaf(q, x[4]*x[4], g[0]);
    g[4] = fmaf(q, x[0]*x[4], g[4]);
    g[4] = fmaf(q, x[0]*x[4], g[4]);
  }
  { const float q = w * __ldg(cf + 26 * C);
    g[0] = fmaf(q, x[5]*x[5], g[0]);
    g[5] = fmaf(q, x[0]*x[5], g[5]);
    g[5] = fmaf(q, x[0]*x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 27 * C);
    g[0] = fmaf(q, x[6]*x[6], g[0]);
    g[6] = fmaf(q, x[0]*x[6], g[6]);
    g[6] = fmaf(q, x[0]*x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 28 * C);
    g[0] = fmaf(q, x[7]*x[7], g[0]);
    g[7] = fmaf(q, x[0]*x[7], g[7]);
    g[7] = fmaf(q, x[0]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 29 * C);
    g[0] = fmaf(q, x[8]*x[8], g[0]);
    g[8] = fmaf(q, x[0]*x[8], g[8]);
    g[8] = fmaf(q, x[0]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 30 * C);
    g[0] = fmaf(q, x[9]*x[9], g[0]);
    g[9] = fmaf(q, x[0]*x[9], g[9]);
    g[9] = fmaf(q, x[0]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 31 * C);
    g[0] = fmaf(q, x[11]*x[11], g[0]);
    g[11] = fmaf(q, x[0]*x[11], g[11]);
    g[11] = fmaf(q, x[0]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 32 * C);
    g[0] = fmaf(q, x[12]*x[12], g[0]);
    g[12] = fmaf(q, x[0]*x[12], g[12]);
    g[12] = fmaf(q, x[0]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 33 * C);
    g[0] = fmaf(q, x[13]*x[13], g[0]);
    g[13] = fmaf(q, x[0]*x[13], g[13]);
    g[13] = fmaf(q, x[0]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 34 * C);
    g[0] = fmaf(q, x[15]*x[15], g[0]);
    g[15] = fmaf(q, x[0]*x[15], g[15]);
    g[15] = fmaf(q, x[0]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 35 * C);
    g[1] = fmaf(q, x[1]*x[6], g[1]);
    g[1] = fmaf(q, x[1]*x[6], g[1]);
    g[6] = fmaf(q, x[1]*x[1], g[6]);
  }
  { const float q = w * __ldg(cf + 36 * C);
    g[1] = fmaf(q, x[1]*x[8], g[1]);
    g[1] = fmaf(q, x[1]*x[8], g[1]);
    g[8] = fmaf(q, x[1]*x[1], g[8]);
  }
  { const float q = w * __ldg(cf + 37 * C);
    g[1] = fmaf(q, x[2]*x[5], g[1]);
    g[2] = fmaf(q, x[1]*x[5], g[2]);
    g[5] = fmaf(q, x[1]*x[2], g[5]);
  }
  { const float q = w * __ldg(cf + 38 * C);
    g[1] = fmaf(q, x[3]*x[4], g[1]);
    g[3] = fmaf(q, x[1]*x[4], g[3]);
    g[4] = fmaf(q, x[1]*x[3], g[4]);
  }
  { const float q = w * __ldg(cf + 39 * C);
    g[1] = fmaf(q, x[4]*x[13], g[1]);
    g[4] = fmaf(q, x[1]*x[13], g[4]);
    g[13] = fmaf(q, x[1]*x[4], g[13]);
  }
  { const float q = w * __ldg(cf + 40 * C);
    g[1] = fmaf(q, x[4]*x[15], g[1]);
    g[4] = fmaf(q, x[1]*x[15], g[4]);
    g[15] = fmaf(q, x[1]*x[4], g[15]);
  }
  { const float q = w * __ldg(cf + 41 * C);
    g[1] = fmaf(q, x[5]*x[12], g[1]);
    g[5] = fmaf(q, x[1]*x[12], g[5]);
    g[12] = fmaf(q, x[1]*x[5], g[12]);
  }
  { const float q = w * __ldg(cf + 42 * C);
    g[1] = fmaf(q, x[5]*x[14], g[1]);
    g[5] = fmaf(q, x[1]*x[14], g[5]);
    g[14] = fmaf(q, x[1]*x[5], g[14]);
  }
  { const float q = w * __ldg(cf + 43 * C);
    g[1] = fmaf(q, x[6]*x[11], g[1]);
    g[6] = fmaf(q, x[1]*x[11], g[6]);
    g[11] = fmaf(q, x[1]*x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 44 * C);
    g[1] = fmaf(q, x[7]*x[10], g[1]);
    g[7] = fmaf(q, x[1]*x[10], g[7]);
    g[10] = fmaf(q, x[1]*x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 45 * C);
    g[1] = fmaf(q, x[8]*x[9], g[1]);
    g[8] = fmaf(q, x[1]*x[9], g[8]);
    g[9] = fmaf(q, x[1]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 46 * C);
    g[1] = fmaf(q, x[8]*x[11], g[1]);
    g[8] = fmaf(q, x[1]*x[11], g[8]);
    g[11] = fmaf(q, x[1]*x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 47 * C);
    g[2] = fmaf(q, x[2]*x[6], g[2]);
    g[2] = fmaf(q, x[2]*x[6], g[2]);
    g[6] = fmaf(q, x[2]*x[2], g[6]);
  }
  { const float q = w * __ldg(cf + 48 * C);
    g[2] = fmaf(q, x[3]*x[7], g[2]);
    g[3] = fmaf(q, x[2]*x[7], g[3]);
    g[7] = fmaf(q, x[2]*x[3], g[7]);
  }
  { const float q = w * __ldg(cf + 49 * C);
    g[2] = fmaf(q, x[4]*x[10], g[2]);
    g[4] = fmaf(q, x[2]*x[10], g[4]);
    g[10] = fmaf(q, x[2]*x[4], g[10]);
  }
  { const float q = w * __ldg(cf + 50 * C);
    g[2] = fmaf(q, x[5]*x[11], g[2]);
    g[5] = fmaf(q, x[2]*x[11], g[5]);
    g[11] = fmaf(q, x[2]*x[5], g[11]);
  }
  { const float q = w * __ldg(cf + 51 * C);
    g[2] = fmaf(q, x[6]*x[12], g[2]);
    g[6] = fmaf(q, x[2]*x[12], g[6]);
    g[12] = fmaf(q, x[2]*x[6], g[12]);
  }
  { const float q = w * __ldg(cf + 52 * C);
    g[2] = fmaf(q, x[7]*x[13], g[2]);
    g[7] = fmaf(q, x[2]*x[13], g[7]);
    g[13] = fmaf(q, x[2]*x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 53 * C);
    g[2] = fmaf(q, x[8]*x[14], g[2]);
    g[8] = fmaf(q, x[2]*x[14], g[8]);
    g[14] = fmaf(q, x[2]*x[8], g[14]);
  }
  { const float q = w * __ldg(cf + 54 * C);
    g[3] = fmaf(q, x[3]*x[6], g[3]);
    g[3] = fmaf(q, x[3]*x[6], g[3]);
    g[6] = fmaf(q, x[3]*x[3], g[6]);
  }
  { const float q = w * __ldg(cf + 55 * C);
    g[3] = fmaf(q, x[3]*x[8], g[3]);
    g[3] = fmaf(q, x[3]*x[8], g[3]);
    g[8] = fmaf(q, x[3]*x[3], g[8]);
  }
  { const float q = w * __ldg(cf + 56 * C);
    g[3] = fmaf(q, x[4]*x[9], g[3]);
    g[4] = fmaf(q, x[3]*x[9], g[4]);
    g[9] = fmaf(q, x[3]*x[4], g[9]);
  }
  { const float q = w * __ldg(cf + 57 * C);
    g[3] = fmaf(q, x[4]*x[11], g[3]);
    g[4] = fmaf(q, x[3]*x[11], g[4]);
    g[11] = fmaf(q, x[3]*x[4], g[11]);
  }
  { const float q = w * __ldg(cf + 58 * C);
    g[3] = fmaf(q, x[5]*x[10], g[3]);
    g[5] = fmaf(q, x[3]*x[10], g[5]);
    g[10] = fmaf(q, x[3]*x[5], g[10]);
  }
  { const float q = w * __ldg(cf + 59 * C);
    g[3] = fmaf(q, x[6]*x[13], g[3]);
    g[6] = fmaf(q, x[3]*x[13], g[6]);
    g[13] = fmaf(q, x[3]*x[6], g[13]);
  }
  { const float q = w * __ldg(cf + 60 * C);
    g[3] = fmaf(q, x[7]*x[12], g[3]);
    g[7] = fmaf(q, x[3]*x[12], g[7]);
    g[12] = fmaf(q, x[3]*x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 61 * C);
    g[3] = fmaf(q, x[7]*x[14], g[3]);
    g[7] = fmaf(q, x[3]*x[14], g[7]);
    g[14] = fmaf(q, x[3]*x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 62 * C);
    g[3] = fmaf(q, x[8]*x[13], g[3]);
    g[8] = fmaf(q, x[3]*x[13], g[8]);
    g[13] = fmaf(q, x[3]*x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 63 * C);
    g[3] = fmaf(q, x[8]*x[15], g[3]);
    g[8] = fmaf(q, x[3]*x[15], g[8]);
    g[15] = fmaf(q, x[3]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 64 * C);
    g[4] = fmaf(q, x[4]*x[6], g[4]);
    g[4] = fmaf(q, x[4]*x[6], g[4]);
    g[6] = fmaf(q, x[4]*x[4], g[6]);
  }
  { const float q = w * __ldg(cf + 65 * C);
    g[4] = fmaf(q, x[9]*x[13], g[4]);
    g[9] = fmaf(q, x[4]*x[13], g[9]);
    g[13] = fmaf(q, x[4]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 66 * C);
    g[4] = fmaf(q, x[10]*x[12], g[4]);
    g[10] = fmaf(q, x[4]*x[12], g[10]);
    g[12] = fmaf(q, x[4]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 67 * C);
    g[4] = fmaf(q, x[11]*x[13], g[4]);
    g[11] = fmaf(q, x[4]*x[13], g[11]);
    g[13] = fmaf(q, x[4]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 68 * C);
    g[4] = fmaf(q, x[11]*x[15], g[4]);
    g[11] = fmaf(q, x[4]*x[15], g[11]);
    g[15] = fmaf(q, x[4]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 69 * C);
    g[5] = fmaf(q, x[5]*x[6], g[5]);
    g[5] = fmaf(q, x[5]*x[6], g[5]);
    g[6] = fmaf(q, x[5]*x[5], g[6]);
  }
  { const float q = w * __ldg(cf + 70 * C);
    g[5] = fmaf(q, x[9]*x[14], g[5]);
    g[9] = fmaf(q, x[5]*x[14], g[9]);
    g[14] = fmaf(q, x[5]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 71 * C);
    g[5] = fmaf(q, x[10]*x[13], g[5]);
    g[10] = fmaf(q, x[5]*x[13], g[10]);
    g[13] = fmaf(q, x[5]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 72 * C);
    g[5] = fmaf(q, x[10]*x[15], g[5]);
    g[10] = fmaf(q, x[5]*x[15], g[10]);
    g[15] = fmaf(q, x[5]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 73 * C);
    g[5] = fmaf(q, x[11]*x[12], g[5]);
    g[11] = fmaf(q, x[5]*x[12], g[11]);
    g[12] = fmaf(q, x[5]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 74 * C);
    g[5] = fmaf(q, x[11]*x[14], g[5]);
    g[11] = fmaf(q, x[5]*x[14], g[11]);
    g[14] = fmaf(q, x[5]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 75 * C);
    g[6] = fmaf(q, x[6]*x[6], g[6]);
    g[6] = fmaf(q, x[6]*x[6], g[6]);
    g[6] = fmaf(q, x[6]*x[6], g[6]);
  }
  { const float q = w * __ldg(cf + 76 * C);
    g[6] = fmaf(q, x[7]*x[7], g[6]);
    g[7] = fmaf(q, x[6]*x[7], g[7]);
    g[7] = fmaf(q, x[6]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 77 * C);
    g[6] = fmaf(q, x[8]*x[8], g[6]);
    g[8] = fmaf(q, x[6]*x[8], g[8]);
    g[8] = fmaf(q, x[6]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 78 * C);
    g[6] = fmaf(q, x[9]*x[9], g[6]);
    g[9] = fmaf(q, x[6]*x[9], g[9]);
    g[9] = fmaf(q, x[6]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 79 * C);
    g[6] = fmaf(q, x[10]*x[10], g[6]);
    g[10] = fmaf(q, x[6]*x[10], g[10]);
    g[10] = fmaf(q, x[6]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 80 * C);
    g[6] = fmaf(q, x[11]*x[11], g[6]);
    g[11] = fmaf(q, x[6]*x[11], g[11]);
    g[11] = fmaf(q, x[6]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 81 * C);
    g[6] = fmaf(q, x[12]*x[12], g[6]);
    g[12] = fmaf(q, x[6]*x[12], g[12]);
    g[12] = fmaf(q, x[6]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 82 * C);
    g[6] = fmaf(q, x[13]*x[13], g[6]);
    g[13] = fmaf(q, x[6]*x[13], g[13]);
    g[13] = fmaf(q, x[6]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 83 * C);
    g[6] = fmaf(q, x[14]*x[14], g[6]);
    g[14] = fmaf(q, x[6]*x[14], g[14]);
    g[14] = fmaf(q, x[6]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 84 * C);
    g[6] = fmaf(q, x[15]*x[15], g[6]);
    g[15] = fmaf(q, x[6]*x[15], g[15]);
    g[15] = fmaf(q, x[6]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 85 * C);
    g[7] = fmaf(q, x[9]*x[10], g[7]);
    g[9] = fmaf(q, x[7]*x[10], g[9]);
    g[10] = fmaf(q, x[7]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 86 * C);
    g[7] = fmaf(q, x[10]*x[11], g[7]);
    g[10] = fmaf(q, x[7]*x[11], g[10]);
    g[11] = fmaf(q, x[7]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 87 * C);
    g[7] = fmaf(q, x[12]*x[13], g[7]);
    g[12] = fmaf(q, x[7]*x[13], g[12]);
    g[13] = fmaf(q, x[7]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 88 * C);
    g[7] = fmaf(q, x[13]*x[14], g[7]);
    g[13] = fmaf(q, x[7]*x[14], g[13]);
    g[14] = fmaf(q, x[7]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 89 * C);
    g[7] = fmaf(q, x[14]*x[15], g[7]);
    g[14] = fmaf(q, x[7]*x[15], g[14]);
    g[15] = fmaf(q, x[7]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 90 * C);
    g[8] = fmaf(q, x[9]*x[11], g[8]);
    g[9] = fmaf(q, x[8]*x[11], g[9]);
    g[11] = fmaf(q, x[8]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 91 * C);
    g[8] = fmaf(q, x[11]*x[11], g[8]);
    g[11] = fmaf(q, x[8]*x[11], g[11]);
    g[11] = fmaf(q, x[8]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 92 * C);
    g[8] = fmaf(q, x[12]*x[14], g[8]);
    g[12] = fmaf(q, x[8]*x[14], g[12]);
    g[14] = fmaf(q, x[8]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 93 * C);
    g[8] = fmaf(q, x[13]*x[13], g[8]);
    g[13] = fmaf(q, x[8]*x[13], g[13]);
    g[13] = fmaf(q, x[8]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 94 * C);
    g[8] = fmaf(q, x[13]*x[15], g[8]);
    g[13] = fmaf(q, x[8]*x[15], g[13]);
    g[15] = fmaf(q, x[8]*x[13], g[15]);
  }
}

__device__ __forceinline__ float value_LM7(const float* x, const float* __restrict__ cf, int C) {
  float f = 0.0f;
  f = fmaf(__ldg(cf + 0 * C), x[7], f);
  f = fmaf(__ldg(cf + 1 * C), x[0]*x[7], f);
  f = fmaf(__ldg(cf + 2 * C), x[1]*x[10], f);
  f = fmaf(__ldg(cf + 3 * C), x[2]*x[3], f);
  f = fmaf(__ldg(cf + 4 * C), x[2]*x[13], f);
  f = fmaf(__ldg(cf + 5 * C), x[3]*x[12], f);
  f = fmaf(__ldg(cf + 6 * C), x[3]*x[14], f);
  f = fmaf(__ldg(cf + 7 * C), x[4]*x[5], f);
  f = fmaf(__ldg(cf + 8 * C), x[6]*x[7], f);
  f = fmaf(__ldg(cf + 9 * C), x[7]*x[8], f);
  f = fmaf(__ldg(cf + 10 * C), x[9]*x[10], f);
  f = fmaf(__ldg(cf + 11 * C), x[10]*x[11], f);
  f = fmaf(__ldg(cf + 12 * C), x[12]*x[13], f);
  f = fmaf(__ldg(cf + 13 * C), x[13]*x[14], f);
  f = fmaf(__ldg(cf + 14 * C), x[14]*x[15], f);
  f = fmaf(__ldg(cf + 15 * C), x[0]*x[0]*x[7], f);
  f = fmaf(__ldg(cf + 16 * C), x[0]*x[1]*x[10], f);
  f = fmaf(__ldg(cf + 17 * C), x[0]*x[2]*x[3], f);
  f = fmaf(__ldg(cf + 18 * C), x[0]*x[2]*x[13], f);
  f = fmaf(__ldg(cf + 19 * C), x[0]*x[3]*x[12], f);
  f = fmaf(__ldg(cf + 20 * C), x[0]*x[3]*x[14], f);
  f = fmaf(__ldg(cf + 21 * C), x[0]*x[4]*x[5], f);
  f = fmaf(__ldg(cf + 22 * C), x[0]*x[6]*x[7], f);
  f = fmaf(__ldg(cf + 23 * C), x[0]*x[7]*x[8], f);
  f = fmaf(__ldg(cf + 24 * C), x[0]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 25 * C), x[0]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 26 * C), x[0]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 27 * C), x[0]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 28 * C), x[0]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 29 * C), x[1]*x[1]*x[7], f);
  f = fmaf(__ldg(cf + 30 * C), x[1]*x[2]*x[4], f);
  f = fmaf(__ldg(cf + 31 * C), x[1]*x[3]*x[5], f);
  f = fmaf(__ldg(cf + 32 * C), x[1]*x[4]*x[12], f);
  f = fmaf(__ldg(cf + 33 * C), x[1]*x[4]*x[14], f);
  f = fmaf(__ldg(cf + 34 * C), x[1]*x[5]*x[13], f);
  f = fmaf(__ldg(cf + 35 * C), x[1]*x[5]*x[15], f);
  f = fmaf(__ldg(cf + 36 * C), x[1]*x[6]*x[10], f);
  f = fmaf(__ldg(cf + 37 * C), x[1]*x[7]*x[9], f);
  f = fmaf(__ldg(cf + 38 * C), x[1]*x[7]*x[11], f);
  f = fmaf(__ldg(cf + 39 * C), x[1]*x[8]*x[10], f);
  f = fmaf(__ldg(cf + 40 * C), x[2]*x[2]*x[7], f);
  f = fmaf(__ldg(cf + 41 * C), x[2]*x[3]*x[6], f);
  f = fmaf(__ldg(cf + 42 * C), x[2]*x[3]*x[8], f);
  f = fmaf(__ldg(cf + 43 * C), x[2]*x[4]*x[9], f);
  f = fmaf(__ldg(cf + 44 * C), x[2]*x[4]*x[11], f);
  f = fmaf(__ldg(cf + 45 * C), x[2]*x[5]*x[10], f);
  f = fmaf(__ldg(cf + 46 * C), x[2]*x[6]*x[13], f);
  f = fmaf(__ldg(cf + 47 * C), x[2]*x[7]*x[12], f);
  f = fmaf(__ldg(cf + 48 * C), x[2]*x[7]*x[14], f);
  f = fmaf(__ldg(cf + 49 * C), x[2]*x[8]*x[13], f);
  f = fmaf(__ldg(cf + 50 * C), x[2]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 51 * C), x[3]*x[3]*x[7], f);
  f = fmaf(__ldg(cf + 52 * C), x[3]*x[4]*x[10], f);
  f = fmaf(__ldg(cf + 53 * C), x[3]*x[5]*x[9], f);
  f = fmaf(__ldg(cf + 54 * C), x[3]*x[5]*x[11], f);
  f = fmaf(__ldg(cf + 55 * C), x[3]*x[6]*x[12], f);
  f = fmaf(__ldg(cf + 56 * C), x[3]*x[6]*x[14], f);
  f = fmaf(__ldg(cf + 57 * C), x[3]*x[7]*x[13], f);
  f = fmaf(__ldg(cf + 58 * C), x[3]*x[7]*x[15], f);
  f = fmaf(__ldg(cf + 59 * C), x[3]*x[8]*x[12], f);
  f = fmaf(__ldg(cf + 60 * C), x[3]*x[8]*x[14], f);
  f = fmaf(__ldg(cf + 61 * C), x[4]*x[4]*x[7], f);
  f = fmaf(__ldg(cf + 62 * C), x[4]*x[9]*x[12], f);
  f = fmaf(__ldg(cf + 63 * C), x[4]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 64 * C), x[4]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 65 * C), x[4]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 66 * C), x[4]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 67 * C), x[4]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 68 * C), x[5]*x[5]*x[7], f);
  f = fmaf(__ldg(cf + 69 * C), x[5]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 70 * C), x[5]*x[10]*x[12], f);
  f = fmaf(__ldg(cf + 71 * C), x[5]*x[11]*x[13], f);
  f = fmaf(__ldg(cf + 72 * C), x[5]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 73 * C), x[6]*x[6]*x[7], f);
  f = fmaf(__ldg(cf + 74 * C), x[6]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 75 * C), x[6]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 76 * C), x[6]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 77 * C), x[6]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 78 * C), x[6]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 79 * C), x[7]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 80 * C), x[7]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 81 * C), x[7]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 82 * C), x[7]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 83 * C), x[7]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 84 * C), x[7]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 85 * C), x[7]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 86 * C), x[7]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 87 * C), x[7]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 88 * C), x[7]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 89 * C), x[7]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 90 * C), x[7]*x[15]*x[15], f);
  f = fmaf(__ldg(cf + 91 * C), x[8]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 92 * C), x[8]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 93 * C), x[8]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 94 * C), x[8]*x[12]*x[15], f);
  f = fmaf(__ldg(cf + 95 * C), x[8]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 96 * C), x[8]*x[14]*x[15], f);
  return f;
}

__device__ __forceinline__ void grad_LM7(const float* x, float w, const float* __restrict__ cf, int C, float* g) {
  { const float q = w * __ldg(cf + 0 * C);
    g[7] += q;
  }
  { const float q = w * __ldg(cf + 1 * C);
    g[0] = fmaf(q, x[7], g[0]);
    g[7] = fmaf(q, x[0], g[7]);
  }
  { const float q = w * __ldg(cf + 2 * C);
    g[1] = fmaf(q, x[10], g[1]);
    g[10] = fmaf(q, x[1], g[10]);
  }
  { const float q = w * __ldg(cf + 3 * C);
    g[2] = fmaf(q, x[3], g[2]);
    g[3] = fmaf(q, x[2], g[3]);
  }
  { const float q = w * __ldg(cf + 4 * C);
    g[2] = fmaf(q, x[13], g[2]);
    g[13] = fmaf(q, x[2], g[13]);
  }
  { const float q = w * __ldg(cf + 5 * C);
    g[3] = fmaf(q, x[12], g[3]);
    g[12] = fmaf(q, x[3], g[12]);
  }
  { const float q = w * __ldg(cf + 6 * C);
    g[3] = fmaf(q, x[14], g[3]);
    g[14] = fmaf(q, x[3], g[14]);
  }
  { const float q = w * __ldg(cf + 7 * C);
    g[4] = fmaf(q, x[5], g[4]);
    g[5] = fmaf(q, x[4], g[5]);
  }
  { const float q = w * __ldg(cf + 8 * C);
    g[6] = fmaf(q, x[7], g[6]);
    g[7] = fmaf(q, x[6], g[7]);
  }
  { const float q = w * __ldg(cf + 9 * C);
    g[7] = fmaf(q, x[8], g[7]);
    g[8] = fmaf(q, x[7], g[8]);
  }
  { const float q = w * __ldg(cf + 10 * C);
    g[9] = fmaf(q, x[10], g[9]);
    g[10] = fmaf(q, x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 11 * C);
    g[10] = fmaf(q, x[11], g[10]);
    g[11] = fmaf(q, x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 12 * C);
    g[12] = fmaf(q, x[13], g[12]);
    g[13] = fmaf(q, x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 13 * C);
    g[13] = fmaf(q, x[14], g[13]);
    g[14] = fmaf(q, x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 14 * C);
    g[14] = fmaf(q, x[15], g[14]);
    g[15] = fmaf(q, x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 15 * C);
    g[0] = fmaf(q, x[0]*x[7], g[0]);
    g[0] = fmaf(q, x[0]*x[7], g[0]);
    g[7] = fmaf(q, x[0]*x[0], g[7]);
  }
  { const float q = w * __ldg(cf + 16 * C);
    g[0] = fmaf(q, x[1]*x[10], g[0]);
    g[1] = fmaf(q, x[0]*x[10], g[1]);
    g[10] = fmaf(q, x[0]*x[1], g[10]);
  }
  { const float q = w * __ldg(cf + 17 * C);
    g[0] = fmaf(q, x[2]*x[3], g[0]);
    g[2] = fmaf(q, x[0]*x[3], g[2]);
    g[3] = fmaf(q, x[0]*x[2], g[3]);
  }
  { const float q = w * __ldg(cf + 18 * C);
    g[0] = fmaf(q, x[2]*x[13], g[0]);
    g[2] = fmaf(q, x[0]*x[13], g[2]);
    g[13] = fmaf(q, x[0]*x[2], g[13]);
  }
  { const float q = w * __ldg(cf + 19 * C);
    g[0] = fmaf(q, x[3]*x[12], g[0]);
    g[3] = fmaf(q, x[0]*x[12], g[3]);
    g[12] = fmaf(q, x[0]*x[3], g[12]);
  }
  { const float q = w * __ldg(cf + 20 * C);
    g[0] = fmaf(q, x[3]*x[14], g[0]);
    g[3] = fmaf(q, x[0]*x[14], g[3]);
    g[14] = fmaf(q, x[0]*x[3], g[14]);
  }
  { const float q = w * __ldg(cf + 21 * C);
    g[0] = fmaf(q, x[4]*x[5], g[0]);
    g[4] = fmaf(q, x[0]*x[5], g[4]);
    g[5] = fmaf(q, x[0]*x[4], g[5]);
  }
  { const float q = w * __ldg(cf + 22 * C);
    g[0] = fmaf(q, x[6]*x[7], g[0]);
    g[6] = fmaf(q, x[0]*x[7], g[6]);
    g[7] = fmaf(q, x[0]*x[6], g[7]);
  }
  { const float q = w * __ldg(cf + 23 * C);
    g[0] = fmaf(q, x[7]*x[8], g[0]);
    g[7] = fmaf(q, x[0]*x[8], g[7]);
    g[8] = fmaf(q, x[0]*x[7], g[8]);
  }
  { const float q = w * __ldg(cf + 24 * C);
    g[0] = fmaf(q, x[9]*x[10], g[0]);
    g[9] = fmaf(q, x[0]*x[10], g[9]);
    g[10] = fmaf(q, x[0]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 25 * C);
    g[0] = fmaf(q, x[10]*x[11], g[0]);
    g[10] = fmaf(q, x[0]*x[11], g[10]);
    g[11] = fmaf(q, x[0]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 26 * C);
    g[0] = fmaf(q, x[12]*x[13], g[0]);
    g[12] = fmaf(q, x[0]*x[13], g[12]);
    g[13] = fmaf(q, x[0]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 27 * C);
    g[0] = fmaf(q, x[13]*x[14], g[0]);
    g[13] = fmaf(q, x[0]*x[14], g[13]);
    g[14] = fmaf(q, x[0]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 28 * C);
    g[0] = fmaf(q, x[14]*x[15], g[0]);
    g[14] = fmaf(q, x[0]*x[15], g[14]);
    g[15] = fmaf(q, x[0]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 29 * C);
    g[1] = fmaf(q, x[1]*x[7], g[1]);
    g[1] = fmaf(q, x[1]*x[7], g[1]);
    g[7] = fmaf(q, x[1]*x[1], g[7]);
  }
  { const float q = w * __ldg(cf + 30 * C);
    g[1] = fmaf(q, x[2]*x[4], g[1]);
    g[2] = fmaf(q, x[1]*x[4], g[2]);
    g[4] = fmaf(q, x[1]*x[2], g[4]);
  }
  { const float q = w * __ldg(cf + 31 * C);
    g[1] = fmaf(q, x[3]*x[5], g[1]);
    g[3] = fmaf(q, x[1]*x[5], g[3]);
    g[5] = fmaf(q, x[1]*x[3], g[5]);
  }
  { const float q = w * __ldg(cf + 32 * C);
    g[1] = fmaf(q, x[4]*x[12], g[1]);
    g[4] = fmaf(q, x[1]*x[12], g[4]);
    g[12] = fmaf(q, x[1]*x[4], g[12]);
  }
  { const float q = w * __ldg(cf + 33 * C);
    g[1] = fmaf(q, x[4]*x[14], g[1]);
    g[4] = fmaf(q, x[1]*x[14], g[4]);
    g[14] = fmaf(q, x[1]*x[4], g[14]);
  }
  { const float q = w * __ldg(cf + 34 * C);
    g[1] = fmaf(q, x[5]*x[13], g[1]);
    g[5] = fmaf(q, x[1]*x[13], g[5]);
    g[13] = fmaf(q, x[1]*x[5], g[13]);
  }
  { const float q = w * __ldg(cf + 35 * C);
    g[1] = fmaf(q, x[5]*x[15], g[1]);
    g[5] = fmaf(q, x[1]*x[15], g[5]);
    g[15] = fmaf(q, x[1]*x[5], g[15]);
  }
  { const float q = w * __ldg(cf + 36 * C);
    g[1] = fmaf(q, x[6]*x[10], g[1]);
    g[6] = fmaf(q, x[1]*x[10], g[6]);
    g[10] = fmaf(q, x[1]*x[6], g[10]);
  }
  { const float q = w * __ldg(cf + 37 * C);
    g[1] = fmaf(q, x[7]*x[9], g[1]);
    g[7] = fmaf(q, x[1]*x[9], g[7]);
    g[9] = fmaf(q, x[1]*x[7], g[9]);
  }
  { const float q = w * __ldg(cf + 38 * C);
    g[1] = fmaf(q, x[7]*x[11], g[1]);
    g[7] = fmaf(q, x[1]*x[11], g[7]);
    g[11] = fmaf(q, x[1]*x[7], g[11]);
  }
  { const float q = w * __ldg(cf + 39 * C);
    g[1] = fmaf(q, x[8]*x[10], g[1]);
    g[8] = fmaf(q, x[1]*x[10], g[8]);
    g[10] = fmaf(q, x[1]*x[8], g[10]);
  }
  { const float q = w * __ldg(cf + 40 * C);
    g[2] = fmaf(q, x[2]*x[7], g[2]);
    g[2] = fmaf(q, x[2]*x[7], g[2]);
    g[7] = fmaf(q, x[2]*x[2], g[7]);
  }
  { const float q = w * __ldg(cf + 41 * C);
    g[2] = fmaf(q, x[3]*x[6], g[2]);
    g[3] = fmaf(q, x[2]*x[6], g[3]);
    g[6] = fmaf(q, x[2]*x[3], g[6]);
  }
  { const float q = w * __ldg(cf + 42 * C);
    g[2] = fmaf(q, x[3]*x[8], g[2]);
    g[3] = fmaf(q, x[2]*x[8], g[3]);
    g[8] = fmaf(q, x[2]*x[3], g[8]);
  }
  { const float q = w * __ldg(cf + 43 * C);
    g[2] = fmaf(q, x[4]*x[9], g[2]);
    g[4] = fmaf(q, x[2]*x[9], g[4]);
    g[9] = fmaf(q, x[2]*x[4], g[9]);
  }
  { const float q = w * __ldg(cf + 44 * C);
    g[2] = fmaf(q, x[4]*x[11], g[2]);
    g[4] = fmaf(q, x[2]*x[11], g[4]);
    g[11] = fmaf(q, x[2]*x[4], g[11]);
  }
  { const float q = w * __ldg(cf + 45 * C);
    g[2] = fmaf(q, x[5]*x[10], g[2]);
    g[5] = fmaf(q, x[2]*x[10], g[5]);
    g[10] = fmaf(q, x[2]*x[5], g[10]);
  }
  { const float q = w * __ldg(cf + 46 * C);
    g[2] = fmaf(q, x[6]*x[13], g[2]);
    g[6] = fmaf(q, x[2]*x[13], g[6]);
    g[13] = fmaf(q, x[2]*x[6], g[13]);
  }
  { const float q = w * __ldg(cf + 47 * C);
    g[2] = fmaf(q, x[7]*x[12], g[2]);
    g[7] = fmaf(q, x[2]*x[12], g[7]);
    g[12] = fmaf(q, x[2]*x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 48 * C);
    g[2] = fmaf(q, x[7]*x[14], g[2]);
    g[7] = fmaf(q, x[2]*x[14], g[7]);
    g[14] = fmaf(q, x[2]*x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 49 * C);
    g[2] = fmaf(q, x[8]*x[13], g[2]);
    g[8] = fmaf(q, x[2]*x[13], g[8]);
    g[13] = fmaf(q, x[2]*x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 50 * C);
    g[2] = fmaf(q, x[8]*x[15], g[2]);
    g[8] = fmaf(q, x[2]*x[15], g[8]);
    g[15] = fmaf(q, x[2]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 51 * C);
    g[3] = fmaf(q, x[3]*x[7], g[3]);
    g[3] = fmaf(q, x[3]*x[7], g[3]);
    g[7] = fmaf(q, x[3]*x[3], g[7]);
  }
  { const float q = w * __ldg(cf + 52 * C);
    g[3] = fmaf(q, x[4]*x[10], g[3]);
    g[4] = fmaf(q, x[3]*x[10], g[4]);
    g[10] = fmaf(q, x[3]*x[4], g[10]);
  }
  { const float q = w * __ldg(cf + 53 * C);
    g[3] = fmaf(q, x[5]*x[9], g[3]);
    g[5] = fmaf(q, x[3]*x[9], g[5]);
    g[9] = fmaf(q, x[3]*x[5], g[9]);
  }
  { const float q = w * __ldg(cf + 54 * C);
    g[3] = fmaf(q, x[5]*x[11], g[3]);
    g[5] = fmaf(q, x[3]*x[11], g[5]);
    g[11] = fmaf(q, x[3]*x[5], g[11]);
  }
  { const float q = w * __ldg(cf + 55 * C);
    g[3] = fmaf(q, x[6]*x[12], g[3]);
    g[6] = fmaf(q, x[3]*x[12], g[6]);
    g[12] = fmaf(q, x[3]*x[6], g[12]);
  }
  { const float q = w * __ldg(cf + 56 * C);
    g[3] = fmaf(q, x[6]*x[14], g[3]);
    g[6] = fmaf(q, x[3]*x[14], g[6]);
    g[14] = fmaf(q, x[3]*x[6], g[14]);
  }
  { const float q = w * __ldg(cf + 57 * C);
    g[3] = fmaf(q, x[7]*x[13], g[3]);
    g[7] = fmaf(q, x[3]*x[13], g[7]);
    g[13] = fmaf(q, x[3]*x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 58 * C);
    g[3] = fmaf(q, x[7]*x[15], g[3]);
    g[7] = fmaf(q, x[3]*x[15], g[7]);
    g[15] = fmaf(q, x[3]*x[7], g[15]);
  }
  { const float q = w * __ldg(cf + 59 * C);
    g[3] = fmaf(q, x[8]*x[12], g[3]);
    g[8] = fmaf(q, x[3]*x[12], g[8]);
    g[12] = fmaf(q, x[3]*x[8], g[12]);
  }
  { const float q = w * __ldg(cf + 60 * C);
    g[3] = fmaf(q, x[8]*x[14], g[3]);
    g[8] = fmaf(q, x[3]*x[14], g[8]);
    g[14] = fmaf(q, x[3]*x[8], g[14]);
  }
  { const float q = w * __ldg(cf + 61 * C);
    g[4] = fmaf(q, x[4]*x[7], g[4]);
    g[4] = fmaf(q, x[4]*x[7], g[4]);
    g[7] = fmaf(q, x[4]*x[4], g[7]);
  }
  { const float q = w * __ldg(cf + 62 * C);
    g[4] = fmaf(q, x[9]*x[12], g[4]);
    g[9] = fmaf(q, x[4]*x[12], g[9]);
    g[12] = fmaf(q, x[4]*x[9], g[12]);
  }
  { const float q = w * __ldg(cf + 63 * C);
    g[4] = fmaf(q, x[9]*x[14], g[4]);
    g[9] = fmaf(q, x[4]*x[14], g[9]);
    g[14] = fmaf(q, x[4]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 64 * C);
    g[4] = fmaf(q, x[10]*x[13], g[4]);
    g[10] = fmaf(q, x[4]*x[13], g[10]);
    g[13] = fmaf(q, x[4]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 65 * C);
    g[4] = fmaf(q, x[10]*x[15], g[4]);
    g[10] = fmaf(q, x[4]*x[15], g[10]);
    g[15] = fmaf(q, x[4]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 66 * C);
    g[4] = fmaf(q, x[11]*x[12], g[4]);
    g[11] = fmaf(q, x[4]*x[12], g[11]);
    g[12] = fmaf(q, x[4]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 67 * C);
    g[4] = fmaf(q, x[11]*x[14], g[4]);
    g[11] = fmaf(q, x[4]*x[14], g[11]);
    g[14] = fmaf(q, x[4]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 68 * C);
    g[5] = fmaf(q, x[5]*x[7], g[5]);
    g[5] = fmaf(q, x[5]*x[7], g[5]);
    g[7] = fmaf(q, x[5]*x[5], g[7]);
  }
  { const float q = w * __ldg(cf + 69 * C);
    g[5] = fmaf(q, x[9]*x[13], g[5]);
    g[9] = fmaf(q, x[5]*x[13], g[9]);
    g[13] = fmaf(q, x[5]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 70 * C);
    g[5] = fmaf(q, x[10]*x[12], g[5]);
    g[10] = fmaf(q, x[5]*x[12], g[10]);
    g[12] = fmaf(q, x[5]*x[10], g[12]);
  }
  { const float q = w * __ldg(cf + 71 * C);
    g[5] = fmaf(q, x[11]*x[13], g[5]);
    g[11] = fmaf(q, x[5]*x[13], g[11]);
    g[13] = fmaf(q, x[5]*x[11], g[13]);
  }
  { const float q = w * __ldg(cf + 72 * C);
    g[5] = fmaf(q, x[11]*x[15], g[5]);
    g[11] = fmaf(q, x[5]*x[15], g[11]);
    g[15] = fmaf(q, x[5]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 73 * C);
    g[6] = fmaf(q, x[6]*x[7], g[6]);
    g[6] = fmaf(q, x[6]*x[7], g[6]);
    g[7] = fmaf(q, x[6]*x[6], g[7]);
  }
  { const float q = w * __ldg(cf + 74 * C);
    g[6] = fmaf(q, x[9]*x[10], g[6]);
    g[9] = fmaf(q, x[6]*x[10], g[9]);
    g[10] = fmaf(q, x[6]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 75 * C);
    g[6] = fmaf(q, x[10]*x[11], g[6]);
    g[10] = fmaf(q, x[6]*x[11], g[10]);
    g[11] = fmaf(q, x[6]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 76 * C);
    g[6] = fmaf(q, x[12]*x[13], g[6]);
    g[12] = fmaf(q, x[6]*x[13], g[12]);
    g[13] = fmaf(q, x[6]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 77 * C);
    g[6] = fmaf(q, x[13]*x[14], g[6]);
    g[13] = fmaf(q, x[6]*x[14], g[13]);
    g[14] = fmaf(q, x[6]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 78 * C);
    g[6] = fmaf(q, x[14]*x[15], g[6]);
    g[14] = fmaf(q, x[6]*x[15], g[14]);
    g[15] = fmaf(q, x[6]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 79 * C);
    g[7] = fmaf(q, x[7]*x[7], g[7]);
    g[7] = fmaf(q, x[7]*x[7], g[7]);
    g[7] = fmaf(q, x[7]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 80 * C);
    g[7] = fmaf(q, x[8]*x[8], g[7]);
    g[8] = fmaf(q, x[7]*x[8], g[8]);
    g[8] = fmaf(q, x[7]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 81 * C);
    g[7] = fmaf(q, x[9]*x[9], g[7]);
    g[9] = fmaf(q, x[7]*x[9], g[9]);
    g[9] = fmaf(q, x[7]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 82 * C);
    g[7] = fmaf(q, x[9]*x[11], g[7]);
    g[9] = fmaf(q, x[7]*x[11], g[9]);
    g[11] = fmaf(q, x[7]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 83 * C);
    g[7] = fmaf(q, x[10]*x[10], g[7]);
    g[10] = fmaf(q, x[7]*x[10], g[10]);
    g[10] = fmaf(q, x[7]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 84 * C);
    g[7] = fmaf(q, x[11]*x[11], g[7]);
    g[11] = fmaf(q, x[7]*x[11], g[11]);
    g[11] = fmaf(q, x[7]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 85 * C);
    g[7] = fmaf(q, x[12]*x[12], g[7]);
    g[12] = fmaf(q, x[7]*x[12], g[12]);
    g[12] = fmaf(q, x[7]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 86 * C);
    g[7] = fmaf(q, x[12]*x[14], g[7]);
    g[12] = fmaf(q, x[7]*x[14], g[12]);
    g[14] = fmaf(q, x[7]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 87 * C);
    g[7] = fmaf(q, x[13]*x[13], g[7]);
    g[13] = fmaf(q, x[7]*x[13], g[13]);
    g[13] = fmaf(q, x[7]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 88 * C);
    g[7] = fmaf(q, x[13]*x[15], g[7]);
    g[13] = fmaf(q, x[7]*x[15], g[13]);
    g[15] = fmaf(q, x[7]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 89 * C);
    g[7] = fmaf(q, x[14]*x[14], g[7]);
    g[14] = fmaf(q, x[7]*x[14], g[14]);
    g[14] = fmaf(q, x[7]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 90 * C);
    g[7] = fmaf(q, x[15]*x[15], g[7]);
    g[15] = fmaf(q, x[7]*x[15], g[15]);
    g[15] = fmaf(q, x[7]*x[15], g[15]);
  }
  { const float q = w * __ldg(cf + 91 * C);
    g[8] = fmaf(q, x[9]*x[10], g[8]);
    g[9] = fmaf(q, x[8]*x[10], g[9]);
    g[10] = fmaf(q, x[8]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 92 * C);
    g[8] = fmaf(q, x[10]*x[11], g[8]);
    g[10] = fmaf(q, x[8]*x[11], g[10]);
    g[11] = fmaf(q, x[8]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 93 * C);
    g[8] = fmaf(q, x[12]*x[13], g[8]);
    g[12] = fmaf(q, x[8]*x[13], g[12]);
    g[13] = fmaf(q, x[8]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 94 * C);
    g[8] = fmaf(q, x[12]*x[15], g[8]);
    g[12] = fmaf(q, x[8]*x[15], g[12]);
    g[15] = fmaf(q, x[8]*x[12], g[15]);
  }
  { const float q = w * __ldg(cf + 95 * C);
    g[8] = fmaf(q, x[13]*x[14], g[8]);
    g[13] = fmaf(q, x[8]*x[14], g[13]);
    g[14] = fmaf(q, x[8]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 96 * C);
    g[8] = fmaf(q, x[14]*x[15], g[8]);
    g[14] = fmaf(q, x[8]*x[15], g[14]);
    g[15] = fmaf(q, x[8]*x[14], g[15]);
  }
}

__device__ __forceinline__ float value_LM8(const float* x, const float* __restrict__ cf, int C) {
  float f = 0.0f;
  f = fmaf(__ldg(cf + 0 * C), x[8], f);
  f = fmaf(__ldg(cf + 1 * C), x[0]*x[8], f);
  f = fmaf(__ldg(cf + 2 * C), x[1]*x[1], f);
  f = fmaf(__ldg(cf + 3 * C), x[1]*x[9], f);
  f = fmaf(__ldg(cf + 4 * C), x[1]*x[11], f);
  f = fmaf(__ldg(cf + 5 * C), x[2]*x[14], f);
  f = fmaf(__ldg(cf + 6 * C), x[3]*x[3], f);
  f = fmaf(__ldg(cf + 7 * C), x[3]*x[13], f);
  f = fmaf(__ldg(cf + 8 * C), x[3]*x[15], f);
  f = fmaf(__ldg(cf + 9 * C), x[5]*x[5], f);
  f = fmaf(__ldg(cf + 10 * C), x[6]*x[8], f);
  f = fmaf(__ldg(cf + 11 * C), x[7]*x[7], f);
  f = fmaf(__ldg(cf + 12 * C), x[9]*x[11], f);
  f = fmaf(__ldg(cf + 13 * C), x[11]*x[11], f);
  f = fmaf(__ldg(cf + 14 * C), x[12]*x[14], f);
  f = fmaf(__ldg(cf + 15 * C), x[13]*x[13], f);
  f = fmaf(__ldg(cf + 16 * C), x[13]*x[15], f);
  f = fmaf(__ldg(cf + 17 * C), x[0]*x[0]*x[8], f);
  f = fmaf(__ldg(cf + 18 * C), x[0]*x[1]*x[1], f);
  f = fmaf(__ldg(cf + 19 * C), x[0]*x[1]*x[9], f);
  f = fmaf(__ldg(cf + 20 * C), x[0]*x[1]*x[11], f);
  f = fmaf(__ldg(cf + 21 * C), x[0]*x[2]*x[14], f);
  f = fmaf(__ldg(cf + 22 * C), x[0]*x[3]*x[3], f);
  f = fmaf(__ldg(cf + 23 * C), x[0]*x[3]*x[13], f);
  f = fmaf(__ldg(cf + 24 * C), x[0]*x[3]*x[15], f);
  f = fmaf(__ldg(cf + 25 * C), x[0]*x[5]*x[5], f);
  f = fmaf(__ldg(cf + 26 * C), x[0]*x[6]*x[8], f);
  f = fmaf(__ldg(cf + 27 * C), x[0]*x[7]*x[7], f);
  f = fmaf(__ldg(cf + 28 * C), x[0]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 29 * C), x[0]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 30 * C), x[0]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 31 * C), x[0]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 32 * C), x[0]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 33 * C), x[1]*x[1]*x[6], f);
  f = fmaf(__ldg(cf + 34 * C), x[1]*x[1]*x[8], f);
  f = fmaf(__ldg(cf + 35 * C), x[1]*x[2]*x[5], f);
  f = fmaf(__ldg(cf + 36 * C), x[1]*x[4]*x[13], f);
  f = fmaf(__ldg(cf + 37 * C), x[1]*x[4]*x[15], f);
  f = fmaf(__ldg(cf + 38 * C), x[1]*x[5]*x[12], f);
  f = fmaf(__ldg(cf + 39 * C), x[1]*x[5]*x[14], f);
  f = fmaf(__ldg(cf + 40 * C), x[1]*x[6]*x[9], f);
  f = fmaf(__ldg(cf + 41 * C), x[1]*x[6]*x[11], f);
  f = fmaf(__ldg(cf + 42 * C), x[1]*x[7]*x[10], f);
  f = fmaf(__ldg(cf + 43 * C), x[1]*x[8]*x[9], f);
  f = fmaf(__ldg(cf + 44 * C), x[1]*x[8]*x[11], f);
  f = fmaf(__ldg(cf + 45 * C), x[2]*x[2]*x[8], f);
  f = fmaf(__ldg(cf + 46 * C), x[2]*x[3]*x[7], f);
  f = fmaf(__ldg(cf + 47 * C), x[2]*x[5]*x[9], f);
  f = fmaf(__ldg(cf + 48 * C), x[2]*x[5]*x[11], f);
  f = fmaf(__ldg(cf + 49 * C), x[2]*x[6]*x[14], f);
  f = fmaf(__ldg(cf + 50 * C), x[2]*x[7]*x[13], f);
  f = fmaf(__ldg(cf + 51 * C), x[2]*x[7]*x[15], f);
  f = fmaf(__ldg(cf + 52 * C), x[2]*x[8]*x[12], f);
  f = fmaf(__ldg(cf + 53 * C), x[3]*x[3]*x[6], f);
  f = fmaf(__ldg(cf + 54 * C), x[3]*x[3]*x[8], f);
  f = fmaf(__ldg(cf + 55 * C), x[3]*x[4]*x[9], f);
  f = fmaf(__ldg(cf + 56 * C), x[3]*x[4]*x[11], f);
  f = fmaf(__ldg(cf + 57 * C), x[3]*x[5]*x[10], f);
  f = fmaf(__ldg(cf + 58 * C), x[3]*x[6]*x[13], f);
  f = fmaf(__ldg(cf + 59 * C), x[3]*x[6]*x[15], f);
  f = fmaf(__ldg(cf + 60 * C), x[3]*x[7]*x[12], f);
  f = fmaf(__ldg(cf + 61 * C), x[3]*x[7]*x[14], f);
  f = fmaf(__ldg(cf + 62 * C), x[3]*x[8]*x[13], f);
  f = fmaf(__ldg(cf + 63 * C), x[3]*x[8]*x[15], f);
  f = fmaf(__ldg(cf + 64 * C), x[4]*x[4]*x[8], f);
  f = fmaf(__ldg(cf + 65 * C), x[4]*x[9]*x[13], f);
  f = fmaf(__ldg(cf + 66 * C), x[4]*x[10]*x[14], f);
  f = fmaf(__ldg(cf + 67 * C), x[4]*x[11]*x[15], f);
  f = fmaf(__ldg(cf + 68 * C), x[5]*x[5]*x[8], f);
  f = fmaf(__ldg(cf + 69 * C), x[5]*x[9]*x[12], f);
  f = fmaf(__ldg(cf + 70 * C), x[5]*x[9]*x[14], f);
  f = fmaf(__ldg(cf + 71 * C), x[5]*x[10]*x[13], f);
  f = fmaf(__ldg(cf + 72 * C), x[5]*x[10]*x[15], f);
  f = fmaf(__ldg(cf + 73 * C), x[5]*x[11]*x[12], f);
  f = fmaf(__ldg(cf + 74 * C), x[5]*x[11]*x[14], f);
  f = fmaf(__ldg(cf + 75 * C), x[6]*x[6]*x[8], f);
  f = fmaf(__ldg(cf + 76 * C), x[6]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 77 * C), x[6]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 78 * C), x[6]*x[12]*x[14], f);
  f = fmaf(__ldg(cf + 79 * C), x[6]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 80 * C), x[6]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 81 * C), x[7]*x[7]*x[8], f);
  f = fmaf(__ldg(cf + 82 * C), x[7]*x[9]*x[10], f);
  f = fmaf(__ldg(cf + 83 * C), x[7]*x[10]*x[11], f);
  f = fmaf(__ldg(cf + 84 * C), x[7]*x[12]*x[13], f);
  f = fmaf(__ldg(cf + 85 * C), x[7]*x[12]*x[15], f);
  f = fmaf(__ldg(cf + 86 * C), x[7]*x[13]*x[14], f);
  f = fmaf(__ldg(cf + 87 * C), x[7]*x[14]*x[15], f);
  f = fmaf(__ldg(cf + 88 * C), x[8]*x[8]*x[8], f);
  f = fmaf(__ldg(cf + 89 * C), x[8]*x[9]*x[9], f);
  f = fmaf(__ldg(cf + 90 * C), x[8]*x[9]*x[11], f);
  f = fmaf(__ldg(cf + 91 * C), x[8]*x[10]*x[10], f);
  f = fmaf(__ldg(cf + 92 * C), x[8]*x[11]*x[11], f);
  f = fmaf(__ldg(cf + 93 * C), x[8]*x[12]*x[12], f);
  f = fmaf(__ldg(cf + 94 * C), x[8]*x[13]*x[13], f);
  f = fmaf(__ldg(cf + 95 * C), x[8]*x[13]*x[15], f);
  f = fmaf(__ldg(cf + 96 * C), x[8]*x[14]*x[14], f);
  f = fmaf(__ldg(cf + 97 * C), x[8]*x[15]*x[15], f);
  return f;
}

__device__ __forceinline__ void grad_LM8(const float* x, float w, const float* __restrict__ cf, int C, float* g) {
  { const float q = w * __ldg(cf + 0 * C);
    g[8] += q;
  }
  { const float q = w * __ldg(cf + 1 * C);
    g[0] = fmaf(q, x[8], g[0]);
    g[8] = fmaf(q, x[0], g[8]);
  }
  { const float q = w * __ldg(cf + 2 * C);
    g[1] = fmaf(q, x[1], g[1]);
    g[1] = fmaf(q, x[1], g[1]);
  }
  { const float q = w * __ldg(cf + 3 * C);
    g[1] = fmaf(q, x[9], g[1]);
    g[9] = fmaf(q, x[1], g[9]);
  }
  { const float q = w * __ldg(cf + 4 * C);
    g[1] = fmaf(q, x[11], g[1]);
    g[11] = fmaf(q, x[1], g[11]);
  }
  { const float q = w * __ldg(cf + 5 * C);
    g[2] = fmaf(q, x[14], g[2]);
    g[14] = fmaf(q, x[2], g[14]);
  }
  { const float q = w * __ldg(cf + 6 * C);
    g[3] = fmaf(q, x[3], g[3]);
    g[3] = fmaf(q, x[3], g[3]);
  }
  { const float q = w * __ldg(cf + 7 * C);
    g[3] = fmaf(q, x[13], g[3]);
    g[13] = fmaf(q, x[3], g[13]);
  }
  { const float q = w * __ldg(cf + 8 * C);
    g[3] = fmaf(q, x[15], g[3]);
    g[15] = fmaf(q, x[3], g[15]);
  }
  { const float q = w * __ldg(cf + 9 * C);
    g[5] = fmaf(q, x[5], g[5]);
    g[5] = fmaf(q, x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 10 * C);
    g[6] = fmaf(q, x[8], g[6]);
    g[8] = fmaf(q, x[6], g[8]);
  }
  { const float q = w * __ldg(cf + 11 * C);
    g[7] = fmaf(q, x[7], g[7]);
    g[7] = fmaf(q, x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 12 * C);
    g[9] = fmaf(q, x[11], g[9]);
    g[11] = fmaf(q, x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 13 * C);
    g[11] = fmaf(q, x[11], g[11]);
    g[11] = fmaf(q, x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 14 * C);
    g[12] = fmaf(q, x[14], g[12]);
    g[14] = fmaf(q, x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 15 * C);
    g[13] = fmaf(q, x[13], g[13]);
    g[13] = fmaf(q, x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 16 * C);
    g[13] = fmaf(q, x[15], g[13]);
    g[15] = fmaf(q, x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 17 * C);
    g[0] = fmaf(q, x[0]*x[8], g[0]);
    g[0] = fmaf(q, x[0]*x[8], g[0]);
    g[8] = fmaf(q, x[0]*x[0], g[8]);
  }
  { const float q = w * __ldg(cf + 18 * C);
    g[0] = fmaf(q, x[1]*x[1], g[0]);
    g[1] = fmaf(q, x[0]*x[1], g[1]);
    g[1] = fmaf(q, x[0]*x[1], g[1]);
  }
  { const float q = w * __ldg(cf + 19 * C);
    g[0] = fmaf(q, x[1]*x[9], g[0]);
    g[1] = fmaf(q, x[0]*x[9], g[1]);
    g[9] = fmaf(q, x[0]*x[1], g[9]);
  }
  { const float q = w * __ldg(cf + 20 * C);
    g[0] = fmaf(q, x[1]*x[11], g[0]);
    g[1] = fmaf(q, x[0]*x[11], g[1]);
    g[11] = fmaf(q, x[0]*x[1], g[11]);
  }
  { const float q = w * __ldg(cf + 21 * C);
    g[0] = fmaf(q, x[2]*x[14], g[0]);
    g[2] = fmaf(q, x[0]*x[14], g[2]);
    g[14] = fmaf(q, x[0]*x[2], g[14]);
  }
  { const float q = w * __ldg(cf + 22 * C);
    g[0] = fmaf(q, x[3]*x[3], g[0]);
    g[3] = fmaf(q, x[0]*x[3], g[3]);
    g[3] = fmaf(q, x[0]*x[3], g[3]);
  }
  { const float q = w * __ldg(cf + 23 * C);
    g[0] = fmaf(q, x[3]*x[13], g[0]);
    g[3] = fmaf(q, x[0]*x[13], g[3]);
    g[13] = fmaf(q, x[0]*x[3], g[13]);
  }
  { const float q = w * __ldg(cf + 24 * C);
    g[0] = fmaf(q, x[3]*x[15], g[0]);
    g[3] = fmaf(q, x[0]*x[15], g[3]);
    g[15] = fmaf(q, x[0]*x[3], g[15]);
  }
  { const float q = w * __ldg(cf + 25 * C);
    g[0] = fmaf(q, x[5]*x[5], g[0]);
    g[5] = fmaf(q, x[0]*x[5], g[5]);
    g[5] = fmaf(q, x[0]*x[5], g[5]);
  }
  { const float q = w * __ldg(cf + 26 * C);
    g[0] = fmaf(q, x[6]*x[8], g[0]);
    g[6] = fmaf(q, x[0]*x[8], g[6]);
    g[8] = fmaf(q, x[0]*x[6], g[8]);
  }
  { const float q = w * __ldg(cf + 27 * C);
    g[0] = fmaf(q, x[7]*x[7], g[0]);
    g[7] = fmaf(q, x[0]*x[7], g[7]);
    g[7] = fmaf(q, x[0]*x[7], g[7]);
  }
  { const float q = w * __ldg(cf + 28 * C);
    g[0] = fmaf(q, x[9]*x[11], g[0]);
    g[9] = fmaf(q, x[0]*x[11], g[9]);
    g[11] = fmaf(q, x[0]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 29 * C);
    g[0] = fmaf(q, x[11]*x[11], g[0]);
    g[11] = fmaf(q, x[0]*x[11], g[11]);
    g[11] = fmaf(q, x[0]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 30 * C);
    g[0] = fmaf(q, x[12]*x[14], g[0]);
    g[12] = fmaf(q, x[0]*x[14], g[12]);
    g[14] = fmaf(q, x[0]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 31 * C);
    g[0] = fmaf(q, x[13]*x[13], g[0]);
    g[13] = fmaf(q, x[0]*x[13], g[13]);
    g[13] = fmaf(q, x[0]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 32 * C);
    g[0] = fmaf(q, x[13]*x[15], g[0]);
    g[13] = fmaf(q, x[0]*x[15], g[13]);
    g[15] = fmaf(q, x[0]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 33 * C);
    g[1] = fmaf(q, x[1]*x[6], g[1]);
    g[1] = fmaf(q, x[1]*x[6], g[1]);
    g[6] = fmaf(q, x[1]*x[1], g[6]);
  }
  { const float q = w * __ldg(cf + 34 * C);
    g[1] = fmaf(q, x[1]*x[8], g[1]);
    g[1] = fmaf(q, x[1]*x[8], g[1]);
    g[8] = fmaf(q, x[1]*x[1], g[8]);
  }
  { const float q = w * __ldg(cf + 35 * C);
    g[1] = fmaf(q, x[2]*x[5], g[1]);
    g[2] = fmaf(q, x[1]*x[5], g[2]);
    g[5] = fmaf(q, x[1]*x[2], g[5]);
  }
  { const float q = w * __ldg(cf + 36 * C);
    g[1] = fmaf(q, x[4]*x[13], g[1]);
    g[4] = fmaf(q, x[1]*x[13], g[4]);
    g[13] = fmaf(q, x[1]*x[4], g[13]);
  }
  { const float q = w * __ldg(cf + 37 * C);
    g[1] = fmaf(q, x[4]*x[15], g[1]);
    g[4] = fmaf(q, x[1]*x[15], g[4]);
    g[15] = fmaf(q, x[1]*x[4], g[15]);
  }
  { const float q = w * __ldg(cf + 38 * C);
    g[1] = fmaf(q, x[5]*x[12], g[1]);
    g[5] = fmaf(q, x[1]*x[12], g[5]);
    g[12] = fmaf(q, x[1]*x[5], g[12]);
  }
  { const float q = w * __ldg(cf + 39 * C);
    g[1] = fmaf(q, x[5]*x[14], g[1]);
    g[5] = fmaf(q, x[1]*x[14], g[5]);
    g[14] = fmaf(q, x[1]*x[5], g[14]);
  }
  { const float q = w * __ldg(cf + 40 * C);
    g[1] = fmaf(q, x[6]*x[9], g[1]);
    g[6] = fmaf(q, x[1]*x[9], g[6]);
    g[9] = fmaf(q, x[1]*x[6], g[9]);
  }
  { const float q = w * __ldg(cf + 41 * C);
    g[1] = fmaf(q, x[6]*x[11], g[1]);
    g[6] = fmaf(q, x[1]*x[11], g[6]);
    g[11] = fmaf(q, x[1]*x[6], g[11]);
  }
  { const float q = w * __ldg(cf + 42 * C);
    g[1] = fmaf(q, x[7]*x[10], g[1]);
    g[7] = fmaf(q, x[1]*x[10], g[7]);
    g[10] = fmaf(q, x[1]*x[7], g[10]);
  }
  { const float q = w * __ldg(cf + 43 * C);
    g[1] = fmaf(q, x[8]*x[9], g[1]);
    g[8] = fmaf(q, x[1]*x[9], g[8]);
    g[9] = fmaf(q, x[1]*x[8], g[9]);
  }
  { const float q = w * __ldg(cf + 44 * C);
    g[1] = fmaf(q, x[8]*x[11], g[1]);
    g[8] = fmaf(q, x[1]*x[11], g[8]);
    g[11] = fmaf(q, x[1]*x[8], g[11]);
  }
  { const float q = w * __ldg(cf + 45 * C);
    g[2] = fmaf(q, x[2]*x[8], g[2]);
    g[2] = fmaf(q, x[2]*x[8], g[2]);
    g[8] = fmaf(q, x[2]*x[2], g[8]);
  }
  { const float q = w * __ldg(cf + 46 * C);
    g[2] = fmaf(q, x[3]*x[7], g[2]);
    g[3] = fmaf(q, x[2]*x[7], g[3]);
    g[7] = fmaf(q, x[2]*x[3], g[7]);
  }
  { const float q = w * __ldg(cf + 47 * C);
    g[2] = fmaf(q, x[5]*x[9], g[2]);
    g[5] = fmaf(q, x[2]*x[9], g[5]);
    g[9] = fmaf(q, x[2]*x[5], g[9]);
  }
  { const float q = w * __ldg(cf + 48 * C);
    g[2] = fmaf(q, x[5]*x[11], g[2]);
    g[5] = fmaf(q, x[2]*x[11], g[5]);
    g[11] = fmaf(q, x[2]*x[5], g[11]);
  }
  { const float q = w * __ldg(cf + 49 * C);
    g[2] = fmaf(q, x[6]*x[14], g[2]);
    g[6] = fmaf(q, x[2]*x[14], g[6]);
    g[14] = fmaf(q, x[2]*x[6], g[14]);
  }
  { const float q = w * __ldg(cf + 50 * C);
    g[2] = fmaf(q, x[7]*x[13], g[2]);
    g[7] = fmaf(q, x[2]*x[13], g[7]);
    g[13] = fmaf(q, x[2]*x[7], g[13]);
  }
  { const float q = w * __ldg(cf + 51 * C);
    g[2] = fmaf(q, x[7]*x[15], g[2]);
    g[7] = fmaf(q, x[2]*x[15], g[7]);
    g[15] = fmaf(q, x[2]*x[7], g[15]);
  }
  { const float q = w * __ldg(cf + 52 * C);
    g[2] = fmaf(q, x[8]*x[12], g[2]);
    g[8] = fmaf(q, x[2]*x[12], g[8]);
    g[12] = fmaf(q, x[2]*x[8], g[12]);
  }
  { const float q = w * __ldg(cf + 53 * C);
    g[3] = fmaf(q, x[3]*x[6], g[3]);
    g[3] = fmaf(q, x[3]*x[6], g[3]);
    g[6] = fmaf(q, x[3]*x[3], g[6]);
  }
  { const float q = w * __ldg(cf + 54 * C);
    g[3] = fmaf(q, x[3]*x[8], g[3]);
    g[3] = fmaf(q, x[3]*x[8], g[3]);
    g[8] = fmaf(q, x[3]*x[3], g[8]);
  }
  { const float q = w * __ldg(cf + 55 * C);
    g[3] = fmaf(q, x[4]*x[9], g[3]);
    g[4] = fmaf(q, x[3]*x[9], g[4]);
    g[9] = fmaf(q, x[3]*x[4], g[9]);
  }
  { const float q = w * __ldg(cf + 56 * C);
    g[3] = fmaf(q, x[4]*x[11], g[3]);
    g[4] = fmaf(q, x[3]*x[11], g[4]);
    g[11] = fmaf(q, x[3]*x[4], g[11]);
  }
  { const float q = w * __ldg(cf + 57 * C);
    g[3] = fmaf(q, x[5]*x[10], g[3]);
    g[5] = fmaf(q, x[3]*x[10], g[5]);
    g[10] = fmaf(q, x[3]*x[5], g[10]);
  }
  { const float q = w * __ldg(cf + 58 * C);
    g[3] = fmaf(q, x[6]*x[13], g[3]);
    g[6] = fmaf(q, x[3]*x[13], g[6]);
    g[13] = fmaf(q, x[3]*x[6], g[13]);
  }
  { const float q = w * __ldg(cf + 59 * C);
    g[3] = fmaf(q, x[6]*x[15], g[3]);
    g[6] = fmaf(q, x[3]*x[15], g[6]);
    g[15] = fmaf(q, x[3]*x[6], g[15]);
  }
  { const float q = w * __ldg(cf + 60 * C);
    g[3] = fmaf(q, x[7]*x[12], g[3]);
    g[7] = fmaf(q, x[3]*x[12], g[7]);
    g[12] = fmaf(q, x[3]*x[7], g[12]);
  }
  { const float q = w * __ldg(cf + 61 * C);
    g[3] = fmaf(q, x[7]*x[14], g[3]);
    g[7] = fmaf(q, x[3]*x[14], g[7]);
    g[14] = fmaf(q, x[3]*x[7], g[14]);
  }
  { const float q = w * __ldg(cf + 62 * C);
    g[3] = fmaf(q, x[8]*x[13], g[3]);
    g[8] = fmaf(q, x[3]*x[13], g[8]);
    g[13] = fmaf(q, x[3]*x[8], g[13]);
  }
  { const float q = w * __ldg(cf + 63 * C);
    g[3] = fmaf(q, x[8]*x[15], g[3]);
    g[8] = fmaf(q, x[3]*x[15], g[8]);
    g[15] = fmaf(q, x[3]*x[8], g[15]);
  }
  { const float q = w * __ldg(cf + 64 * C);
    g[4] = fmaf(q, x[4]*x[8], g[4]);
    g[4] = fmaf(q, x[4]*x[8], g[4]);
    g[8] = fmaf(q, x[4]*x[4], g[8]);
  }
  { const float q = w * __ldg(cf + 65 * C);
    g[4] = fmaf(q, x[9]*x[13], g[4]);
    g[9] = fmaf(q, x[4]*x[13], g[9]);
    g[13] = fmaf(q, x[4]*x[9], g[13]);
  }
  { const float q = w * __ldg(cf + 66 * C);
    g[4] = fmaf(q, x[10]*x[14], g[4]);
    g[10] = fmaf(q, x[4]*x[14], g[10]);
    g[14] = fmaf(q, x[4]*x[10], g[14]);
  }
  { const float q = w * __ldg(cf + 67 * C);
    g[4] = fmaf(q, x[11]*x[15], g[4]);
    g[11] = fmaf(q, x[4]*x[15], g[11]);
    g[15] = fmaf(q, x[4]*x[11], g[15]);
  }
  { const float q = w * __ldg(cf + 68 * C);
    g[5] = fmaf(q, x[5]*x[8], g[5]);
    g[5] = fmaf(q, x[5]*x[8], g[5]);
    g[8] = fmaf(q, x[5]*x[5], g[8]);
  }
  { const float q = w * __ldg(cf + 69 * C);
    g[5] = fmaf(q, x[9]*x[12], g[5]);
    g[9] = fmaf(q, x[5]*x[12], g[9]);
    g[12] = fmaf(q, x[5]*x[9], g[12]);
  }
  { const float q = w * __ldg(cf + 70 * C);
    g[5] = fmaf(q, x[9]*x[14], g[5]);
    g[9] = fmaf(q, x[5]*x[14], g[9]);
    g[14] = fmaf(q, x[5]*x[9], g[14]);
  }
  { const float q = w * __ldg(cf + 71 * C);
    g[5] = fmaf(q, x[10]*x[13], g[5]);
    g[10] = fmaf(q, x[5]*x[13], g[10]);
    g[13] = fmaf(q, x[5]*x[10], g[13]);
  }
  { const float q = w * __ldg(cf + 72 * C);
    g[5] = fmaf(q, x[10]*x[15], g[5]);
    g[10] = fmaf(q, x[5]*x[15], g[10]);
    g[15] = fmaf(q, x[5]*x[10], g[15]);
  }
  { const float q = w * __ldg(cf + 73 * C);
    g[5] = fmaf(q, x[11]*x[12], g[5]);
    g[11] = fmaf(q, x[5]*x[12], g[11]);
    g[12] = fmaf(q, x[5]*x[11], g[12]);
  }
  { const float q = w * __ldg(cf + 74 * C);
    g[5] = fmaf(q, x[11]*x[14], g[5]);
    g[11] = fmaf(q, x[5]*x[14], g[11]);
    g[14] = fmaf(q, x[5]*x[11], g[14]);
  }
  { const float q = w * __ldg(cf + 75 * C);
    g[6] = fmaf(q, x[6]*x[8], g[6]);
    g[6] = fmaf(q, x[6]*x[8], g[6]);
    g[8] = fmaf(q, x[6]*x[6], g[8]);
  }
  { const float q = w * __ldg(cf + 76 * C);
    g[6] = fmaf(q, x[9]*x[11], g[6]);
    g[9] = fmaf(q, x[6]*x[11], g[9]);
    g[11] = fmaf(q, x[6]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 77 * C);
    g[6] = fmaf(q, x[11]*x[11], g[6]);
    g[11] = fmaf(q, x[6]*x[11], g[11]);
    g[11] = fmaf(q, x[6]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 78 * C);
    g[6] = fmaf(q, x[12]*x[14], g[6]);
    g[12] = fmaf(q, x[6]*x[14], g[12]);
    g[14] = fmaf(q, x[6]*x[12], g[14]);
  }
  { const float q = w * __ldg(cf + 79 * C);
    g[6] = fmaf(q, x[13]*x[13], g[6]);
    g[13] = fmaf(q, x[6]*x[13], g[13]);
    g[13] = fmaf(q, x[6]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 80 * C);
    g[6] = fmaf(q, x[13]*x[15], g[6]);
    g[13] = fmaf(q, x[6]*x[15], g[13]);
    g[15] = fmaf(q, x[6]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 81 * C);
    g[7] = fmaf(q, x[7]*x[8], g[7]);
    g[7] = fmaf(q, x[7]*x[8], g[7]);
    g[8] = fmaf(q, x[7]*x[7], g[8]);
  }
  { const float q = w * __ldg(cf + 82 * C);
    g[7] = fmaf(q, x[9]*x[10], g[7]);
    g[9] = fmaf(q, x[7]*x[10], g[9]);
    g[10] = fmaf(q, x[7]*x[9], g[10]);
  }
  { const float q = w * __ldg(cf + 83 * C);
    g[7] = fmaf(q, x[10]*x[11], g[7]);
    g[10] = fmaf(q, x[7]*x[11], g[10]);
    g[11] = fmaf(q, x[7]*x[10], g[11]);
  }
  { const float q = w * __ldg(cf + 84 * C);
    g[7] = fmaf(q, x[12]*x[13], g[7]);
    g[12] = fmaf(q, x[7]*x[13], g[12]);
    g[13] = fmaf(q, x[7]*x[12], g[13]);
  }
  { const float q = w * __ldg(cf + 85 * C);
    g[7] = fmaf(q, x[12]*x[15], g[7]);
    g[12] = fmaf(q, x[7]*x[15], g[12]);
    g[15] = fmaf(q, x[7]*x[12], g[15]);
  }
  { const float q = w * __ldg(cf + 86 * C);
    g[7] = fmaf(q, x[13]*x[14], g[7]);
    g[13] = fmaf(q, x[7]*x[14], g[13]);
    g[14] = fmaf(q, x[7]*x[13], g[14]);
  }
  { const float q = w * __ldg(cf + 87 * C);
    g[7] = fmaf(q, x[14]*x[15], g[7]);
    g[14] = fmaf(q, x[7]*x[15], g[14]);
    g[15] = fmaf(q, x[7]*x[14], g[15]);
  }
  { const float q = w * __ldg(cf + 88 * C);
    g[8] = fmaf(q, x[8]*x[8], g[8]);
    g[8] = fmaf(q, x[8]*x[8], g[8]);
    g[8] = fmaf(q, x[8]*x[8], g[8]);
  }
  { const float q = w * __ldg(cf + 89 * C);
    g[8] = fmaf(q, x[9]*x[9], g[8]);
    g[9] = fmaf(q, x[8]*x[9], g[9]);
    g[9] = fmaf(q, x[8]*x[9], g[9]);
  }
  { const float q = w * __ldg(cf + 90 * C);
    g[8] = fmaf(q, x[9]*x[11], g[8]);
    g[9] = fmaf(q, x[8]*x[11], g[9]);
    g[11] = fmaf(q, x[8]*x[9], g[11]);
  }
  { const float q = w * __ldg(cf + 91 * C);
    g[8] = fmaf(q, x[10]*x[10], g[8]);
    g[10] = fmaf(q, x[8]*x[10], g[10]);
    g[10] = fmaf(q, x[8]*x[10], g[10]);
  }
  { const float q = w * __ldg(cf + 92 * C);
    g[8] = fmaf(q, x[11]*x[11], g[8]);
    g[11] = fmaf(q, x[8]*x[11], g[11]);
    g[11] = fmaf(q, x[8]*x[11], g[11]);
  }
  { const float q = w * __ldg(cf + 93 * C);
    g[8] = fmaf(q, x[12]*x[12], g[8]);
    g[12] = fmaf(q, x[8]*x[12], g[12]);
    g[12] = fmaf(q, x[8]*x[12], g[12]);
  }
  { const float q = w * __ldg(cf + 94 * C);
    g[8] = fmaf(q, x[13]*x[13], g[8]);
    g[13] = fmaf(q, x[8]*x[13], g[13]);
    g[13] = fmaf(q, x[8]*x[13], g[13]);
  }
  { const float q = w * __ldg(cf + 95 * C);
    g[8] = fmaf(q, x[13]*x[15], g[8]);
    g[13] = fmaf(q, x[8]*x[15], g[13]);
    g[15] = fmaf(q, x[8]*x[13], g[15]);
  }
  { const float q = w * __ldg(cf + 96 * C);
    g[8] = fmaf(q, x[14]*x[14], g[8]);
    g[14] = fmaf(q, x[8]*x[14], g[14]);
    g[14] = fmaf(q, x[8]*x[14], g[14]);
  }
  { const float q = w * __ldg(cf + 97 * C);
    g[8] = fmaf(q, x[15]*x[15], g[8]);
    g[15] = fmaf(q, x[8]*x[15], g[15]);
    g[15] = fmaf(q, x[8]*x[15], g[15]);
  }
}

// the layer-1 contraction is the LM = 0 set
__device__ __forceinline__ float value_grad_M1(const float* x, const float* __restrict__ cf, int C, float* g) {
  float f0 = 0.0f, f1 = 0.0f, f2 = 0.0f, f3 = 0.0f;
  { const float q = __ldg(cf + 0 * C);
    f0 = fmaf(q, x[0], f0);
    g[0] += q;
  }
  { const float q = __ldg(cf + 1 * C);
    f1 = fmaf(q, x[0]*x[0], f1);
    g[0] = fmaf(q, x[0], g[0]);
    g[0] = fmaf(q, x[0], g[0]);
  }
  { const float q = __ldg(cf + 2 * C);
    f2 = fmaf(q, x[1]*x[1], f2);
    g[1] = fmaf(q, x[1], g[1]);
    g[1] = fmaf(q, x[1], g[1]);
  }
  { const float q = __ldg(cf + 3 * C);
    f3 = fmaf(q, x[2]*x[2], f3);
    g[2] = fmaf(q, x[2], g[2]);
    g[2] = fmaf(q, x[2], g[2]);
  }
  { const float q = __ldg(cf + 4 * C);
    f0 = fmaf(q, x[3]*x[3], f0);
    g[3] = fmaf(q, x[3], g[3]);
    g[3] = fmaf(q, x[3], g[3]);
  }
  { const float q = __ldg(cf + 5 * C);
    f1 = fmaf(q, x[4]*x[4], f1);
    g[4] = fmaf(q, x[4], g[4]);
    g[4] = fmaf(q, x[4], g[4]);
  }
  { const float q = __ldg(cf + 6 * C);
    f2 = fmaf(q, x[5]*x[5], f2);
    g[5] = fmaf(q, x[5], g[5]);
    g[5] = fmaf(q, x[5], g[5]);
  }
  { const float q = __ldg(cf + 7 * C);
    f3 = fmaf(q, x[6]*x[6], f3);
    g[6] = fmaf(q, x[6], g[6]);
    g[6] = fmaf(q, x[6], g[6]);
  }
  { const float q = __ldg(cf + 8 * C);
    f0 = fmaf(q, x[7]*x[7], f0);
    g[7] = fmaf(q, x[7], g[7]);
    g[7] = fmaf(q, x[7], g[7]);
  }
  { const float q = __ldg(cf + 9 * C);
    f1 = fmaf(q, x[8]*x[8], f1);
    g[8] = fmaf(q, x[8], g[8]);
    g[8] = fmaf(q, x[8], g[8]);
  }
  { const float q = __ldg(cf + 10 * C);
    f2 = fmaf(q, x[9]*x[9], f2);
    g[9] = fmaf(q, x[9], g[9]);
    g[9] = fmaf(q, x[9], g[9]);
  }
  { const float q = __ldg(cf + 11 * C);
    f3 = fmaf(q, x[10]*x[10], f3);
    g[10] = fmaf(q, x[10], g[10]);
    g[10] = fmaf(q, x[10], g[10]);
  }
  { const float q = __ldg(cf + 12 * C);
    f0 = fmaf(q, x[11]*x[11], f0);
    g[11] = fmaf(q, x[11], g[11]);
    g[11] = fmaf(q, x[11], g[11]);
  }
  { const float q = __ldg(cf + 13 * C);
    f1 = fmaf(q, x[12]*x[12], f1);
    g[12] = fmaf(q, x[12], g[12]);
    g[12] = fmaf(q, x[12], g[12]);
  }
  { const float q = __ldg(cf + 14 * C);
    f2 = fmaf(q, x[13]*x[13], f2);
    g[13] = fmaf(q, x[13], g[13]);
    g[13] = fmaf(q, x[13], g[13]);
  }
  { const float q = __ldg(cf + 15 * C);
    f3 = fmaf(q, x[14]*x[14], f3);
    g[14] = fmaf(q, x[14], g[14]);
    g[14] = fmaf(q, x[14], g[14]);
  }
  { const float q = __ldg(cf + 16 * C);
    f0 = fmaf(q, x[15]*x[15], f0);
    g[15] = fmaf(q, x[15], g[15]);
    g[15] = fmaf(q, x[15], g[15]);
  }
  { const float q = __ldg(cf + 17 * C);
    f1 = fmaf(q, x[0]*x[0]*x[0], f1);
    g[0] = fmaf(q, x[0]*x[0], g[0]);
    g[0] = fmaf(q, x[0]*x[0], g[0]);
    g[0] = fmaf(q, x[0]*x[0], g[0]);
  }
  { const float q = __ldg(cf + 18 * C);
    f2 = fmaf(q, x[0]*x[1]*x[1], f2);
    g[0] = fmaf(q, x[1]*x[1], g[0]);
    g[1] = fmaf(q, x[0]*x[1], g[1]);
    g[1] = fmaf(q, x[0]*x[1], g[1]);
  }
  { const float q = __ldg(cf + 19 * C);
    f3 = fmaf(q, x[0]*x[2]*x[2], f3);
    g[0] = fmaf(q, x[2]*x[2], g[0]);
    g[2] = fmaf(q, x[0]*x[2], g[2]);
    g[2] = fmaf(q, x[0]*x[2], g[2]);
  }
  { const float q = __ldg(cf + 20 * C);
    f0 = fmaf(q, x[0]*x[3]*x[3], f0);
    g[0] = fmaf(q, x[3]*x[3], g[0]);
    g[3] = fmaf(q, x[0]*x[3], g[3]);
    g[3] = fmaf(q, x[0]*x[3], g[3]);
  }
  { const float q = __ldg(cf + 21 * C);
    f1 = fmaf(q, x[0]*x[4]*x[4], f1);
    g[0] = fmaf(q, x[4]*x[4], g[0]);
    g[4] = fmaf(q, x[0]*x[4], g[4]);
    g[4] = fmaf(q, x[0]*x[4], g[4]);
  }
  { const float q = __ldg(cf + 22 * C);
    f2 = fmaf(q, x[0]*x[5]*x[5], f2);
    g[0] = fmaf(q, x[5]*x[5], g[0]);
    g[5] = fmaf(q, x[0]*x[5], g[5]);
    g[5] = fmaf(q, x[0]*x[5], g[5]);
  }
  { const float q = __ldg(cf + 23 * C);
    f3 = fmaf(q, x[0]*x[6]*x[6], f3);
    g[0] = fmaf(q, x[6]*x[6], g[0]);
    g[6] = fmaf(q, x[0]*x[6], g[6]);
    g[6] = fmaf(q, x[0]*x[6], g[6]);
  }
  { const float q = __ldg(cf + 24 * C);
    f0 = fmaf(q, x[0]*x[7]*x[7], f0);
    g[0] = fmaf(q, x[7]*x[7], g[0]);
    g[7] = fmaf(q, x[0]*x[7], g[7]);
    g[7] = fmaf(q, x[0]*x[7], g[7]);
  }
  { const float q = __ldg(cf + 25 * C);
    f1 = fmaf(q, x[0]*x[8]*x[8], f1);
    g[0] = fmaf(q, x[8]*x[8], g[0]);
    g[8] = fmaf(q, x[0]*x[8], g[8]);
    g[8] = fmaf(q, x[0]*x[8], g[8]);
  }
  { const float q = __ldg(cf + 26 * C);
    f2 = fmaf(q, x[0]*x[9]*x[9], f2);
    g[0] = fmaf(q, x[9]*x[9], g[0]);
    g[9] = fmaf(q, x[0]*x[9], g[9]);
    g[9] = fmaf(q, x[0]*x[9], g[9]);
  }
  { const float q = __ldg(cf + 27 * C);
    f3 = fmaf(q, x[0]*x[10]*x[10], f3);
    g[0] = fmaf(q, x[10]*x[10], g[0]);
    g[10] = fmaf(q, x[0]*x[10], g[10]);
    g[10] = fmaf(q, x[0]*x[10], g[10]);
  }
  { const float q = __ldg(cf + 28 * C);
    f0 = fmaf(q, x[0]*x[11]*x[11], f0);
    g[0] = fmaf(q, x[11]*x[11], g[0]);
    g[11] = fmaf(q, x[0]*x[11], g[11]);
    g[11] = fmaf(q, x[0]*x[11], g[11]);
  }
  { const float q = __ldg(cf + 29 * C);
    f1 = fmaf(q, x[0]*x[12]*x[12], f1);
    g[0] = fmaf(q, x[12]*x[12], g[0]);
    g[12] = fmaf(q, x[0]*x[12], g[12]);
    g[12] = fmaf(q, x[0]*x[12], g[12]);
  }
  { const float q = __ldg(cf + 30 * C);
    f2 = fmaf(q, x[0]*x[13]*x[13], f2);
    g[0] = fmaf(q, x[13]*x[13], g[0]);
    g[13] = fmaf(q, x[0]*x[13], g[13]);
    g[13] = fmaf(q, x[0]*x[13], g[13]);
  }
  { const float q = __ldg(cf + 31 * C);
    f3 = fmaf(q, x[0]*x[14]*x[14], f3);
    g[0] = fmaf(q, x[14]*x[14], g[0]);
    g[14] = fmaf(q, x[0]*x[14], g[14]);
    g[14] = fmaf(q, x[0]*x[14], g[14]);
  }
  { const float q = __ldg(cf + 32 * C);
    f0 = fmaf(q, x[0]*x[15]*x[15], f0);
    g[0] = fmaf(q, x[15]*x[15], g[0]);
    g[15] = fmaf(q, x[0]*x[15], g[15]);
    g[15] = fmaf(q, x[0]*x[15], g[15]);
  }
  { const float q = __ldg(cf + 33 * C);
    f1 = fmaf(q, x[1]*x[1]*x[6], f1);
    g[1] = fmaf(q, x[1]*x[6], g[1]);
    g[1] = fmaf(q, x[1]*x[6], g[1]);
    g[6] = fmaf(q, x[1]*x[1], g[6]);
  }
  { const float q = __ldg(cf + 34 * C);
    f2 = fmaf(q, x[1]*x[1]*x[8], f2);
    g[1] = fmaf(q, x[1]*x[8], g[1]);
    g[1] = fmaf(q, x[1]*x[8], g[1]);
    g[8] = fmaf(q, x[1]*x[1], g[8]);
  }
  { const float q = __ldg(cf + 35 * C);
    f3 = fmaf(q, x[1]*x[2]*x[5], f3);
    g[1] = fmaf(q, x[2]*x[5], g[1]);
    g[2] = fmaf(q, x[1]*x[5], g[2]);
    g[5] = fmaf(q, x[1]*x[2], g[5]);
  }
  { const float q = __ldg(cf + 36 * C);
    f0 = fmaf(q, x[1]*x[3]*x[4], f0);
    g[1] = fmaf(q, x[3]*x[4], g[1]);
    g[3] = fmaf(q, x[1]*x[4], g[3]);
    g[4] = fmaf(q, x[1]*x[3], g[4]);
  }
  { const float q = __ldg(cf + 37 * C);
    f1 = fmaf(q, x[1]*x[4]*x[13], f1);
    g[1] = fmaf(q, x[4]*x[13], g[1]);
    g[4] = fmaf(q, x[1]*x[13], g[4]);
    g[13] = fmaf(q, x[1]*x[4], g[13]);
  }
  { const float q = __ldg(cf + 38 * C);
    f2 = fmaf(q, x[1]*x[4]*x[15], f2);
    g[1] = fmaf(q, x[4]*x[15], g[1]);
    g[4] = fmaf(q, x[1]*x[15], g[4]);
    g[15] = fmaf(q, x[1]*x[4], g[15]);
  }
  { const float q = __ldg(cf + 39 * C);
    f3 = fmaf(q, x[1]*x[5]*x[12], f3);
    g[1] = fmaf(q, x[5]*x[12], g[1]);
    g[5] = fmaf(q, x[1]*x[12], g[5]);
    g[12] = fmaf(q, x[1]*x[5], g[12]);
  }
  { const float q = __ldg(cf + 40 * C);
    f0 = fmaf(q, x[1]*x[5]*x[14], f0);
    g[1] = fmaf(q, x[5]*x[14], g[1]);
    g[5] = fmaf(q, x[1]*x[14], g[5]);
    g[14] = fmaf(q, x[1]*x[5], g[14]);
  }
  { const float q = __ldg(cf + 41 * C);
    f1 = fmaf(q, x[1]*x[6]*x[11], f1);
    g[1] = fmaf(q, x[6]*x[11], g[1]);
    g[6] = fmaf(q, x[1]*x[11], g[6]);
    g[11] = fmaf(q, x[1]*x[6], g[11]);
  }
  { const float q = __ldg(cf + 42 * C);
    f2 = fmaf(q, x[1]*x[7]*x[10], f2);
    g[1] = fmaf(q, x[7]*x[10], g[1]);
    g[7] = fmaf(q, x[1]*x[10], g[7]);
    g[10] = fmaf(q, x[1]*x[7], g[10]);
  }
  { const float q = __ldg(cf + 43 * C);
    f3 = fmaf(q, x[1]*x[8]*x[9], f3);
    g[1] = fmaf(q, x[8]*x[9], g[1]);
    g[8] = fmaf(q, x[1]*x[9], g[8]);
    g[9] = fmaf(q, x[1]*x[8], g[9]);
  }
  { const float q = __ldg(cf + 44 * C);
    f0 = fmaf(q, x[1]*x[8]*x[11], f0);
    g[1] = fmaf(q, x[8]*x[11], g[1]);
    g[8] = fmaf(q, x[1]*x[11], g[8]);
    g[11] = fmaf(q, x[1]*x[8], g[11]);
  }
  { const float q = __ldg(cf + 45 * C);
    f1 = fmaf(q, x[2]*x[2]*x[6], f1);
    g[2] = fmaf(q, x[2]*x[6], g[2]);
    g[2] = fmaf(q, x[2]*x[6], g[2]);
    g[6] = fmaf(q, x[2]*x[2], g[6]);
  }
  { const float q = __ldg(cf + 46 * C);
    f2 = fmaf(q, x[2]*x[3]*x[7], f2);
    g[2] = fmaf(q, x[3]*x[7], g[2]);
    g[3] = fmaf(q, x[2]*x[7], g[3]);
    g[7] = fmaf(q, x[2]*x[3], g[7]);
  }
  { const float q = __ldg(cf + 47 * C);
    f3 = fmaf(q, x[2]*x[4]*x[10], f3);
    g[2] = fmaf(q, x[4]*x[10], g[2]);
    g[4] = fmaf(q, x[2]*x[10], g[4]);
    g[10] = fmaf(q, x[2]*x[4], g[10]);
  }
  { const float q = __ldg(cf + 48 * C);
    f0 = fmaf(q, x[2]*x[5]*x[11], f0);
    g[2] = fmaf(q, x[5]*x[11], g[2]);
    g[5] = fmaf(q, x[2]*x[11], g[5]);
    g[11] = fmaf(q, x[2]*x[5], g[11]);
  }
  { const float q = __ldg(cf + 49 * C);
    f1 = fmaf(q, x[2]*x[6]*x[12], f1);
    g[2] = fmaf(q, x[6]*x[12], g[2]);
    g[6] = fmaf(q, x[2]*x[12], g[6]);
    g[12] = fmaf(q, x[2]*x[6], g[12]);
  }
  { const float q = __ldg(cf + 50 * C);
    f2 = fmaf(q, x[2]*x[7]*x[13], f2);
    g[2] = fmaf(q, x[7]*x[13], g[2]);
    g[7] = fmaf(q, x[2]*x[13], g[7]);
    g[13] = fmaf(q, x[2]*x[7], g[13]);
  }
  { const float q = __ldg(cf + 51 * C);
    f3 = fmaf(q, x[2]*x[8]*x[14], f3);
    g[2] = fmaf(q, x[8]*x[14], g[2]);
    g[8] = fmaf(q, x[2]*x[14], g[8]);
    g[14] = fmaf(q, x[2]*x[8], g[14]);
  }
  { const float q = __ldg(cf + 52 * C);
    f0 = fmaf(q, x[3]*x[3]*x[6], f0);
    g[3] = fmaf(q, x[3]*x[6], g[3]);
    g[3] = fmaf(q, x[3]*x[6], g[3]);
    g[6] = fmaf(q, x[3]*x[3], g[6]);
  }
  { const float q = __ldg(cf + 53 * C);
    f1 = fmaf(q, x[3]*x[3]*x[8], f1);
    g[3] = fmaf(q, x[3]*x[8], g[3]);
    g[3] = fmaf(q, x[3]*x[8], g[3]);
    g[8] = fmaf(q, x[3]*x[3], g[8]);
  }
  { const float q = __ldg(cf + 54 * C);
    f2 = fmaf(q, x[3]*x[4]*x[9], f2);
    g[3] = fmaf(q, x[4]*x[9], g[3]);
    g[4] = fmaf(q, x[3]*x[9], g[4]);
    g[9] = fmaf(q, x[3]*x[4], g[9]);
  }
  { const float q = __ldg(cf + 55 * C);
    f3 = fmaf(q, x[3]*x[4]*x[11], f3);
    g[3] = fmaf(q, x[4]*x[11], g[3]);
    g[4] = fmaf(q, x[3]*x[11], g[4]);
    g[11] = fmaf(q, x[3]*x[4], g[11]);
  }
  { const float q = __ldg(cf + 56 * C);
    f0 = fmaf(q, x[3]*x[5]*x[10], f0);
    g[3] = fmaf(q, x[5]*x[10], g[3]);
    g[5] = fmaf(q, x[3]*x[10], g[5]);
    g[10] = fmaf(q, x[3]*x[5], g[10]);
  }
  { const float q = __ldg(cf + 57 * C);
    f1 = fmaf(q, x[3]*x[6]*x[13], f1);
    g[3] = fmaf(q, x[6]*x[13], g[3]);
    g[6] = fmaf(q, x[3]*x[13], g[6]);
    g[13] = fmaf(q, x[3]*x[6], g[13]);
  }
  { const float q = __ldg(cf + 58 * C);
    f2 = fmaf(q, x[3]*x[7]*x[12], f2);
    g[3] = fmaf(q, x[7]*x[12], g[3]);
    g[7] = fmaf(q, x[3]*x[12], g[7]);
    g[12] = fmaf(q, x[3]*x[7], g[12]);
  }
  { const float q = __ldg(cf + 59 * C);
    f3 = fmaf(q, x[3]*x[7]*x[14], f3);
    g[3] = fmaf(q, x[7]*x[14], g[3]);
    g[7] = fmaf(q, x[3]*x[14], g[7]);
    g[14] = fmaf(q, x[3]*x[7], g[14]);
  }
  { const float q = __ldg(cf + 60 * C);
    f0 = fmaf(q, x[3]*x[8]*x[13], f0);
    g[3] = fmaf(q, x[8]*x[13], g[3]);
    g[8] = fmaf(q, x[3]*x[13], g[8]);
    g[13] = fmaf(q, x[3]*x[8], g[13]);
  }
  { const float q = __ldg(cf + 61 * C);
    f1 = fmaf(q, x[3]*x[8]*x[15], f1);
    g[3] = fmaf(q, x[8]*x[15], g[3]);
    g[8] = fmaf(q, x[3]*x[15], g[8]);
    g[15] = fmaf(q, x[3]*x[8], g[15]);
  }
  { const float q = __ldg(cf + 62 * C);
    f2 = fmaf(q, x[4]*x[4]*x[6], f2);
    g[4] = fmaf(q, x[4]*x[6], g[4]);
    g[4] = fmaf(q, x[4]*x[6], g[4]);
    g[6] = fmaf(q, x[4]*x[4], g[6]);
  }
  { const float q = __ldg(cf + 63 * C);
    f3 = fmaf(q, x[4]*x[5]*x[7], f3);
    g[4] = fmaf(q, x[5]*x[7], g[4]);
    g[5] = fmaf(q, x[4]*x[7], g[5]);
    g[7] = fmaf(q, x[4]*x[5], g[7]);
  }
  { const float q = __ldg(cf + 64 * C);
    f0 = fmaf(q, x[4]*x[9]*x[13], f0);
    g[4] = fmaf(q, x[9]*x[13], g[4]);
    g[9] = fmaf(q, x[4]*x[13], g[9]);
    g[13] = fmaf(q, x[4]*x[9], g[13]);
  }
  { const float q = __ldg(cf + 65 * C);
    f1 = fmaf(q, x[4]*x[10]*x[12], f1);
    g[4] = fmaf(q, x[10]*x[12], g[4]);
    g[10] = fmaf(q, x[4]*x[12], g[10]);
    g[12] = fmaf(q, x[4]*x[10], g[12]);
  }
  { const float q = __ldg(cf + 66 * C);
    f2 = fmaf(q, x[4]*x[11]*x[13], f2);
    g[4] = fmaf(q, x[11]*x[13], g[4]);
    g[11] = fmaf(q, x[4]*x[13], g[11]);
    g[13] = fmaf(q, x[4]*x[11], g[13]);
  }
  { const float q = __ldg(cf + 67 * C);
    f3 = fmaf(q, x[4]*x[11]*x[15], f3);
    g[4] = fmaf(q, x[11]*x[15], g[4]);
    g[11] = fmaf(q, x[4]*x[15], g[11]);
    g[15] = fmaf(q, x[4]*x[11], g[15]);
  }
  { const float q = __ldg(cf + 68 * C);
    f0 = fmaf(q, x[5]*x[5]*x[6], f0);
    g[5] = fmaf(q, x[5]*x[6], g[5]);
    g[5] = fmaf(q, x[5]*x[6], g[5]);
    g[6] = fmaf(q, x[5]*x[5], g[6]);
  }
  { const float q = __ldg(cf + 69 * C);
    f1 = fmaf(q, x[5]*x[5]*x[8], f1);
    g[5] = fmaf(q, x[5]*x[8], g[5]);
    g[5] = fmaf(q, x[5]*x[8], g[5]);
    g[8] = fmaf(q, x[5]*x[5], g[8]);
  }
  { const float q = __ldg(cf + 70 * C);
    f2 = fmaf(q, x[5]*x[9]*x[14], f2);
    g[5] = fmaf(q, x[9]*x[14], g[5]);
    g[9] = fmaf(q, x[5]*x[14], g[9]);
    g[14] = fmaf(q, x[5]*x[9], g[14]);
  }
  { const float q = __ldg(cf + 71 * C);
    f3 = fmaf(q, x[5]*x[10]*x[13], f3);
    g[5] = fmaf(q, x[10]*x[13], g[5]);
    g[10] = fmaf(q, x[5]*x[13], g[10]);
    g[13] = fmaf(q, x[5]*x[10], g[13]);
  }
  { const float q = __ldg(cf + 72 * C);
    f0 = fmaf(q, x[5]*x[10]*x[15], f0);
    g[5] = fmaf(q, x[10]*x[15], g[5]);
    g[10] = fmaf(q, x[5]*x[15], g[10]);
    g[15] = fmaf(q, x[5]*x[10], g[15]);
  }
  { const float q = __ldg(cf + 73 * C);
    f1 = fmaf(q, x[5]*x[11]*x[12], f1);
    g[5] = fmaf(q, x[11]*x[12], g[5]);
    g[11] = fmaf(q, x[5]*x[12], g[11]);
    g[12] = fmaf(q, x[5]*x[11], g[12]);
  }
  { const float q = __ldg(cf + 74 * C);
    f2 = fmaf(q, x[5]*x[11]*x[14], f2);
    g[5] = fmaf(q, x[11]*x[14], g[5]);
    g[11] = fmaf(q, x[5]*x[14], g[11]);
    g[14] = fmaf(q, x[5]*x[11], g[14]);
  }
  { const float q = __ldg(cf + 75 * C);
    f3 = fmaf(q, x[6]*x[6]*x[6], f3);
    g[6] = fmaf(q, x[6]*x[6], g[6]);
    g[6] = fmaf(q, x[6]*x[6], g[6]);
    g[6] = fmaf(q, x[6]*x[6], g[6]);
  }
  { const float q = __ldg(cf + 76 * C);
    f0 = fmaf(q, x[6]*x[7]*x[7], f0);
    g[6] = fmaf(q, x[7]*x[7], g[6]);
    g[7] = fmaf(q, x[6]*x[7], g[7]);
    g[7] = fmaf(q, x[6]*x[7], g[7]);
  }
  { const float q = __ldg(cf + 77 * C);
    f1 = fmaf(q, x[6]*x[8]*x[8], f1);
    g[6] = fmaf(q, x[8]*x[8], g[6]);
    g[8] = fmaf(q, x[6]*x[8], g[8]);
    g[8] = fmaf(q, x[6]*x[8], g[8]);
  }
  { const float q = __ldg(cf + 78 * C);
    f2 = fmaf(q, x[6]*x[9]*x[9], f2);
    g[6] = fmaf(q, x[9]*x[9], g[6]);
    g[9] = fmaf(q, x[6]*x[9], g[9]);
    g[9] = fmaf(q, x[6]*x[9], g[9]);
  }
  { const float q = __ldg(cf + 79 * C);
    f3 = fmaf(q, x[6]*x[11]*x[11], f3);
    g[6] = fmaf(q, x[11]*x[11], g[6]);
    g[11] = fmaf(q, x[6]*x[11], g[11]);
    g[11] = fmaf(q, x[6]*x[11], g[11]);
  }
  { const float q = __ldg(cf + 80 * C);
    f0 = fmaf(q, x[6]*x[12]*x[12], f0);
    g[6] = fmaf(q, x[12]*x[12], g[6]);
    g[12] = fmaf(q, x[6]*x[12], g[12]);
    g[12] = fmaf(q, x[6]*x[12], g[12]);
  }
  { const float q = __ldg(cf + 81 * C);
    f1 = fmaf(q, x[6]*x[13]*x[13], f1);
    g[6] = fmaf(q, x[13]*x[13], g[6]);
    g[13] = fmaf(q, x[6]*x[13], g[13]);
    g[13] = fmaf(q, x[6]*x[13], g[13]);
  }
  { const float q = __ldg(cf + 82 * C);
    f2 = fmaf(q, x[6]*x[15]*x[15], f2);
    g[6] = fmaf(q, x[15]*x[15], g[6]);
    g[15] = fmaf(q, x[6]*x[15], g[15]);
    g[15] = fmaf(q, x[6]*x[15], g[15]);
  }
  { const float q = __ldg(cf + 83 * C);
    f3 = fmaf(q, x[7]*x[7]*x[8], f3);
    g[7] = fmaf(q, x[7]*x[8], g[7]);
    g[7] = fmaf(q, x[7]*x[8], g[7]);
    g[8] = fmaf(q, x[7]*x[7], g[8]);
  }
  { const float q = __ldg(cf + 84 * C);
    f0 = fmaf(q, x[7]*x[9]*x[10], f0);
    g[7] = fmaf(q, x[9]*x[10], g[7]);
    g[9] = fmaf(q, x[7]*x[10], g[9]);
    g[10] = fmaf(q, x[7]*x[9], g[10]);
  }
  { const float q = __ldg(cf + 85 * C);
    f1 = fmaf(q, x[7]*x[10]*x[11], f1);
    g[7] = fmaf(q, x[10]*x[11], g[7]);
    g[10] = fmaf(q, x[7]*x[11], g[10]);
    g[11] = fmaf(q, x[7]*x[10], g[11]);
  }
  { const float q = __ldg(cf + 86 * C);
    f2 = fmaf(q, x[7]*x[12]*x[13], f2);
    g[7] = fmaf(q, x[12]*x[13], g[7]);
    g[12] = fmaf(q, x[7]*x[13], g[12]);
    g[13] = fmaf(q, x[7]*x[12], g[13]);
  }
  { const float q = __ldg(cf + 87 * C);
    f3 = fmaf(q, x[7]*x[13]*x[14], f3);
    g[7] = fmaf(q, x[13]*x[14], g[7]);
    g[13] = fmaf(q, x[7]*x[14], g[13]);
    g[14] = fmaf(q, x[7]*x[13], g[14]);
  }
  { const float q = __ldg(cf + 88 * C);
    f0 = fmaf(q, x[7]*x[14]*x[15], f0);
    g[7] = fmaf(q, x[14]*x[15], g[7]);
    g[14] = fmaf(q, x[7]*x[15], g[14]);
    g[15] = fmaf(q, x[7]*x[14], g[15]);
  }
  { const float q = __ldg(cf + 89 * C);
    f1 = fmaf(q, x[8]*x[9]*x[11], f1);
    g[8] = fmaf(q, x[9]*x[11], g[8]);
    g[9] = fmaf(q, x[8]*x[11], g[9]);
    g[11] = fmaf(q, x[8]*x[9], g[11]);
  }
  { const float q = __ldg(cf + 90 * C);
    f2 = fmaf(q, x[8]*x[11]*x[11], f2);
    g[8] = fmaf(q, x[11]*x[11], g[8]);
    g[11] = fmaf(q, x[8]*x[11], g[11]);
    g[11] = fmaf(q, x[8]*x[11], g[11]);
  }
  { const float q = __ldg(cf + 91 * C);
    f3 = fmaf(q, x[8]*x[12]*x[14], f3);
    g[8] = fmaf(q, x[12]*x[14], g[8]);
    g[12] = fmaf(q, x[8]*x[14], g[12]);
    g[14] = fmaf(q, x[8]*x[12], g[14]);
  }
  { const float q = __ldg(cf + 92 * C);
    f0 = fmaf(q, x[8]*x[13]*x[13], f0);
    g[8] = fmaf(q, x[13]*x[13], g[8]);
    g[13] = fmaf(q, x[8]*x[13], g[13]);
    g[13] = fmaf(q, x[8]*x[13], g[13]);
  }
  { const float q = __ldg(cf + 93 * C);
    f1 = fmaf(q, x[8]*x[13]*x[15], f1);
    g[8] = fmaf(q, x[13]*x[15], g[8]);
    g[13] = fmaf(q, x[8]*x[15], g[13]);
    g[15] = fmaf(q, x[8]*x[13], g[15]);
  }
  return (f0 + f1) + (f2 + f3);
}

}  // namespace poly
}  // namespace smx
