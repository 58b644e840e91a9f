// fv3g_ff.cuh -- float-float arithmetic shared by the FP32 remap and the
// FP32 global mass sums.
#pragma once

#include <cuda_runtime.h>

namespace fv3g {

// Float-float arithmetic (an unevaluated sum of two floats, ~48-bit
// significand): the error-free transformations TwoSum (Knuth) and TwoProd
// (with fma), then one renormalisation.
struct FF {
  float hi, lo;
};
__device__ __forceinline__ FF ff_add(FF a, FF b) {
  const float s = a.hi + b.hi;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b.hi - bb);
  e += a.lo + b.lo;
  const float h = s + e;
  return FF{h, e - (h - s)};
}
__device__ __forceinline__ FF ff_neg(FF a) { return FF{-a.hi, -a.lo}; }
__device__ __forceinline__ FF ff_prod(float a, float b) {
  const float p = a * b;
  return FF{p, fmaf(a, b, -p)};
}

// the exact product a * b * c of three floats as float-float (to ~2^-48):
// TwoProd of a*b, then of its leading part with c, the low part's product
// folded in with one fma
__device__ __forceinline__ FF ff_prod3(float a, float b, float c) {
  const FF ab = ff_prod(a, b);
  const float p = ab.hi * c;
  return FF{p, fmaf(ab.lo, c, fmaf(ab.hi, c, -p))};
}

}  // namespace fv3g
