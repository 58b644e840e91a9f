// fv3g_pair.cuh -- two FP32 values advanced in lockstep (two tracers of one
// cell): add, subtract, multiply and fused multiply-add on the packed
// f32x2 forms of sm_100 and later, one instruction for both values; min,
// max, |.| and sign per value (no packed form exists for them).
#pragma once

#include <cuda_runtime.h>

namespace fv3g {

struct __align__(8) F2 {
  float x, y;
};

__device__ __forceinline__ unsigned long long f2_bits(F2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ F2 f2_from(unsigned long long r) {
  F2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ F2 bc(float s) { return F2{s, s}; }  // the same value twice

__device__ __forceinline__ F2 add2(F2 a, F2 b) {
  unsigned long long r;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(r);
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
  unsigned long long r;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(r);
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
  unsigned long long r;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(r);
}
// a * b + c, one rounding
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
  unsigned long long r;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(f2_bits(a)), "l"(f2_bits(b)), "l"(f2_bits(c)));
  return f2_from(r);
}
__device__ __forceinline__ F2 neg2(F2 a) { return F2{-a.x, -a.y}; }
__device__ __forceinline__ F2 abs2(F2 a) { return F2{fabsf(a.x), fabsf(a.y)}; }
__device__ __forceinline__ F2 min2(F2 a, F2 b) { return F2{fminf(a.x, b.x), fminf(a.y, b.y)}; }

// three-input min / max per value (one instruction each on sm_100 and later)
__device__ __forceinline__ float fmax3f(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float fmin3f(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ F2 max3_2(F2 a, F2 b, F2 c) { return F2{fmax3f(a.x, b.x, c.x), fmax3f(a.y, b.y, c.y)}; }
__device__ __forceinline__ F2 min3_2(F2 a, F2 b, F2 c) { return F2{fmin3f(a.x, b.x, c.x), fmin3f(a.y, b.y, c.y)}; }

// +1 or -1 with the sign bit of a (so m * sign2(a) is copysign(m, a) for m >= 0)
__device__ __forceinline__ float sign1(float a) {
  return __int_as_float((__float_as_int(a) & 0x80000000) | 0x3f800000);
}
__device__ __forceinline__ F2 sign2(F2 a) { return F2{sign1(a.x), sign1(a.y)}; }

}  // namespace fv3g
