// fv3g_dual.cuh -- forward-mode (value, tangent) scalar for the tangent-linear
// kernels.  Every comparison, min/max and sign test acts on the value, so a
// kernel instantiated on Dual<R> follows the trajectory's limiter branches and
// carries their derivative: the tangent-linear model with frozen branches.
#pragma once

#include <cuda_runtime.h>

namespace fv3g {

template <typename R>
struct Dual {
  R v, d;
  __host__ __device__ Dual() : v(0), d(0) {}
  __host__ __device__ Dual(R a) : v(a), d(0) {}  // constants and frozen fields
  __host__ __device__ Dual(R a, R b) : v(a), d(b) {}

  friend __host__ __device__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
  friend __host__ __device__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
  friend __host__ __device__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
  friend __host__ __device__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
  friend __host__ __device__ Dual operator/(Dual a, Dual b) {
    const R r = R(1) / b.v;
    return Dual(a.v * r, (a.d - a.v * r * b.d) * r);
  }
  __host__ __device__ Dual& operator+=(Dual b) { return *this = *this + b; }
  __host__ __device__ Dual& operator-=(Dual b) { return *this = *this - b; }
  __host__ __device__ Dual& operator*=(Dual b) { return *this = *this * b; }
  friend __host__ __device__ bool operator<(Dual a, Dual b) { return a.v < b.v; }
  friend __host__ __device__ bool operator>(Dual a, Dual b) { return a.v > b.v; }
  friend __host__ __device__ bool operator<=(Dual a, Dual b) { return a.v <= b.v; }
  friend __host__ __device__ bool operator>=(Dual a, Dual b) { return a.v >= b.v; }
  friend __host__ __device__ bool operator==(Dual a, Dual b) { return a.v == b.v; }
  friend __host__ __device__ bool operator!=(Dual a, Dual b) { return a.v != b.v; }
};

template <typename R>
__device__ __forceinline__ Dual<R> copysign_t(Dual<R> a, Dual<R> b) {
  return (signbit(a.v) == signbit(b.v)) ? a : -a;
}
template <typename R>
__device__ __forceinline__ Dual<R> tmax3(Dual<R> a, Dual<R> b, Dual<R> c) {
  const Dual<R> m = a > b ? a : b;
  return m > c ? m : c;
}
template <typename R>
__device__ __forceinline__ Dual<R> tmin3(Dual<R> a, Dual<R> b, Dual<R> c) {
  const Dual<R> m = a < b ? a : b;
  return m < c ? m : c;
}

// the value part of a scalar, as double
__host__ __device__ inline double value_of(double x) { return x; }
__host__ __device__ inline double value_of(float x) { return x; }
template <typename R>
__host__ __device__ inline double value_of(const Dual<R>& x) { return x.v; }

// precision of the arithmetic a type carries (float: single)
template <typename T> struct Single { static constexpr bool value = false; };
template <> struct Single<float> { static constexpr bool value = true; };

}  // namespace fv3g
