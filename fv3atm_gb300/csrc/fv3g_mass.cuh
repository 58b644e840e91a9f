// fv3g_mass.cuh -- arguments of the compensated global mass sum.
#pragma once

#include "fv3g_internal.cuh"

namespace fv3g {

constexpr int MASS_BLOCKS = 304;  // 2 x 152 SMs; partials hold 2*MASS_BLOCKS doubles per tracer

template <typename T>
struct MassArgs {
  const T* q;
  long long sQt, sQq, sQk;
  const T* dp;
  long long sFt, sFk;
  const T* area;
  long long sMt;
  PlaneGeom pg;
  int i1, j1, ni, nj;
  int npz, ntiles;
  double* partials;  // 2 * MASS_BLOCKS * nq doubles
};

template <typename T>
int launch_mass(const MassArgs<T>& a, int nq, double* d_out, cudaStream_t s);

}  // namespace fv3g
