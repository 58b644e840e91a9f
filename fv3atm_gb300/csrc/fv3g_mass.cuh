// fv3g_mass.cuh -- arguments of the compensated global mass sum and of the
// global mass fixer.
#pragma once

#include "fv3g_internal.cuh"

namespace fv3g {

constexpr int MASS_BLOCKS = 304;  // 2 x 152 SMs
// partials: 2 doubles per block and summed quantity; a mass sum of nq
// tracers with the fixer-row sums (below) fills 3 nq quantities
constexpr int MASS_PARTIALS_PER_TRACER = 6 * MASS_BLOCKS;
// the FP32 fixer moves values in 1/MASS_FIX_ROWS of the rows (a power of 2),
// in its second pass only values below 2^-MASS_CLASS_SHIFT of the tracer's
// largest binade
constexpr int MASS_FIX_ROWS = 16;
constexpr int MASS_CLASS_SHIFT = 10;

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
  double* partials;     // MASS_PARTIALS_PER_TRACER * nq doubles
  int* emax_out;        // optional (FP32): per tracer, atomicMax of the biased exponent of |q| (zeroed before)
  const int* cls_emax;  // optional (FP32): per tracer, the exponent that defines the small-value class
};

// mass of nq tracers into d_out[0..nq); with a.cls_emax also the mass of the
// fixer's rows into d_out[nq..2nq) and of their small-value class into
// d_out[2nq..3nq)
template <typename T>
int launch_mass(const MassArgs<T>& a, int nq, double* d_out, cudaStream_t s);

// Restore each tracer's global mass to mass0[iq] (see fv3g_mass.cu).  a
// addresses the fixed field (q is its writable pointer); iq_base: the state's
// index of its first tracer (seeds the dithering); mass1c: the field's
// masses from launch_mass with a.cls_emax, 3 nq doubles; dm: 2 nq doubles of
// scratch; emax: the class exponents.  3 launches for FP32 fields, 1 for
// FP64.
template <typename T>
int launch_mass_fix(const MassArgs<T>& a, T* q, int nq, int iq_base, const double* mass0, const double* mass1c,
                    double* dm, const int* emax, cudaStream_t s);

}  // namespace fv3g
