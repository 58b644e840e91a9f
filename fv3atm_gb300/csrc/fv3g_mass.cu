// fv3g_mass.cu -- compensated FP64 global tracer mass, sum(q * delp * area)
// over the compute domain of every tile (the global-sum diagnostic that FV3
// computes with g_sum; MPI_Allreduce analogue at atmos_model.F90:496-502).
//
// Each thread accumulates a strided subset with Neumaier's compensated sum;
// blocks combine (sum, compensation) pairs in a fixed tree order into a
// partials buffer, and a single block reduces the partials per tracer, so
// the result is bitwise reproducible for a given problem size.
#include "fv3g_ff.cuh"
#include "fv3g_internal.cuh"
#include "fv3g_mass.cuh"

namespace fv3g {

__device__ __forceinline__ void neumaier(double& s, double& c, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x)) c += (s - t) + x;
  else c += (x - t) + s;
  s = t;
}

// Combine every thread's (sum, compensation) pair of a tracer in a fixed
// tree order into the tracer's partials slot of this block.
__device__ __forceinline__ void block_partial(double s, double c, double* partials, int iq, double* ss,
                                              double* sc) {
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      double s0 = ss[threadIdx.x], c0 = sc[threadIdx.x] + sc[threadIdx.x + o];
      neumaier(s0, c0, ss[threadIdx.x + o]);
      ss[threadIdx.x] = s0;
      sc[threadIdx.x] = c0;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    partials[2 * ((long long)iq * gridDim.x + blockIdx.x) + 0] = ss[0];
    partials[2 * ((long long)iq * gridDim.x + blockIdx.x) + 1] = sc[0];
  }
  __syncthreads();
}

// One warp per row (tile, level, j) in a grid-stride loop, lanes along i;
// each block sums MASS_CHUNK tracers (blockIdx.y picks the chunk), so delp
// and the area are read once per chunk of tracers.
// FP64 fields: every term q*dp*area goes through Neumaier's sum.  FP32 fields:
// dp*area is formed exactly as float-float, each term q*(dp*area) as
// float-float (to ~2^-48), a lane adds its terms in float-float over
// MASS_FLUSH rows and then moves the float-float sum into the FP64 Neumaier
// sum -- the mass of the stored FP32 state to ~1e-14, with the FP64 pipe
// (1/64 of the FP32 rate on this GPU) out of the inner loop.
// FP32 options for the mass fixer: MAXE records the largest biased exponent
// of |q| per tracer (a.emax_out); FIXR also sums, over the fixer's rows
// (fixer_row), all terms into the quantity nq + iq and the terms of the
// values with |q| < 2^(a.cls_emax - MASS_CLASS_SHIFT) (the small-value
// class) into the quantity 2 nq + iq.
constexpr int MASS_CHUNK = 4;
constexpr int MASS_FLUSH = 8;
constexpr int MASS_LOADS = 4;  // elements per lane whose loads are in flight together

// |q|'s bit pattern below which an FP32 value is in the small-value class
__device__ __forceinline__ unsigned class_cut(int emax) {
  const int e = emax - MASS_CLASS_SHIFT;
  return e > 0 ? (unsigned)e << 23 : 0u;
}

__device__ __forceinline__ unsigned mix32(unsigned x) {  // integer hash (xorshift-multiply)
  x ^= x >> 16;
  x *= 0x7feb352dU;
  x ^= x >> 15;
  x *= 0x846ca68bU;
  x ^= x >> 16;
  return x;
}

// the rows (tile, level, j) the FP32 fixer moves values in: a fixed
// pseudo-random 1/MASS_FIX_ROWS of them
__device__ __forceinline__ bool fixer_row(int r) {
  return (mix32((unsigned)r * 0x9e3779b9U + 0x7f4a7c15U) & (MASS_FIX_ROWS - 1)) == 0u;
}

__device__ __forceinline__ void ff_flush(double& s, double& c, FF& acc) {
  neumaier(s, c, (double)acc.hi);
  neumaier(s, c, (double)acc.lo);
  acc = FF{0.f, 0.f};
}

template <typename T, bool MAXE, bool FIXR>
__global__ void __launch_bounds__(256, 2) k_mass_partial(const MassArgs<T> a, int nq) {
  const int q0 = blockIdx.y * MASS_CHUNK;
  const int nc = min(MASS_CHUNK, nq - q0);
  const int lane = threadIdx.x & 31;
  const int rows = a.ntiles * a.npz * a.nj;
  double s[MASS_CHUNK], c[MASS_CHUNK], s2[MASS_CHUNK], c2[MASS_CHUNK], s3[MASS_CHUNK], c3[MASS_CHUNK];
  FF acc[MASS_CHUNK], acc2[MASS_CHUNK], acc3[MASS_CHUNK];
  unsigned top[MASS_CHUNK], cut[MASS_CHUNK];
#pragma unroll
  for (int m = 0; m < MASS_CHUNK; ++m) {
    s[m] = c[m] = s2[m] = c2[m] = s3[m] = c3[m] = 0.0;
    acc[m] = acc2[m] = acc3[m] = FF{0.f, 0.f};
    top[m] = 0u;
    cut[m] = (FIXR && m < nc) ? class_cut(a.cls_emax[q0 + m]) : 0u;
  }
  int pending = 0;
  for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += gridDim.x * (blockDim.x >> 5)) {
    const int j = r % a.nj;
    const int tk = r / a.nj;
    const int k = tk % a.npz, t = tk / a.npz;
    const long long p0 = a.pg.at(a.i1, a.j1 + j);
    const T* qr = a.q + t * a.sQt + q0 * a.sQq + k * a.sQk + p0;
    const T* dr = a.dp + t * a.sFt + k * a.sFk + p0;
    const T* ar = a.area + t * a.sMt + p0;
    if constexpr (Single<T>::value) {
      const bool sub = FIXR && fixer_row(r);  // warp-uniform
      // MASS_LOADS elements of the row per lane and round: their loads are issued together
      for (int i0 = lane; i0 < a.ni; i0 += 32 * MASS_LOADS) {
        float dv[MASS_LOADS], av[MASS_LOADS], qv[MASS_CHUNK][MASS_LOADS];
#pragma unroll
        for (int u = 0; u < MASS_LOADS; ++u) {
          const int i = i0 + 32 * u;
          const bool in = i < a.ni;
          dv[u] = in ? (float)dr[i] : 0.f;
          av[u] = in ? (float)ar[i] : 0.f;
#pragma unroll
          for (int m = 0; m < MASS_CHUNK; ++m) qv[m][u] = (in && m < nc) ? (float)qr[m * a.sQq + i] : 0.f;
        }
#pragma unroll
        for (int u = 0; u < MASS_LOADS; ++u) {
          const FF w = ff_prod(dv[u], av[u]);
#pragma unroll
          for (int m = 0; m < MASS_CHUNK; ++m) {
            const float v = qv[m][u];
            const float p = v * w.hi;
            const FF term{p, fmaf(v, w.lo, fmaf(v, w.hi, -p))};
            acc[m] = ff_add(acc[m], term);
            const unsigned mag = (unsigned)__float_as_int(v) & 0x7fffffffu;
            if (MAXE) top[m] = max(top[m], mag);
            if (sub) {
              acc2[m] = ff_add(acc2[m], term);
              if (mag < cut[m]) acc3[m] = ff_add(acc3[m], term);
            }
          }
        }
      }
      if (++pending == MASS_FLUSH) {
        pending = 0;
#pragma unroll
        for (int m = 0; m < MASS_CHUNK; ++m) {
          ff_flush(s[m], c[m], acc[m]);
          if (FIXR) {
            ff_flush(s2[m], c2[m], acc2[m]);
            ff_flush(s3[m], c3[m], acc3[m]);
          }
        }
      }
    } else {
      for (int i = lane; i < a.ni; i += 32) {
        const double w = (double)dr[i] * (double)ar[i];
#pragma unroll
        for (int m = 0; m < MASS_CHUNK; ++m)
          if (m < nc) neumaier(s[m], c[m], (double)qr[m * a.sQq + i] * w);
      }
    }
  }
  __shared__ double ss[256], sc[256];
#pragma unroll
  for (int m = 0; m < MASS_CHUNK; ++m) {
    if (m >= nc) continue;
    if (Single<T>::value) ff_flush(s[m], c[m], acc[m]);
    block_partial(s[m], c[m], a.partials, q0 + m, ss, sc);
    if (FIXR) {
      ff_flush(s2[m], c2[m], acc2[m]);
      ff_flush(s3[m], c3[m], acc3[m]);
      block_partial(s2[m], c2[m], a.partials, nq + q0 + m, ss, sc);
      block_partial(s3[m], c3[m], a.partials, 2 * nq + q0 + m, ss, sc);
    }
    if (MAXE) {
      unsigned tm = top[m];
      for (int o = 16; o > 0; o >>= 1) tm = max(tm, __shfl_xor_sync(0xffffffffu, tm, o));
      if (lane == 0 && tm != 0u) atomicMax(a.emax_out + q0 + m, (int)(tm >> 23));
    }
  }
}

__global__ void k_mass_final(const double* partials, int nblk, int nq, double* out) {
  const int iq = blockIdx.x;
  __shared__ double ss[256], sc[256];
  double s = 0.0, c = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    neumaier(s, c, partials[2 * ((long long)iq * nblk + b)]);
    c += partials[2 * ((long long)iq * nblk + b) + 1];
  }
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      double s0 = ss[threadIdx.x], c0 = sc[threadIdx.x] + sc[threadIdx.x + o];
      neumaier(s0, c0, ss[threadIdx.x + o]);
      ss[threadIdx.x] = s0;
      sc[threadIdx.x] = c0;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[iq] = ss[0] + sc[0];
}

template <typename T>
int launch_mass(const MassArgs<T>& a, int nq, double* d_out, cudaStream_t s) {
  const dim3 grid(MASS_BLOCKS, (nq + MASS_CHUNK - 1) / MASS_CHUNK);
  const bool fixr = Single<T>::value && a.cls_emax != nullptr;
  const bool maxe = Single<T>::value && a.emax_out != nullptr;
  if (fixr && maxe) return set_error(FV3G_E_ARG, "mass sum: one of the fixer-row sums and the exponent maximum");
  if (fixr) k_mass_partial<T, false, true><<<grid, 256, 0, s>>>(a, nq);
  else if (maxe) k_mass_partial<T, true, false><<<grid, 256, 0, s>>>(a, nq);
  else k_mass_partial<T, false, false><<<grid, 256, 0, s>>>(a, nq);
  FV3G_CUDA(cudaGetLastError());
  const int nout = fixr ? 3 * nq : nq;
  k_mass_final<<<nout, 256, 0, s>>>(a.partials, MASS_BLOCKS, nout, d_out);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

// ------------------------------------------------------------ mass fixer ---
// Restore each tracer's global mass after a step, mass0[iq] (at the step's
// start) from mass1[iq] (after the remap):
//   FP64 values: q <- q (1 + eps), eps = (mass0 - mass1)/mass1, rounded (one
//     pass; the roundings leave ~1e-16 of the mass).
//   FP32 values: only values in the fixer's rows (a fixed pseudo-random
//     1/MASS_FIX_ROWS of the rows) move, by eps = (mass0 - mass1)/(the rows'
//     mass), ~1e-9 relative.  A value moves by k ulps, k = floor(eps |q| /
//     ulp(q) + h), h in [0, 1) from a Weyl sequence over the value's place,
//     offset by a hash of mass1 (so it changes from step to step): unbiased
//     dithered rounding of q (1 + eps), so k is 0 for almost every value and
//     only the values that move are written; zero and denormal values stay.
//     The moved values leave a residual of the order of the ulps of the
//     largest values (~1e-12 of the mass when a few percent of the cells
//     carry it), so the first pass also sums the exact mass it moved, dm,
//     and the part of it inside the small-value class (|q| below
//     2^-MASS_CLASS_SHIFT of the tracer's largest binade), dmc; a second pass
//     moves only those small values, by eps_c = residual / (their mass),
//     whose ulps are 2^-MASS_CLASS_SHIFT finer: ~1e-14 of the mass.  Where
//     the rows or their class carry no positive mass or the factor would
//     exceed 2^-20, that pass acts on every value of every row (first pass)
//     or of the fixer's rows (second pass) instead.
constexpr int FIX_LOADS = 8;

// pass 1: dm == nullptr, sums the moved mass (quantity iq) and the class
// mass it moved in the fixer's rows (quantity nq + iq) into the partials;
// pass 2: dm holds them.  mass1c: the mass, the fixer rows' mass and their
// class mass (3 nq).
template <typename T>
__global__ void __launch_bounds__(256) k_mass_fix(const MassArgs<T> a, T* q, int nq, int iq_base,
                                                  const double* mass0, const double* mass1c, const double* dm,
                                                  const int* emax) {
  const int iq = blockIdx.y;
  const bool second = dm != nullptr;
  const double m0 = mass0[iq];
  double m1 = mass1c[iq], eps = 0.0;
  const bool finite = m0 == m0 && m1 == m1;
  unsigned cut = 0xffffffffu;  // |q| bit patterns below it may move
  bool all_rows = !Single<T>::value;
  if (!second) {
    const double ms = mass1c[nq + iq], e = ms > 0.0 ? (m0 - m1) / ms : 0.0;
    if (!Single<T>::value || !(ms > 0.0) || !(fabs(e) <= 0x1p-20)) {
      all_rows = true;
      if (m1 != 0.0 && finite) eps = (m0 - m1) / m1;
    } else {
      eps = e;
    }
  } else {
    m1 += dm[iq];
    const double res = m0 - m1, cm = mass1c[2 * nq + iq] + dm[nq + iq];
    const double ec = cm > 0.0 ? res / cm : 0.0;
    if (cm > 0.0 && fabs(ec) <= 0x1p-20) {
      eps = ec;
      cut = class_cut(emax[iq]);
    } else {
      // the fixer rows' mass after the first pass (exact when that pass moved values in those rows only)
      const double ms = mass1c[nq + iq] + dm[iq];
      if (ms > 0.0 && finite) eps = fmax(fmin(res / ms, 0x1p-20), -0x1p-20);
    }
  }
  const unsigned ccut = Single<T>::value ? class_cut(emax[iq]) : 0u;
  const int lane = threadIdx.x & 31;
  const int rows = a.ntiles * a.npz * a.nj;
  double s = 0.0, c = 0.0, s2 = 0.0, c2 = 0.0;  // FP32 pass 1: the moved mass, of it the class's in fixer rows
  if (eps != 0.0) {
    const unsigned long long mb = (unsigned long long)__double_as_longlong(m1);
    const unsigned seed =
        mix32((unsigned)mb ^
              mix32((unsigned)(mb >> 32) + 0x9e3779b9U * (unsigned)(iq_base + iq + 1) + (second ? 7u : 0u)));
    for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows;
         r += gridDim.x * (blockDim.x >> 5)) {
      const bool sub = fixer_row(r);
      if (!all_rows && !sub) continue;
      const int j = r % a.nj;
      const int tk = r / a.nj;
      const int k = tk % a.npz, t = tk / a.npz;
      const long long p0 = a.pg.at(a.i1, a.j1 + j);
      T* qr = q + t * a.sQt + iq * a.sQq + k * a.sQk + p0;
      if constexpr (!Single<T>::value) {
        for (int i = lane; i < a.ni; i += 32) qr[i] = (T)((double)qr[i] * (1.0 + eps));
        continue;
      }
      // FIX_LOADS elements of the row per lane and round: their loads are issued together
      for (int i0 = lane; i0 < a.ni; i0 += 32 * FIX_LOADS) {
        float vv[FIX_LOADS];
#pragma unroll
        for (int u = 0; u < FIX_LOADS; ++u) vv[u] = i0 + 32 * u < a.ni ? (float)qr[i0 + 32 * u] : 0.f;
#pragma unroll
        for (int u = 0; u < FIX_LOADS; ++u) {
          const int i = i0 + 32 * u;
          const float v = vv[u];
          const int bits = __float_as_int(v);
          const unsigned mag = (unsigned)bits & 0x7fffffffu;
          const int ex = (int)(mag >> 23);
          if (ex == 0 || ex == 0xff || mag >= cut) continue;  // zero, denormal, inf, nan; outside the class
          const float mant = (float)((bits & 0x7fffff) | 0x800000);  // |v| / ulp(v), exact
          const unsigned wy = seed + ((unsigned)r * (unsigned)a.ni + (unsigned)i) * 0x9e3779b9U;  // Weyl, 2^32/phi
          const float h = (float)(wy >> 8) * (1.0f / 16777216.0f);
          const int kk = (int)floorf((float)eps * mant + h);
          if (kk == 0 || kk > (1 << 22) || kk < -(1 << 22)) continue;
          const int nbits = bits + kk;  // the magnitude moves by kk ulps, either sign
          const float nv = __int_as_float(nbits);
          qr[i] = (T)nv;
          if (!second) {  // nv - v is exact (the two are within a factor 2)
            const T* dr = a.dp + t * a.sFt + k * a.sFk + p0;
            const T* ar = a.area + t * a.sMt + p0;
            const double w = (double)dr[i] * (double)ar[i];
            neumaier(s, c, (double)(nv - v) * w);
            const bool in0 = mag < ccut, in1 = ((unsigned)nbits & 0x7fffffffu) < ccut;
            if (sub && (in0 || in1)) neumaier(s2, c2, ((in1 ? (double)nv : 0.0) - (in0 ? (double)v : 0.0)) * w);
          }
        }
      }
    }
  }
  if (Single<T>::value && !second) {
    __shared__ double ss[256], sc[256];
    block_partial(s, c, a.partials, iq, ss, sc);
    block_partial(s2, c2, a.partials, nq + iq, ss, sc);
  }
}

template <typename T>
int launch_mass_fix(const MassArgs<T>& a, T* q, int nq, int iq_base, const double* mass0, const double* mass1c,
                    double* dm, const int* emax, cudaStream_t s) {
  k_mass_fix<T><<<dim3(MASS_BLOCKS, nq), 256, 0, s>>>(a, q, nq, iq_base, mass0, mass1c, nullptr, emax);
  FV3G_CUDA(cudaGetLastError());
  if (Single<T>::value) {
    k_mass_final<<<2 * nq, 256, 0, s>>>(a.partials, MASS_BLOCKS, 2 * nq, dm);
    FV3G_CUDA(cudaGetLastError());
    k_mass_fix<T><<<dim3(MASS_BLOCKS, nq), 256, 0, s>>>(a, q, nq, iq_base, mass0, mass1c, dm, emax);
    FV3G_CUDA(cudaGetLastError());
  }
  return 0;
}

template int launch_mass_fix<float>(const MassArgs<float>&, float*, int, int, const double*, const double*,
                                    double*, const int*, cudaStream_t);
template int launch_mass_fix<double>(const MassArgs<double>&, double*, int, int, const double*, const double*,
                                     double*, const int*, cudaStream_t);
template int launch_mass<float>(const MassArgs<float>&, int, double*, cudaStream_t);
template int launch_mass<double>(const MassArgs<double>&, int, double*, cudaStream_t);

}  // namespace fv3g
