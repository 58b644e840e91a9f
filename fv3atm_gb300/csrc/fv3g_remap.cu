// fv3g_remap.cu -- Lagrangian-to-Eulerian column remap (map_scalar / map1_ppm
// with the cs_profile reconstruction of fv_mapz.F90, GFDL_atmos_cubed_sphere,
// absent submodule .gitmodules:1-4).
//
// Two kernels share the schemes of fv3g_profile.cuh:
//   * k_remap_warp, the batched and drop-in remap: one warp per column, lane l
//     owning interfaces / layers l*NPL .. l*NPL+NPL-1, the column's constants
//     (interface pressures, overlap schedule, LU factors of the interface
//     system) in registers for all its fields, the recurrences as warp scans
//     (see the comment above the kernel);
//   * k_remap_scratch, one thread per column with its column arrays in a
//     caller-owned scratch buffer laid out [level][column], for the
//     allocation-free entry and the tangent-linear remap.
// Per column, once for all fields: the Lagrangian interface pressures pe1
// (FP64 running sum of delp), the target interfaces pe2 = ak + bk*ps (FP64),
// the overlap schedule (for every target interface the source layer that
// holds it and its fractional position) and the LU factors of the C1 system.
// Per field: the interface values (kord 9: forward and back substitution;
// kord 4: the explicit PPM stencil), the kord constraints, and the
// integration of the sub-grid parabolas over the overlaps.  The FP32
// thread-per-column form of the batched remap is fv3g_remap_col.cu.
#include <algorithm>
#include <cfloat>
#include <mutex>
#include <type_traits>

#include "fv3g_ff.cuh"
#include "fv3g_internal.cuh"
#include "fv3g_profile.cuh"
#include "fv3g_remap.cuh"

namespace fv3g {


// mean of the parabola (aL, aR, a6) over the fractional interval [x1, x2]
template <typename T> __device__ __forceinline__ T pmean(T l, T r, T s6, T x1, T x2) {
  return l + T(0.5) * (x1 + x2) * ((r - l) + s6) - s6 * ((x2 * x2 + x1 * x2 + x1 * x1) * T(1.0 / 3.0));
}

// Thread-per-column form with a global scratch (the caller's fixed buffer);
// used where the library may not allocate (fv3g_remap_columns_noalloc).
template <typename T, int KORD>
__global__ void __launch_bounds__(128) k_remap_scratch(const RemapArgs<T> a) {
  const long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= a.ncol) return;
  const int km = a.km, kn = a.kn;
  const long long nc = a.ncol;
  // column -> (tile, i, j) -> field offset
  const int ci = (int)(col % a.ni);
  const long long rest = col / a.ni;
  const int cj = (int)(rest % a.nj);
  const int ct = (int)(rest / a.nj);
  const long long fo = ct * a.sFt + a.pg.at(a.i1 + ci, a.j1 + cj);  // per-level fields
  const long long qo = ct * a.sQt + a.pg.at(a.i1 + ci, a.j1 + cj);  // tracer fields

  // scratch arrays, [level][column]
  T* s_dp = a.scratch + 0 * (long long)(KMAX + 1) * nc;
  T* s_cp = a.scratch + 1 * (long long)(KMAX + 1) * nc;
  T* s_rd = a.scratch + 2 * (long long)(KMAX + 1) * nc;
  T* s_d = a.scratch + 3 * (long long)(KMAX + 1) * nc;
  T* s_x = a.scratch + 4 * (long long)(KMAX + 1) * nc;
  T* s_a = a.scratch + 5 * (long long)(KMAX + 1) * nc;
  unsigned char* s_L = a.sched + 0;
#define SC(arr, k) arr[(long long)(k) * nc + col]

  // ------------------------------------------------ pressures and schedule
  double ptop, ps;
  if (a.pe1 != nullptr) {
    ptop = a.pe1[col];
    ps = a.pe1[(long long)km * nc + col];
  } else {
    ptop = a.ak[0];
    double s = ptop;
    for (int k = 0; k < km; ++k) s += value_of(a.dp[fo + k * a.sFk]);
    ps = s;
  }
  auto pe2_at = [&](int k) -> double {
    if (a.pe2 != nullptr) return a.pe2[(long long)k * nc + col];
    return a.ak[k] + a.bk[k] * ps;
  };
  auto dp_src = [&](int k) -> double { return value_of(a.dp[fo + k * a.sFk]); };
  // source thickness (from pe differences, as the oracle) and schedule
  {
    double p1 = ptop;
    for (int k = 0; k < km; ++k) {
      double p2 = (a.pe1 != nullptr) ? a.pe1[(long long)(k + 1) * nc + col] : p1 + dp_src(k);
      SC(s_dp, k) = T(p2 - p1);
      p1 = p2;
    }
    if (a.dp_out != nullptr)
      for (int k = 0; k < kn; ++k) a.dp_out[fo + k * a.sFk] = T(pe2_at(k + 1) - pe2_at(k));
    // merge: the source layer containing each target interface
    int k1 = 0;
    double lo = ptop;
    double hi = (a.pe1 != nullptr) ? a.pe1[(long long)nc + col] : ptop + dp_src(0);
    for (int k2 = 0; k2 <= kn; ++k2) {
      const double p = pe2_at(k2);
      while (k1 < km - 1 && hi <= p) {
        ++k1;
        lo = hi;
        hi = (a.pe1 != nullptr) ? a.pe1[(long long)(k1 + 1) * nc + col] : hi + dp_src(k1);
      }
      s_L[(long long)k2 * nc + col] = (unsigned char)k1;
      SC(s_x, k2) = Single<T>::value ? T(float(p - lo) / float(hi - lo)) : T((p - lo) / (hi - lo));
    }
  }
  // LU factors of the kord 9 interface system (rows 0..km)
  if (KORD == 9 && km > 1) {
    const T g = SC(s_dp, 1) / SC(s_dp, 0);
    T di = g, up = g + T(1);
    T cp = up / di;
    SC(s_cp, 0) = cp;
    SC(s_rd, 0) = T(1) / di;
    for (int k = 1; k < km; ++k) {
      const T d = SC(s_dp, k - 1) / SC(s_dp, k);
      SC(s_d, k) = d;
      const T den = T(2) * (T(1) + d) - cp;
      const T rden = T(1) / den;
      cp = d * rden;
      SC(s_cp, k) = cp;
      SC(s_rd, k) = rden;
    }
    T lo, dd;
    if (a.iv == -2) { lo = T(0); dd = T(1); }
    else {
      const T gb = SC(s_dp, km - 2) / SC(s_dp, km - 1);
      lo = gb + T(1);
      dd = gb;
      SC(s_d, km) = gb;
    }
    const T den = dd - lo * cp;
    SC(s_rd, km) = T(1) / den;
    SC(s_cp, km) = lo;  // bottom row keeps its sub-diagonal in cp[km]
  }

  const T floor_v = (a.iv == 1) ? T(a.q_min) : T(0);
  for (int f = 0; f < a.nfield; ++f) {
    const T* q1 = a.q_in + qo + f * a.sQq;
    T* q2 = a.q_out + qo + f * a.sQqo;
    const T qsv = a.qs ? T(a.qs[col]) : T(0);
    auto qf = [&](int k) -> T { return q1[(long long)min(max(k, 0), km - 1) * a.sQk]; };
    auto hf = [&](int k) -> T { return SC(s_dp, min(max(k, 0), km - 1)); };
    // -------------------------------------------- interface values a[0..km]
    if (km == 1) {
      SC(s_a, 0) = q1[0];
      SC(s_a, 1) = q1[0];
    } else if (KORD == 9) {
      const T g = SC(s_dp, 1) / SC(s_dp, 0);
      T qm = q1[0], qk = q1[a.sQk];
      T ap = ((g * (T(2) * g + T(3))) * qm + qk) / (g + T(1)) * SC(s_rd, 0);
      SC(s_a, 0) = ap;
      for (int k = 1; k < km; ++k) {
        qk = q1[k * a.sQk];
        const T rhs = T(3) * (qm + SC(s_d, k) * qk);
        ap = (rhs - ap) * SC(s_rd, k);
        SC(s_a, k) = ap;
        qm = qk;
      }
      T rhs;
      if (a.iv == -2) rhs = qsv;
      else {
        const T gb = SC(s_d, km);
        rhs = ((gb * (T(2) * gb + T(3))) * q1[(km - 1) * a.sQk] + q1[(km - 2) * a.sQk]) / (gb + T(1));
      }
      // back substitution on the raw values; each interface is limited on its own
      T av = (rhs - SC(s_cp, km) * ap) * SC(s_rd, km);
      SC(s_a, km) = k9_interface_f(av, km, km, a.iv, floor_v, qf);
      for (int k = km - 1; k >= 0; --k) {
        av = SC(s_a, k) - SC(s_cp, k) * av;
        SC(s_a, k) = k9_interface_f(av, k, km, a.iv, floor_v, qf);
      }
    } else {
      // kord 4: the layer slopes (kept in s_d), then the PPM interfaces
      for (int k = 0; k < km; ++k) SC(s_d, k) = ppm_slope_f<T>(k, km, qf, hf);
      for (int u = 0; u <= km; ++u)
        SC(s_a, u) = ppm_interface<T>(u, km, a.iv, qsv, u >= 1 ? SC(s_d, u - 1) : T(0), u < km ? SC(s_d, u) : T(0),
                                      qf, hf);
    }
    // ------------------------------------------------------- integration
    int kc = -1;  // layer whose profile is cached
    Profile<T> P{};
    auto prof = [&](int k) -> const Profile<T>& {
      if (k != kc) {
        P = layer_profile_f<T, KORD>(k, km, q1[k * a.sQk], SC(s_a, k), SC(s_a, k + 1), KORD == 9 ? T(0) : SC(s_d, k),
                                   a.iv, floor_v, qf);
        kc = k;
      }
      return P;
    };
    int Lt = s_L[col];
    T Xt = SC(s_x, 0);
    for (int k2 = 0; k2 < kn; ++k2) {
      const int Lb = s_L[(long long)(k2 + 1) * nc + col];
      const T Xb = SC(s_x, k2 + 1);
      T out;
      const bool inside = (Lb == Lt) || (Lb == Lt + 1 && Xb == T(0));
      if (inside) {
        if (Xt == T(0) && (Lb == Lt + 1 || Xb == T(1))) {
          out = q1[Lt * a.sQk];
        } else {
          const Profile<T>& p = prof(Lt);
          out = pmean(p.l, p.r, p.s6, Xt, Lb == Lt ? Xb : T(1));
        }
      } else {
        T mass;
        const T dpt = SC(s_dp, Lt);
        if (Xt == T(0)) mass = q1[Lt * a.sQk] * dpt;
        else {
          const Profile<T>& p = prof(Lt);
          mass = (dpt * (T(1) - Xt)) * pmean(p.l, p.r, p.s6, Xt, T(1));
        }
        for (int m = Lt + 1; m < Lb; ++m) mass = mass + q1[m * a.sQk] * SC(s_dp, m);
        const T dpb = SC(s_dp, Lb);
        if (Xb >= T(1)) {
          mass = mass + q1[Lb * a.sQk] * (dpb * Xb);
        } else if (Xb > T(0)) {
          const Profile<T>& p = prof(Lb);
          mass = mass + (dpb * Xb) * pmean(p.l, p.r, p.s6, T(0), Xb);
        }
        // target thickness from the FP64 interface pressures (or the caller's)
        const T dpk = a.dp2 ? T(a.dp2[(long long)k2 * nc + col]) : T(pe2_at(k2 + 1) - pe2_at(k2));
        out = mass / dpk;
      }
      q2[k2 * a.sQk] = out;
      Lt = Lb;
      Xt = Xb;
    }
  }
#undef SC
}

// ------------------------------------------------ warp-per-column form ---
// One warp per column; lane l owns interfaces / layers u = l*NPL .. l*NPL+NPL-1,
// so the column's constants stay in registers for all fields.  The three
// first-order recurrences of the column are evaluated as warp scans and then
// re-run locally with the sequential formulas from the scanned start value:
//   * the FP64 running sum of delp (interface pressures pe1);
//   * the LU pivots of the interface system, cp_u = d_u / (2(1+d_u) - cp_{u-1}),
//     a Moebius map composed as 2x2 matrices (scaled by powers of two, exact);
//   * per field, forward substitution y_u = (rhs_u - y_{u-1}) rd_u and back
//     substitution a_u = y_u - cp_u a_{u+1}, affine maps composed in the scan.
// The overlap schedule (source layer and fractional position of every target
// interface) is a binary search in the warp's copy of pe1.
// Shared arrays indexed by level take one pad element per 32 floats (16
// doubles), so that lane l reading level 4l+j (the blocked ownership) hits
// distinct banks.
template <typename T>
__host__ __device__ constexpr int pk(int k) { return k + (k >> (sizeof(T) == 8 ? 4 : 5)); }

// Fields per pass of the warp kernel: FP32 columns advance two fields at a
// time, so the lane-to-lane scans of both interleave (the scans are latency
// chains of shuffles); FP64 keeps one (its ring has three slots).
template <typename T>
__host__ __device__ constexpr int fields_per_pass() { return sizeof(T) == 4 ? 2 : 1; }

template <typename T, int NPL>
struct ColSmem {
  static constexpr int FP = fields_per_pass<T>();
  double pe1[pk<double>(32 * NPL) + 1];
  T dp[pk<T>(32 * NPL)];
  T pl[FP][pk<T>(32 * NPL)];  // sub-grid parabola of every source layer: left, right edge and curvature
  T pr[FP][pk<T>(32 * NPL)];
  T p6[FP][pk<T>(32 * NPL)];
  float mh[FP][pk<float>(32 * NPL) + 1];  // FP32 fields: cumulative layer mass at every source interface,
  float ml[FP][pk<float>(32 * NPL) + 1];  // as an unevaluated sum hi + lo (float-float)
};

// Fields reach shared memory through a ring of RING slots, filled by
// cp.async RING-1 fields ahead.  Each slot holds the CTA's 8 columns,
// [column][padded level].  The CTA's threads copy it together:
// thread t moves levels t/8 + 32r of column t%8, so 8 consecutive threads read
// one 32-byte sector (consecutive columns are consecutive i).
template <typename T>
__host__ __device__ constexpr int ring_slots() { return sizeof(T) == 8 ? 3 : 4; }

// Columns (warps) per CTA of the warp remap; its threads copy one level of
// all RCOL columns at a time (8 FP32 columns: one 32-byte sector; 4 measured
// 9 % slower at C384 L127 x 20).
constexpr int RCOL = 8;

// Slot pitch per column: room for the padded levels, and a residue (4 mod 32
// floats, 2 mod 16 doubles) that spreads the 8 columns of one copy
// instruction over distinct banks.
template <typename T, int NPL>
__host__ __device__ constexpr int ring_pitch() {
  int p = pk<T>(32 * NPL) + 1;
  while (sizeof(T) == 8 ? (p % 16 != 2) : (p % 32 != 4)) ++p;
  return p;
}

template <typename T, int NPL>
__host__ __device__ constexpr size_t remap_warp_smem() {
  return RCOL * sizeof(ColSmem<T, NPL>) + (size_t)ring_slots<T>() * RCOL * ring_pitch<T, NPL>() * sizeof(T);
}

template <typename T>
__device__ __forceinline__ void cp_async_elem(T* dst, const T* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  if (sizeof(T) == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
  else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// 2^-e with e the binary exponent of m > 0: m * pow2_recip(m) lies in [1, 2)
__device__ __forceinline__ float pow2_recip(float m) {
  const int e = (__float_as_int(m) >> 23) & 0xff;
  return __int_as_float((254 - e) << 23);
}
__device__ __forceinline__ double pow2_recip(double m) {
  const long long e = (__double_as_longlong(m) >> 52) & 0x7ff;
  return __longlong_as_double((2046 - e) << 52);
}

template <typename T>
struct Mat2 {  // [[a, b], [c, d]]
  T a, b, c, d;
};

// m2 * m1 (m1 applied first), rescaled by a power of two
template <typename T>
__device__ __forceinline__ Mat2<T> mat_after(const Mat2<T>& m2, const Mat2<T>& m1) {
  Mat2<T> r{m2.a * m1.a + m2.b * m1.c, m2.a * m1.b + m2.b * m1.d, m2.c * m1.a + m2.d * m1.c,
            m2.c * m1.b + m2.d * m1.d};
  const T s = pow2_recip(tmax(tmax(tabs(r.a), tabs(r.b)), tmax(tabs(r.c), tabs(r.d))));
  r.a *= s; r.b *= s; r.c *= s; r.d *= s;
  return r;
}

template <typename T>
__device__ __forceinline__ Mat2<T> shfl_up_mat(const Mat2<T>& m, int o) {
  return Mat2<T>{__shfl_up_sync(0xffffffffu, m.a, o), __shfl_up_sync(0xffffffffu, m.b, o),
                 __shfl_up_sync(0xffffffffu, m.c, o), __shfl_up_sync(0xffffffffu, m.d, o)};
}

// Affine map x -> al * x + be.  Inclusive scans: forward (lane-o first) and
// backward (lane+o first); both return the exclusive prefix's offset, i.e.
// the recurrence value entering this lane's first (forward) or last
// (backward) element, given that the chain starts with a constant map.
//
// The multipliers of the remap's substitution scans depend on the column only
// (the LU factors), not on the field: their values entering each of the five
// scan steps are computed once per column (scan_muls_*), and each field's
// scans then move only their offsets, N chains interleaved (one shuffle and
// one multiply-add per step and chain).
template <typename T>
__device__ __forceinline__ void scan_muls_fwd(T al, T (&m)[5], int lane) {
#pragma unroll
  for (int o = 1, s = 0; o < 32; o <<= 1, ++s) {
    m[s] = al;
    const T pa = __shfl_up_sync(0xffffffffu, al, o);
    if (lane >= o) al = al * pa;
  }
}
template <typename T>
__device__ __forceinline__ void scan_muls_bwd(T al, T (&m)[5], int lane) {
#pragma unroll
  for (int o = 1, s = 0; o < 32; o <<= 1, ++s) {
    m[s] = al;
    const T pa = __shfl_down_sync(0xffffffffu, al, o);
    if (lane + o < 32) al = al * pa;
  }
}
template <typename T, int N>
__device__ __forceinline__ void affine_enter_fwd_m(const T (&m)[5], T (&be)[N], T (&out)[N], int lane) {
#pragma unroll
  for (int o = 1, s = 0; o < 32; o <<= 1, ++s) {
    T pb[N];
#pragma unroll
    for (int h = 0; h < N; ++h) pb[h] = __shfl_up_sync(0xffffffffu, be[h], o);
#pragma unroll
    for (int h = 0; h < N; ++h)
      if (lane >= o) be[h] = m[s] * pb[h] + be[h];
  }
#pragma unroll
  for (int h = 0; h < N; ++h) out[h] = __shfl_up_sync(0xffffffffu, be[h], 1);
}
template <typename T, int N>
__device__ __forceinline__ void affine_enter_bwd_m(const T (&m)[5], T (&be)[N], T (&out)[N], int lane) {
#pragma unroll
  for (int o = 1, s = 0; o < 32; o <<= 1, ++s) {
    T pb[N];
#pragma unroll
    for (int h = 0; h < N; ++h) pb[h] = __shfl_down_sync(0xffffffffu, be[h], o);
#pragma unroll
    for (int h = 0; h < N; ++h)
      if (lane + o < 32) be[h] = m[s] * pb[h] + be[h];
  }
#pragma unroll
  for (int h = 0; h < N; ++h) out[h] = __shfl_down_sync(0xffffffffu, be[h], 1);
}

template <typename T>
__device__ __forceinline__ T affine_enter_fwd(T al, T be, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T pa = __shfl_up_sync(0xffffffffu, al, o), pb = __shfl_up_sync(0xffffffffu, be, o);
    if (lane >= o) {
      be = al * pb + be;
      al = al * pa;
    }
  }
  return __shfl_up_sync(0xffffffffu, be, 1);
}
template <typename T>
__device__ __forceinline__ T affine_enter_bwd(T al, T be, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const T pa = __shfl_down_sync(0xffffffffu, al, o), pb = __shfl_down_sync(0xffffffffu, be, o);
    if (lane + o < 32) {
      be = al * pb + be;
      al = al * pa;
    }
  }
  return __shfl_down_sync(0xffffffffu, be, 1);
}

template <typename T, int KORD, int NPL>
__global__ void __launch_bounds__(32 * RCOL, sizeof(T) == 4 ? 2 : 1) k_remap_warp(const RemapArgs<T> a) {
  constexpr int RING = ring_slots<T>(), RP = ring_pitch<T, NPL>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  ColSmem<T, NPL>& S = reinterpret_cast<ColSmem<T, NPL>*>(smem_raw)[warp];
  T* const ring = reinterpret_cast<T*>(smem_raw + RCOL * sizeof(ColSmem<T, NPL>));
  const int nc = (int)a.ncol;  // launch_remap checks that it fits in an int
  const int col0 = blockIdx.x * RCOL;
  // the last CTA's surplus warps repeat the last column and store nothing
  const bool real = col0 + warp < nc;
  const int col = real ? col0 + warp : nc - 1;
  auto offsets = [&a](int c, long long& fo_, long long& qo_) {
    const unsigned ni = (unsigned)a.ni, nj = (unsigned)a.nj;
    const unsigned rest = (unsigned)c / ni, ci = (unsigned)c - rest * ni;
    const unsigned ct = rest / nj, cj = rest - ct * nj;
    fo_ = ct * a.sFt + a.pg.at(a.i1 + ci, a.j1 + cj);
    qo_ = ct * a.sQt + a.pg.at(a.i1 + ci, a.j1 + cj);
  };
  long long fo, qo;
  offsets(col, fo, qo);
  const int km = a.km, kn = a.kn;
  const int u0 = lane * NPL;  // first interface / layer of this lane

  // cooperative field copy: this thread's column and levels
  const int cc = threadIdx.x % RCOL, kk = threadIdx.x / RCOL;
  long long fo_c, qo_c;
  offsets(min(col0 + cc, nc - 1), fo_c, qo_c);
  auto issue = [&](int f) {
    if (f < a.nfield) {
      const T* src = a.q_in + qo_c + f * a.sQq;
      T* dst = ring + ((f % RING) * RCOL + cc) * RP;
#pragma unroll
      for (int r = 0; r < NPL; ++r) {
        const int k = kk + 32 * r;
        if (k < km) cp_async_elem(dst + pk<T>(k), src + (long long)k * a.sQk);
      }
    }
    cp_async_commit();
  };
#pragma unroll
  for (int f = 0; f < RING - fields_per_pass<T>(); ++f) issue(f);

  // ------------------------------------------------ interface pressures pe1
  if (a.pe1 != nullptr) {
#pragma unroll
    for (int j = 0; j < NPL; ++j)
      if (u0 + j <= km) S.pe1[pk<double>(u0 + j)] = a.pe1[(long long)(u0 + j) * nc + col];
  } else {
    const double ptop = a.ak[0];
    double dl[NPL], tot = 0.0;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
      dl[j] = (u0 + j < km) ? (double)a.dp[fo + (long long)(u0 + j) * a.sFk] : 0.0;
      tot += dl[j];
    }
    double excl = affine_enter_fwd<double>(1.0, tot, lane);  // sum over lower lanes
    double s = lane == 0 ? ptop : ptop + excl;
    if (lane == 0) S.pe1[pk<double>(0)] = ptop;
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
      s += dl[j];
      if (u0 + j < km) S.pe1[pk<double>(u0 + j + 1)] = s;
    }
  }
  __syncwarp();
  const double ps = S.pe1[pk<double>(km)];
  auto pe2_at = [&](int k) -> double {
    if (a.pe2 != nullptr) return a.pe2[(long long)k * nc + col];
    return a.ak[k] + a.bk[k] * ps;
  };
#pragma unroll
  for (int j = 0; j < NPL; ++j)
    if (u0 + j < km) S.dp[pk<T>(u0 + j)] = T(S.pe1[pk<double>(u0 + j + 1)] - S.pe1[pk<double>(u0 + j)]);
  __syncwarp();

  // ----------------------------------------- overlap schedule, target dp
  // Source layer k1 holding target interface p: the number of interior source
  // interfaces at or above p (a short walk from the target's own index).
  int Ls[NPL + 1];
  T Xs[NPL + 1], dpk[NPL];
  double p2v[NPL + 1];
#pragma unroll
  for (int j = 0; j <= NPL; ++j) {
    const int k2 = min(u0 + j, kn);
    const double p = pe2_at(k2);
    p2v[j] = p;
    int k1 = min(k2, km - 1);
    while (k1 > 0 && S.pe1[pk<double>(k1)] > p) --k1;
    while (k1 < km - 1 && S.pe1[pk<double>(k1 + 1)] <= p) ++k1;
    const double pl = S.pe1[pk<double>(k1)], ph = S.pe1[pk<double>(k1 + 1)];
    Ls[j] = k1;
    Xs[j] = Single<T>::value ? T(float(p - pl) / float(ph - pl)) : T((p - pl) / (ph - pl));
  }
#pragma unroll
  for (int j = 0; j < NPL; ++j) {
    const int t = u0 + j;
    dpk[j] = (t < kn) ? (a.dp2 ? T(a.dp2[(long long)t * nc + col]) : T(p2v[j + 1] - p2v[j])) : T(1);
    if (real && t < kn && a.dp_out != nullptr) a.dp_out[fo + (long long)t * a.sFk] = dpk[j];
  }

  // ------------------------------------------- LU of the interface system
  // Row u of the system: rhs_u = wa q_a + wb q_b + wc qs with layers a, b =
  // u-1, u (top row: 0, 1; bottom row: km-1, km-2), forward step
  // y_u = (rhs_u - mco_u y_{u-1}) rd_u, back step a_u = y_u - cpb_u a_{u+1};
  // rows above km have rd = 0.  kord 4 has no system: its interfaces are an
  // explicit stencil.
  T wa[NPL], wb[NPL], wc[NPL], mco[NPL], rdv[NPL], cpb[NPL];
#pragma unroll
  for (int j = 0; j < NPL; ++j) wa[j] = wb[j] = wc[j] = mco[j] = rdv[j] = cpb[j] = T(0);
  if (KORD == 9 && km > 1) {
    const T g = S.dp[pk<T>(1)] / S.dp[pk<T>(0)];
    T dd[NPL];
    Mat2<T> m{T(1), T(0), T(0), T(1)};
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
      const int u = u0 + j;
      dd[j] = (u >= 1 && u < km) ? S.dp[pk<T>(u - 1)] / S.dp[pk<T>(u)] : T(0);
      if (u >= 1 && u < km) m = mat_after(Mat2<T>{T(0), dd[j], T(-1), T(2) * (T(1) + dd[j])}, m);
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const Mat2<T> p = shfl_up_mat(m, o);
      if (lane >= o) m = mat_after(m, p);
    }
    const Mat2<T> e = shfl_up_mat(m, 1);
    const T cp0 = (g + T(1)) / g;
    T cprev = (e.a * cp0 + e.b) / (e.c * cp0 + e.d);  // cp of interface u0-1 (lanes >= 1)
    const T gb = S.dp[pk<T>(km - 2)] / S.dp[pk<T>(km - 1)];
    const T lo_b = a.iv == -2 ? T(0) : gb + T(1);
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
      const int u = u0 + j;
      if (u == 0) {
        rdv[j] = T(1) / g;
        cpb[j] = cp0;
        wa[j] = (g * (T(2) * g + T(3))) / (g + T(1));
        wb[j] = T(1) / (g + T(1));
      } else if (u < km) {
        rdv[j] = T(1) / (T(2) * (T(1) + dd[j]) - cprev);
        cpb[j] = dd[j] * rdv[j];
        mco[j] = T(1);
        wa[j] = T(3);
        wb[j] = T(3) * dd[j];
      } else if (u == km) {
        rdv[j] = T(1) / ((a.iv == -2 ? T(1) : gb) - lo_b * cprev);
        mco[j] = lo_b;
        if (a.iv == -2) {
          wc[j] = T(1);
        } else {
          wa[j] = (gb * (T(2) * gb + T(3))) / (gb + T(1));
          wb[j] = T(1) / (gb + T(1));
        }
      }
      cprev = cpb[j];
    }
  }

  const T floor_v = (a.iv == 1) ? T(a.q_min) : T(0);
  const T qsv = a.qs ? T(a.qs[col]) : T(0);
  T rdpk[NPL];
#pragma unroll
  for (int j = 0; j < NPL; ++j) rdpk[j] = T(1) / dpk[j];
  // the substitution scans' multipliers (column constants): forward a_j = -mco_j rd_j, backward -cp_j
  T ajv[NPL], mf[5], mb[5];
  {
    T alf = T(1), alb = T(1);
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
      ajv[j] = -mco[j] * rdv[j];
      alf = ajv[j] * alf;
    }
#pragma unroll
    for (int j = NPL - 1; j >= 0; --j) alb = -cpb[j] * alb;
    scan_muls_fwd(alf, mf, lane);
    scan_muls_bwd(alb, mb, lane);
  }
  // kord 4: thicknesses of layers u0-2 .. u0+NPL+1 (clamped into the column)
  T hw[NPL + 4];
#pragma unroll
  for (int i = 0; i < NPL + 4; ++i) hw[i] = KORD == 9 ? T(1) : S.dp[pk<T>(min(max(u0 - 2 + i, 0), km - 1))];
  constexpr int FP = fields_per_pass<T>();
  for (int f0 = 0; f0 < a.nfield; f0 += FP) {
    __syncthreads();  // every warp is done with the previous pass, whose slots are refilled now
#pragma unroll
    for (int h = 0; h < FP; ++h) issue(f0 + RING - FP + h);
    cp_async_wait<RING - FP>();
    __syncthreads();  // the pass's fields are in their slots
    // a pass past the last field repeats it and stores nothing
    const T* Q[FP];
    T* q2[FP];
    bool store[FP];
#pragma unroll
    for (int h = 0; h < FP; ++h) {
      const int f = min(f0 + h, a.nfield - 1);
      Q[h] = ring + ((f % RING) * RCOL + warp) * RP;
      q2[h] = a.q_out + qo + f * a.sQqo;
      store[h] = real && f0 + h < a.nfield;
    }
    // w[h][i]: mean of layer u0 - 2 + i (clamped into the column), the lane's
    // layers and two on either side; qv: the lane's own layers (0 past km)
    T qv[FP][NPL], st[FP][NPL], w[FP][NPL + 4];
#pragma unroll
    for (int h = 0; h < FP; ++h) {
#pragma unroll
      for (int i = 0; i < NPL + 4; ++i) w[h][i] = Q[h][pk<T>(min(max(u0 - 2 + i, 0), km - 1))];
#pragma unroll
      for (int j = 0; j < NPL; ++j) qv[h][j] = (u0 + j < km) ? w[h][j + 2] : T(0);
    }
    // -------------------------------------------- interface values a[0..km]
    // st[h][j]: the limited interface u0 + j (kord 9) or the PPM one (kord 4);
    // the interface after the lane's last layer is the next lane's first
    // (kord 9) or computed here as well (kord 4, st_end).
    T st_end[FP], dmv[FP][NPL];
    if (km == 1) {
#pragma unroll
      for (int h = 0; h < FP; ++h) {
        st_end[h] = qv[h][0];
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
          st[h][j] = qv[h][0];
          dmv[h][j] = T(0);
        }
      }
    } else if (KORD == 9) {
      T rhs[FP][NPL], be[FP];
#pragma unroll
      for (int h = 0; h < FP; ++h) {
        be[h] = T(0);
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
          // the two layers of row u (ia, ib) from the window: u-1 and u inside the
          // column, 0 and 1 at the top row, km-1 and km-2 at the bottom one
          const int u = u0 + j;
          const T qa = u == 0 ? w[h][j + 2] : w[h][j + 1];
          const T qb = u == 0 ? w[h][j + 3] : (u == km ? w[h][j] : w[h][j + 2]);
          rhs[h][j] = wa[j] * qa + wb[j] * qb + wc[j] * qsv;
          be[h] = ajv[j] * be[h] + rhs[h][j] * rdv[j];
          dmv[h][j] = T(0);
        }
      }
      T y[FP][NPL];
      {
        T yp[FP];
        affine_enter_fwd_m<T, FP>(mf, be, yp, lane);
#pragma unroll
        for (int h = 0; h < FP; ++h)
#pragma unroll
          for (int j = 0; j < NPL; ++j) {
            yp[h] = (rhs[h][j] - mco[j] * yp[h]) * rdv[j];
            y[h][j] = yp[h];
          }
      }
#pragma unroll
      for (int h = 0; h < FP; ++h) {
        be[h] = T(0);
#pragma unroll
        for (int j = NPL - 1; j >= 0; --j) be[h] = -cpb[j] * be[h] + y[h][j];
      }
      T av[FP];
      affine_enter_bwd_m<T, FP>(mb, be, av, lane);
#pragma unroll
      for (int h = 0; h < FP; ++h) {
#pragma unroll
        for (int j = NPL - 1; j >= 0; --j) {
          av[h] = y[h][j] - cpb[j] * av[h];
          st[h][j] = k9_interface(av[h], min(u0 + j, km), km, a.iv, floor_v, w[h][j], w[h][j + 1], w[h][j + 2],
                                  w[h][j + 3]);
        }
        st_end[h] = __shfl_down_sync(0xffffffffu, st[h][0], 1);
      }
    } else {
#pragma unroll
      for (int h = 0; h < FP; ++h) {
        // slopes of layers u0-1 .. u0+NPL, then interfaces u0 .. u0+NPL
        T dmw[NPL + 2];
#pragma unroll
        for (int i = 0; i < NPL + 2; ++i) {
          const int k = u0 - 1 + i;
          const T m = ppm_slope(w[h][i], w[h][i + 1], w[h][i + 2], hw[i], hw[i + 1], hw[i + 2]);
          dmw[i] = (k >= 1 && k <= km - 2) ? m : T(0);
        }
        const T* Qh = Q[h];
        auto qf = [Qh, km](int k) -> T { return Qh[pk<T>(min(max(k, 0), km - 1))]; };
        auto hf = [&S, km](int k) -> T { return S.dp[pk<T>(min(max(k, 0), km - 1))]; };
        T ai[NPL + 1];
#pragma unroll
        for (int j = 0; j <= NPL; ++j) {
          const int u = min(u0 + j, km);
          if (km > 2 && u >= 2 && u <= km - 2)
            ai[j] = ppm_interface_inner(w[h][j + 1], w[h][j + 2], dmw[j], dmw[j + 1], hw[j], hw[j + 1], hw[j + 2],
                                        hw[j + 3]);
          else
            ai[j] = ppm_interface<T>(u, km, a.iv, qsv, dmw[j], dmw[j + 1], qf, hf);
        }
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
          st[h][j] = ai[j];
          dmv[h][j] = dmw[j + 1];
        }
        st_end[h] = ai[NPL];
      }
    }
    // ------------------------------------------ sub-grid parabolas of layers
    // every layer takes both the interior constraint and CW84 and keeps the
    // one its position calls for (the two layers at each end of the column:
    // CW84), uniform across the warp, then the floor
#pragma unroll
    for (int h = 0; h < FP; ++h) {
#pragma unroll
      for (int j = 0; j < NPL; ++j) {
        const int u = u0 + j;
        const T qk = qv[h][j];
        T bl = st[h][j] - qk, br = (j + 1 < NPL ? st[h][j + 1] : st_end[h]) - qk;
        T ble = bl, bre = br;
        cw84_sel(ble, bre);
        interior_constraint<T, KORD>(w[h][j], w[h][j + 1], qk, w[h][j + 3], w[h][j + 4], dmv[h][j], bl, br);
        const bool end = u < 2 || u > km - 3;
        bl = end ? ble : bl;
        br = end ? bre : br;
        if (a.iv >= 0) positivity(qk, floor_v, bl, br);
        if (u < km) {
          S.pl[h][pk<T>(u)] = qk + bl;
          S.pr[h][pk<T>(u)] = qk + br;
          S.p6[h][pk<T>(u)] = T(-3) * (bl + br);
        }
      }
    }
    if (Single<T>::value) {
      // FP32 fields: cumulative source mass in float-float at every source
      // interface (layer masses q*dp are exact as float-float products), so a
      // target layer's mass is a difference of two cumulative values and the
      // column mass telescopes; only the final division rounds per value.
      FF m[FP][NPL], ex[FP];
#pragma unroll
      for (int h = 0; h < FP; ++h) {
        ex[h] = FF{0.f, 0.f};
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
          m[h][j] = (u0 + j < km) ? ff_prod((float)qv[h][j], (float)S.dp[pk<T>(u0 + j)]) : FF{0.f, 0.f};
          ex[h] = ff_add(ex[h], m[h][j]);
        }
      }
      // inclusive scan of the lane totals, then shifted by one lane
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        FF p[FP];
#pragma unroll
        for (int h = 0; h < FP; ++h)
          p[h] = FF{__shfl_up_sync(0xffffffffu, ex[h].hi, o), __shfl_up_sync(0xffffffffu, ex[h].lo, o)};
#pragma unroll
        for (int h = 0; h < FP; ++h)
          if (lane >= o) ex[h] = ff_add(p[h], ex[h]);
      }
#pragma unroll
      for (int h = 0; h < FP; ++h) {
        FF run{__shfl_up_sync(0xffffffffu, ex[h].hi, 1), __shfl_up_sync(0xffffffffu, ex[h].lo, 1)};
        if (lane == 0) run = FF{0.f, 0.f};
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
          if (u0 + j <= km) {
            S.mh[h][pk<float>(u0 + j)] = run.hi;
            S.ml[h][pk<float>(u0 + j)] = run.lo;
          }
          run = ff_add(run, m[h][j]);
        }
      }
    }
    __syncwarp();
    // ------------------------------------------------------- integration
#pragma unroll
    for (int h = 0; h < FP; ++h) {
      if (Single<T>::value) {
        // cumulative mass at this lane's target interfaces; the last one is the
        // next lane's first (32 NPL > kn, so lane 31's last is never used)
        FF cm[NPL + 1];
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
          const int L = Ls[j];
          const float X = (float)Xs[j];
          const int il = pk<float>(L), iu = pk<float>(L + 1);
          FF c{S.mh[h][il], S.ml[h][il]};
          if (X >= 1.f) {
            c = FF{S.mh[h][iu], S.ml[h][iu]};
          } else if (X > 0.f) {
            const int it = pk<T>(L);
            const float part =
                (float)S.dp[it] * X * (float)pmean(S.pl[h][it], S.pr[h][it], S.p6[h][it], T(0), T(X));
            c = ff_add(c, FF{part, 0.f});
          }
          cm[j] = c;
        }
        cm[NPL] = FF{__shfl_down_sync(0xffffffffu, cm[0].hi, 1), __shfl_down_sync(0xffffffffu, cm[0].lo, 1)};
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
          const int t = u0 + j;
          const FF mass = ff_add(cm[j + 1], ff_neg(cm[j]));
          // the quotient mass / dp, not mass times the rounded reciprocal (that rounding is shared by every
          // tracer of the layer and biased the global mass, +5e-10 per step at C384 L127 x20): the
          // reciprocal's product corrected by one Newton step on the exact residual (fma), which gives the
          // rounded quotient but for rare ties, unbiased
          const float mm = mass.hi + mass.lo, d = (float)dpk[j], r = (float)rdpk[j];
          const float q0 = mm * r;
          const float qq = fmaf(fmaf(-q0, d, mm), r, q0);
          if (store[h] && t < kn) q2[h][(long long)t * a.sQk] = T(qq);
        }
      } else {
#pragma unroll
        for (int j = 0; j < NPL; ++j) {
          const int t = u0 + j;
          const int Lt = Ls[j], Lb = Ls[j + 1];
          const T Xt = Xs[j], Xb = Xs[j + 1];
          const bool inside = (Lb == Lt) || (Lb == Lt + 1 && Xb == T(0));
          const int it = pk<T>(Lt), ib_ = pk<T>(Lb);
          const T qt = Q[h][it], dpt = S.dp[it];
          const T pm1 = pmean(S.pl[h][it], S.pr[h][it], S.p6[h][it], Xt, (inside && Lb == Lt) ? Xb : T(1));
          const T vin = (Xt == T(0) && (Lb == Lt + 1 || Xb == T(1))) ? qt : pm1;
          T mass = Xt == T(0) ? qt * dpt : (dpt * (T(1) - Xt)) * pm1;
          for (int mm = Lt + 1; mm < Lb; ++mm) mass = mass + Q[h][pk<T>(mm)] * S.dp[pk<T>(mm)];
          const T qb_ = Q[h][ib_], dpb = S.dp[ib_];
          const T pm2 = pmean(S.pl[h][ib_], S.pr[h][ib_], S.p6[h][ib_], T(0), Xb);
          const T bot = Xb >= T(1) ? qb_ * (dpb * Xb) : (Xb > T(0) ? (dpb * Xb) * pm2 : T(0));
          mass = mass + bot;
          const T out = inside ? vin : mass * rdpk[j];
          if (store[h] && t < kn) q2[h][(long long)t * a.sQk] = out;
        }
      }
    }
  }
}

template <typename T, int KORD, int NPL>
static cudaError_t set_remap_attr() {
  return cudaFuncSetAttribute(k_remap_warp<T, KORD, NPL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)remap_warp_smem<T, NPL>());
}

// Raise the dynamic shared-memory limit of the remap kernels once per process
// (before any stream capture).
int prepare_remap_kernels() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    cudaError_t es[] = {set_remap_attr<float, 9, 4>(),  set_remap_attr<float, 9, 5>(),  set_remap_attr<float, 4, 4>(),
                        set_remap_attr<float, 4, 5>(),  set_remap_attr<double, 9, 4>(), set_remap_attr<double, 9, 5>(),
                        set_remap_attr<double, 4, 4>(), set_remap_attr<double, 4, 5>()};
    for (cudaError_t e : es)
      if (e != cudaSuccess && err == cudaSuccess) err = e;
  });
  return err == cudaSuccess ? 0 : cuda_error(err, "cudaFuncSetAttribute(k_remap_warp)");
}

template <typename T, int KORD, int NPL>
static cudaError_t launch_warp_npl(const RemapArgs<T>& a, cudaStream_t s) {
  constexpr size_t smem = remap_warp_smem<T, NPL>();
  const unsigned nb = (unsigned)((a.ncol + RCOL - 1) / RCOL);
  k_remap_warp<T, KORD, NPL><<<nb, 32 * RCOL, smem, s>>>(a);
  return cudaGetLastError();
}

template <typename T, int KORD>
static cudaError_t launch_warp_form(const RemapArgs<T>& a, cudaStream_t s) {
  if (std::max(a.km, a.kn) < 32 * 4) return launch_warp_npl<T, KORD, 4>(a, s);
  return launch_warp_npl<T, KORD, 5>(a, s);
}

template <typename T>
int launch_remap(const RemapArgs<T>& a, int kord, cudaStream_t s) {
  if (a.km < 1 || a.km > KMAX || a.kn < 1 || a.kn > KMAX)
    return set_error(FV3G_E_ARG, "remap supports 1..%d layers (km=%d, kn=%d)", KMAX, a.km, a.kn);
  if (kord != 9 && kord != 4) return set_error(FV3G_E_UNSUPPORTED, "kord %d not implemented (4 and 9 are)", kord);
  if (a.ncol > (1LL << 30)) return set_error(FV3G_E_ARG, "remap supports at most 2^30 columns per call");
  {
    const int prc = prepare_remap_kernels();
    if (prc) return prc;
  }
  if constexpr (std::is_same<T, float>::value) {
    if (a.form == 1 && remap_col_applies(a, kord)) {
      FV3G_CUDA(launch_remap_col(a, s));
      return 0;
    }
  }
  if (a.scratch != nullptr) {
    const unsigned nb = (unsigned)((a.ncol + 127) / 128);
    if (kord == 9) k_remap_scratch<T, 9><<<nb, 128, 0, s>>>(a);
    else k_remap_scratch<T, 4><<<nb, 128, 0, s>>>(a);
  } else {
    const cudaError_t e = kord == 9 ? launch_warp_form<T, 9>(a, s) : launch_warp_form<T, 4>(a, s);
    FV3G_CUDA(e);
  }
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

// Interface pressures of the columns of a field kind (0: cells; 1: y faces
// (i, j) between cells (i, j-1) and (i, j), the u winds; 2: x faces between
// (i-1, j) and (i, j), the v winds) from the Lagrangian thickness planes dp
// ([tile][level], halo cells filled for the faces): pe1 = ptop + the running
// sum of dp (the mean of the two columns beside a face), pe2 = ak + bk ps with
// the same ps; with log_p both in ln p.  [k][col] layout, col = (t nj + cj) ni
// + ci over the kind's columns ci < ni, cj < nj.
template <typename T>
__global__ void k_field_pressures(const T* dp, long long sFt, long long sFk, PlaneGeom pg, int nt, int km, int ni,
                                  int nj, int kind, int log_p, const double* ak, const double* bk, double* pe1,
                                  double* pe2) {
  const long long nc = (long long)nt * ni * nj;
  const long long col = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= nc) return;
  const int ci = (int)(col % ni);
  const long long rest = col / ni;
  const int cj = (int)(rest % nj), t = (int)(rest / nj);
  const int i = 1 + ci, j = 1 + cj;
  const T* da = dp + t * sFt + pg.at(i, j);
  const T* db = dp + t * sFt + (kind == 1 ? pg.at(i, j - 1) : kind == 2 ? pg.at(i - 1, j) : pg.at(i, j));
  double pa = ak[0], pb = ak[0];
  pe1[col] = log_p ? log(pa) : pa;
  for (int k = 0; k < km; ++k) {
    pa += (double)da[(long long)k * sFk];
    pb += (double)db[(long long)k * sFk];
    const double p = kind == 0 ? pa : 0.5 * (pa + pb);
    pe1[(long long)(k + 1) * nc + col] = log_p ? log(p) : p;
  }
  const double ps = kind == 0 ? pa : 0.5 * (pa + pb);
  for (int k = 0; k <= km; ++k) {
    const double p = ak[k] + bk[k] * ps;
    pe2[(long long)k * nc + col] = log_p ? log(p) : p;
  }
}

template <typename T>
int launch_field_pressures(const T* dp, long long sFt, long long sFk, PlaneGeom pg, int nt, int km, int ni, int nj,
                           int kind, int log_p, const double* ak, const double* bk, double* pe1, double* pe2,
                           cudaStream_t s) {
  const long long nc = (long long)nt * ni * nj;
  k_field_pressures<T><<<(unsigned)((nc + 127) / 128), 128, 0, s>>>(dp, sFt, sFk, pg, nt, km, ni, nj, kind, log_p, ak,
                                                                   bk, pe1, pe2);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}
template int launch_field_pressures<float>(const float*, long long, long long, PlaneGeom, int, int, int, int, int,
                                           int, const double*, const double*, double*, double*, cudaStream_t);
template int launch_field_pressures<double>(const double*, long long, long long, PlaneGeom, int, int, int, int, int,
                                            int, const double*, const double*, double*, double*, cudaStream_t);

// Tangent-linear remap: the thread-per-column kernel on value/tangent pairs
// (scratch supplied by the caller, remap_scratch_bytes(ncol, 16)).
int launch_remap_tl(const RemapArgs<Dual<double>>& a, int kord, cudaStream_t s) {
  if (a.km < 1 || a.km > KMAX || a.kn < 1 || a.kn > KMAX)
    return set_error(FV3G_E_ARG, "remap supports 1..%d layers (km=%d, kn=%d)", KMAX, a.km, a.kn);
  if (a.scratch == nullptr || a.sched == nullptr) return set_error(FV3G_E_ARG, "tangent-linear remap needs scratch");
  const unsigned nb = (unsigned)((a.ncol + 127) / 128);
  if (kord == 9) k_remap_scratch<Dual<double>, 9><<<nb, 128, 0, s>>>(a);
  else if (kord == 4) k_remap_scratch<Dual<double>, 4><<<nb, 128, 0, s>>>(a);
  else return set_error(FV3G_E_UNSUPPORTED, "kord %d not implemented (4 and 9 are)", kord);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

size_t remap_scratch_bytes(long long ncol, size_t elem_bytes) {
  return (size_t)ncol * (KMAX + 1) * (6 * elem_bytes + 1) + 256;
}

template int launch_remap<float>(const RemapArgs<float>&, int, cudaStream_t);
template int launch_remap<double>(const RemapArgs<double>&, int, cudaStream_t);

}  // namespace fv3g
