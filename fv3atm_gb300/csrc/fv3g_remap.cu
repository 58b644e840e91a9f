// fv3g_remap.cu -- Lagrangian-to-Eulerian column remap (map_scalar / map1_ppm
// with the cs_profile reconstruction of fv_mapz.F90, GFDL_atmos_cubed_sphere,
// absent submodule .gitmodules:1-4).
//
// One thread per column; consecutive threads own consecutive i, so every
// level of every field is read and written as a coalesced row.  Per column,
// once for all fields:
//   * the Lagrangian interface pressures pe1 (FP64 running sum of delp) and
//     the target interfaces pe2 = ak + bk*ps (FP64);
//   * the overlap schedule: for every target interface, the source layer that
//     contains it and its fractional position (FP64 differences, stored in T);
//   * the LU factors of the tridiagonal interface system (they depend on the
//     layer thicknesses only).
// Per field: forward/back substitution for the interface values, the kord
// constraints, and the integration of the sub-grid parabolas over the
// overlaps.  Column-constant arrays and the interface values live in a
// scratch buffer laid out [level][column] (coalesced, L2-resident).
#include <cfloat>

#include "fv3g_internal.cuh"
#include "fv3g_remap.cuh"

namespace fv3g {

template <typename T> __device__ __forceinline__ T clampv(T a, T x0, T x1) { return clamp2(a, x0, x1); }

// mean of the parabola (aL, aR, a6) over the fractional interval [x1, x2]
template <typename T> __device__ __forceinline__ T pmean(T l, T r, T s6, T x1, T x2) {
  return l + T(0.5) * (x1 + x2) * ((r - l) + s6) - s6 * ((x2 * x2 + x1 * x2 + x1 * x1) * T(1.0 / 3.0));
}

template <typename T>
struct Profile {  // sub-grid parabola of one source layer
  T q, l, r, s6;
};

template <typename T, int KORD>
__device__ __forceinline__ Profile<T> layer_profile(T q, T aL, T aR, int iv, T floor_v) {
  if (KORD != 9 && iv >= 0) {
    aL = tmax(aL, floor_v);
    aR = tmax(aR, floor_v);
  }
  T bl = aL - q, br = aR - q;
  cw84(bl, br);
  if (KORD != 9 && iv >= 0 && (q + bl < floor_v || q + br < floor_v)) {  // keep the floor: flatten
    bl = T(0);
    br = T(0);
  }
  return Profile<T>{q, q + bl, q + br, T(-3) * (bl + br)};
}

template <typename T, int KORD>
__global__ void __launch_bounds__(128) k_remap(const RemapArgs<T> a) {
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
    for (int k = 0; k < km; ++k) s += (double)a.dp[fo + k * a.sFk];
    ps = s;
  }
  auto pe2_at = [&](int k) -> double {
    if (a.pe2 != nullptr) return a.pe2[(long long)k * nc + col];
    return a.ak[k] + a.bk[k] * ps;
  };
  auto dp_src = [&](int k) -> double { return (double)a.dp[fo + k * a.sFk]; };
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
      SC(s_x, k2) = (sizeof(T) == 8) ? T((p - lo) / (hi - lo)) : T(float(p - lo) / float(hi - lo));
    }
  }
  // LU factors of the interface system (rows 0..km), see the oracle restatement
  if (km > 1) {
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
    // -------------------------------------------- interface values a[0..km]
    if (km == 1) {
      SC(s_a, 0) = q1[0];
      SC(s_a, 1) = q1[0];
    } else {
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
      T av = (rhs - SC(s_cp, km) * ap) * SC(s_rd, km);
      SC(s_a, km) = (KORD == 9 && a.iv != -2) ? clampv(av, q1[(km - 2) * a.sQk], q1[(km - 1) * a.sQk]) : av;
      for (int k = km - 1; k >= 0; --k) {
        av = SC(s_a, k) - SC(s_cp, k) * av;
        T st = av;
        if (KORD == 9) {
          if (k == 0) st = clampv(av, q1[0], q1[a.sQk]);
          else st = clampv(av, q1[(k - 1) * a.sQk], q1[k * a.sQk]);
        }
        SC(s_a, k) = st;
      }
    }
    // ------------------------------------------------------- integration
    int kc = -1;  // layer whose profile is cached
    Profile<T> P{};
    auto prof = [&](int k) -> const Profile<T>& {
      if (k != kc) {
        P = layer_profile<T, KORD>(q1[k * a.sQk], SC(s_a, k), SC(s_a, k + 1), a.iv, floor_v);
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
        // target thickness from the FP64 interface pressures
        const T dpk = T(pe2_at(k2 + 1) - pe2_at(k2));
        out = mass / dpk;
      }
      q2[k2 * a.sQk] = out;
      Lt = Lb;
      Xt = Xb;
    }
  }
#undef SC
}

template <typename T>
int launch_remap(const RemapArgs<T>& a, int kord, cudaStream_t s) {
  if (a.km < 1 || a.km > KMAX || a.kn < 1 || a.kn > KMAX)
    return set_error(FV3G_E_ARG, "remap supports 1..%d layers (km=%d, kn=%d)", KMAX, a.km, a.kn);
  const unsigned nb = (unsigned)((a.ncol + 127) / 128);
  if (kord == 9) k_remap<T, 9><<<nb, 128, 0, s>>>(a);
  else if (kord == 4) k_remap<T, 4><<<nb, 128, 0, s>>>(a);
  else return set_error(FV3G_E_UNSUPPORTED, "kord %d not implemented (4 and 9 are)", kord);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

size_t remap_scratch_bytes(long long ncol, bool fp64) {
  return (size_t)ncol * (KMAX + 1) * (6 * (fp64 ? 8 : 4) + 1) + 256;
}

template int launch_remap<float>(const RemapArgs<float>&, int, cudaStream_t);
template int launch_remap<double>(const RemapArgs<double>&, int, cudaStream_t);

}  // namespace fv3g
