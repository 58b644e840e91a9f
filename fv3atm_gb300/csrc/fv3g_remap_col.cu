// fv3g_remap_col.cu -- FP32 kord-9 column remap of the batched state, one
// thread per column (map_scalar with the cs_profile reconstruction of
// fv_mapz.F90, GFDL_atmos_cubed_sphere, absent submodule .gitmodules:1-4).
//
// Consecutive threads own consecutive i of a row of columns, so every level of
// every field moves as a coalesced row, and each thread runs its column's
// recurrences in level order: no lane-to-lane scans, and every branch on the
// level (the end rows of the interface system, the CW84 end layers, the top
// interface) is uniform across the warp.  FP fields advance together in one
// pass, sharing the column's pivots and overlap schedule.
//
// Pass A (top-down) runs the forward elimination of the C1 interface system
// (pivots from the layer thicknesses; the substitution of each field) and the
// float-float column pressure ps, and keeps only a checkpoint in shared
// memory: the elimination state entering the first row of every chunk of
// RC_CHUNK rows.  Pass B walks the column bottom-up one chunk at a time: the
// chunk's elimination is recomputed from its checkpoint into registers; the
// back substitution gives each interface value (the raw values carry the
// recurrence, each interface is limited on its own); each layer takes its
// constraint (CW84 on the two end layers at each end, the extremum-aware
// Huynh constraint inside) and the positivity scaling; the float-float mass
// below each source interface accumulates; and each target interface that
// falls inside the layer gets its mass below (the layer's part beneath it plus
// everything deeper).  A target layer's mean is the difference of the masses
// below its two interfaces over its thickness, so the column mass telescopes.
// Source interfaces (ps minus the running thickness) and target interfaces
// (ak + bk ps) are float-float (~48-bit significands): the overlap schedule
// needs no FP64 instruction.
//
// The schemes are those of fv3g_profile.cuh (shared with the warp-per-column
// kernel and the oracle), restated here with the FP32 min / max / abs
// instructions.
#include "fv3g_ff.cuh"
#include "fv3g_internal.cuh"
#include "fv3g_remap.cuh"

namespace fv3g {
namespace {

constexpr int RC_CHUNK = 8;     // rows per recomputed chunk
constexpr int RC_THREADS = 128;  // columns per CTA
constexpr int RC_FIELDS = 2;    // fields per pass

__device__ __forceinline__ bool opp_f(float x, float y) { return (x > 0.f && y < 0.f) || (x < 0.f && y > 0.f); }
__device__ __forceinline__ bool same_f(float x, float y) { return (x > 0.f && y > 0.f) || (x < 0.f && y < 0.f); }
__device__ __forceinline__ float clamp_f(float a, float x0, float x1) {
  return fminf(fmaxf(a, fminf(x0, x1)), fmaxf(x0, x1));
}

// float-float plus a float, and the order of two normalised float-floats
__device__ __forceinline__ FF ff_addf(FF a, float b) {
  const float s = a.hi + b;
  const float bb = s - a.hi;
  float e = (a.hi - (s - bb)) + (b - bb);
  e += a.lo;
  const float h = s + e;
  return FF{h, e - (h - s)};
}
__device__ __forceinline__ bool ff_ge(FF a, FF b) { return a.hi > b.hi || (a.hi == b.hi && a.lo >= b.lo); }
// a * b of two float-floats (the lo * lo term dropped)
__device__ __forceinline__ FF ff_mul(FF a, FF b) {
  const float p = a.hi * b.hi;
  float e = fmaf(a.hi, b.hi, -p);
  e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
  const float h = p + e;
  return FF{h, e - (h - p)};
}

// kord 9, interfaces 1..km-1: the limited value of the raw interface a
// between layer means qa (above) and qb (below), given the jumps dl, dc, dr
// across the interfaces above, at and below it
__device__ __forceinline__ float k9_mid(float a, int iv, float floor_v, float dl, float dr, float qa, float qb) {
  const float lo = fminf(qa, qb), hi = fmaxf(qa, qb);
  const bool mono = same_f(dl, dr);
  const bool near_max = !mono && dl > 0.f;
  const float below = fminf(a, hi);
  return mono ? fminf(fmaxf(a, lo), hi) : (near_max ? fmaxf(a, lo) : (iv >= 0 ? fmaxf(below, floor_v) : below));
}

// CW84 eq. 1.10 in perturbation form (the two layers at each end)
__device__ __forceinline__ void cw84_f(float& bl, float& br) {
  const bool flat = !opp_f(bl, br);
  const float d = br - bl;
  const float t = 3.f * d * (bl + br);
  const float d2 = d * d;
  const bool lo = -t > d2, hi = !lo && t > d2;
  const float nbl = lo ? -2.f * br : bl, nbr = hi ? -2.f * bl : br;
  bl = flat ? 0.f : nbl;
  br = flat ? 0.f : nbr;
}

// interior layer: flattened beside another extremum, else Huynh's second
// constraint when the parabola has an interior extremum
__device__ __forceinline__ void k9_layer(float qm2, float qm1, float qk, float qp1, float qp2, float& bl, float& br) {
  const float Dm = qm1 - qm2, D0 = qk - qm1, D1 = qp1 - qk, D2 = qp2 - qp1;
  const bool flat = opp_f(D0, D1) && (opp_f(Dm, D0) || opp_f(D1, D2));
  const bool nonmono = 3.f * fabsf(bl + br) > fabsf(br - bl);
  const float pr = 2.f * D0, lr = fmaf(-1.5f, Dm, pr);
  const float pl = -2.f * D1, ll = fmaf(1.5f, D2, pl);
  const float brc = fminf(fmaxf(br, tmin3(0.f, pr, lr)), tmax3(0.f, pr, lr));
  const float blc = fminf(fmaxf(bl, tmin3(0.f, pl, ll)), tmax3(0.f, pl, ll));
  bl = flat ? 0.f : (nonmono ? blc : bl);
  br = flat ? 0.f : (nonmono ? brc : br);
}

// Zhang & Shu (2010) scaling for iv >= 0 (see fv3g_profile.cuh)
__device__ __forceinline__ void positivity_f(float qk, float floor_v, float& bl, float& br) {
  const float s6 = -3.f * (bl + br), da = br - bl;
  const bool inner = -s6 > fabsf(da);
  const bool low = (qk + bl < floor_v) || (qk + br < floor_v) ||
                   (inner && fmaf(3.f * da, da, fmaf(s6, s6, 12.f * s6 * (qk - floor_v))) > 0.f);
  if (low) {
    float pmin = fminf(qk + bl, qk + br);
    if (inner) pmin = fminf(pmin, qk + __fdividef(s6, 12.f) + __fdividef(da * da, 4.f * s6));
    float lam = qk > floor_v ? __fdividef(qk - floor_v, qk - pmin) : 0.f;
    lam = lam * (1.f - 1.f / (1 << 21));
    bl = lam * bl;
    br = lam * br;
  }
}

// mean of the parabola (l, r, s6) of a layer over its fraction [x, 1]
__device__ __forceinline__ float pmean_to_bottom(float l, float r, float s6, float x) {
  return fmaf(-s6, (fmaf(x, x, x) + 1.f) * (1.f / 3.f), fmaf(0.5f * (x + 1.f), (r - l) + s6, l));
}

struct ColSched {
  const float *akh, *akl, *bkh, *bkl;  // ak, bk as float-float (shared memory)
  FF ps;
  __device__ __forceinline__ FF pe2(int t) const {
    return ff_add(FF{akh[t], akl[t]}, ff_mul(FF{bkh[t], bkl[t]}, ps));
  }
};

template <int FP>
struct PassB {
  float ar[FP], al1[FP];  // raw and limited value of interface k+1
  FF D[FP];               // mass below source interface k+1
  FF Dn[FP];              // mass below target interface t+1
  FF p1;                  // pe1 at interface k+1
  FF p2, p2n;             // pe2 at target interfaces t and t+1
  int t;                  // next target interface (descending)
};

// One chunk of pass B: rows s .. s+n-1 (n = RC_CHUNK unless PARTIAL), the
// elimination entering row s given by yin / cin (s > 0) or recomputed from
// row 0 (s == 0).
template <int FP, bool PARTIAL>
__device__ __forceinline__ void chunk_b(const RemapArgs<float>& a, const float* __restrict__ dpc,
                                        const float* const (&Q)[FP], float* const (&Q2)[FP], const bool (&st)[FP],
                                        bool write_dp, long long fo, int s, int n, const float (&yin)[FP], float cin,
                                        float floor_v, const ColSched& sc, PassB<FP>& b) {
  constexpr int C = RC_CHUNK;
  const int km = a.km, kn = a.kn, iv = a.iv;
  const long long sk = a.sFk, sq = a.sQk;
  // rows s-1 .. s+C-1 of dp, s-2 .. s+C+1 of every field (clamped into the column)
  float dv[C + 1], qv[FP][C + 4];
#pragma unroll
  for (int i = 0; i <= C; ++i) dv[i] = dpc[(long long)min(max(s - 1 + i, 0), km - 1) * sk];
#pragma unroll
  for (int h = 0; h < FP; ++h)
#pragma unroll
    for (int i = 0; i < C + 4; ++i) qv[h][i] = Q[h][(long long)min(max(s - 2 + i, 0), km - 1) * sq];
  // ---- the chunk's forward elimination
  float yv[FP][C], cpv[C];
  {
    float yy[FP], cc = cin;
#pragma unroll
    for (int h = 0; h < FP; ++h) yy[h] = yin[h];
#pragma unroll
    for (int i = 0; i < C; ++i) {
      if (PARTIAL && i >= n) break;
      if (PARTIAL && i == 0) {  // row 0 (the chunk at the top of the column)
        const float g = __fdividef(dv[2], dv[1]);
        const float rg = __fdividef(1.f, g + 1.f);
        const float wa = fmaf(2.f, g, 3.f) * g * rg;
        const float rd = __fdividef(1.f, g);
        cc = (g + 1.f) * rd;
#pragma unroll
        for (int h = 0; h < FP; ++h) yy[h] = fmaf(wa, qv[h][2], rg * qv[h][3]) * rd;
      } else {
        const float d = __fdividef(dv[i], dv[i + 1]);
        const float rd = __fdividef(1.f, fmaf(2.f, d, 2.f) - cc);
        cc = d * rd;
#pragma unroll
        for (int h = 0; h < FP; ++h) yy[h] = fmaf(3.f, fmaf(d, qv[h][i + 2], qv[h][i + 1]), -yy[h]) * rd;
      }
      cpv[i] = cc;
#pragma unroll
      for (int h = 0; h < FP; ++h) yv[h][i] = yy[h];
    }
  }
  // ---- back substitution, layers and targets, bottom-up
#pragma unroll
  for (int i = C - 1; i >= 0; --i) {
    if (PARTIAL && i >= n) continue;
    const int k = s + i;
    float pl[FP], pr[FP], p6[FP];
    FF Dtop[FP];
    const float dpk = dv[i + 1];
#pragma unroll
    for (int h = 0; h < FP; ++h) {
      const float qm2 = qv[h][i], qm1 = qv[h][i + 1], q0 = qv[h][i + 2], qp1 = qv[h][i + 3], qp2 = qv[h][i + 4];
      b.ar[h] = fmaf(-cpv[i], b.ar[h], yv[h][i]);
      float al;
      if (k == 0) {
        al = clamp_f(b.ar[h], q0, qp1);
      } else {
        const float dc = q0 - qm1;
        const float dl = k > 1 ? qm1 - qm2 : dc;
        const float dr = k < km - 1 ? qp1 - q0 : dc;
        al = k9_mid(b.ar[h], iv, floor_v, dl, dr, qm1, q0);
      }
      float bl = al - q0, br = b.al1[h] - q0;
      if (k < 2 || k > km - 3) cw84_f(bl, br);
      else k9_layer(qm2, qm1, q0, qp1, qp2, bl, br);
      if (iv >= 0) positivity_f(q0, floor_v, bl, br);
      pl[h] = q0 + bl;
      pr[h] = q0 + br;
      p6[h] = -3.f * (bl + br);
      b.al1[h] = al;
      Dtop[h] = ff_add(b.D[h], ff_prod(q0, dpk));
    }
    const FF p1k = ff_addf(b.p1, -dpk);  // pe1 at interface k
    // target interfaces inside layer k (every one left at the top layer)
    while (b.t >= 0 && (k == 0 || ff_ge(b.p2, p1k))) {
      const FF dx = ff_add(b.p2, ff_neg(p1k));
      const float X = __fdividef(dx.hi + dx.lo, dpk);
      FF Dt[FP];
#pragma unroll
      for (int h = 0; h < FP; ++h) {
        const float part = (dpk * (1.f - X)) * pmean_to_bottom(pl[h], pr[h], p6[h], X);
        Dt[h] = X <= 0.f ? Dtop[h] : (X >= 1.f ? b.D[h] : ff_addf(b.D[h], part));
      }
      if (b.t < kn) {  // target layer t: between interfaces t and t+1
        const FF dd = ff_add(b.p2n, ff_neg(b.p2));
        const float dpt = dd.hi + dd.lo;
        const float r = 1.f / dpt;
        if (write_dp) a.dp_out[fo + (long long)b.t * sk] = dpt;
#pragma unroll
        for (int h = 0; h < FP; ++h) {
          const FF m = ff_add(Dt[h], ff_neg(b.Dn[h]));
          const float mm = m.hi + m.lo;
          // the quotient mm / dpt from the reciprocal, corrected by one step on the exact residual
          const float q0 = mm * r;
          const float qq = fmaf(fmaf(-q0, dpt, mm), r, q0);
          if (st[h]) Q2[h][(long long)b.t * sq] = qq;
        }
      }
#pragma unroll
      for (int h = 0; h < FP; ++h) b.Dn[h] = Dt[h];
      b.p2n = b.p2;
      --b.t;
      if (b.t >= 0) b.p2 = sc.pe2(b.t);
    }
#pragma unroll
    for (int h = 0; h < FP; ++h) b.D[h] = Dtop[h];
    b.p1 = p1k;
  }
}

template <int FP>
__global__ void __launch_bounds__(RC_THREADS, 4) k_remap_col(const RemapArgs<float> a) {
  constexpr int C = RC_CHUNK;
  extern __shared__ __align__(16) float rc_sm[];
  const int tid = threadIdx.x;
  const int km = a.km, kn = a.kn;
  const int nch = (km + C - 1) / C;
  const int r0 = km - C * (nch - 1);  // rows of the top chunk (1..C); the others hold C
  float* const ck = rc_sm;            // checkpoints [chunk][FP + 1][RC_THREADS]
  float* const akh = rc_sm + nch * (FP + 1) * RC_THREADS;
  float* const akl = akh + (kn + 1);
  float* const bkh = akl + (kn + 1);
  float* const bkl = bkh + (kn + 1);
  for (int i = tid; i <= kn; i += RC_THREADS) {
    const double ak = a.ak[i], bk = a.bk[i];
    const float ah = (float)ak, bh = (float)bk;
    akh[i] = ah;
    akl[i] = (float)(ak - (double)ah);
    bkh[i] = bh;
    bkl[i] = (float)(bk - (double)bh);
  }
  __syncthreads();
  const long long c0 = (long long)blockIdx.x * RC_THREADS + tid;
  const bool real = c0 < a.ncol;
  const long long col = real ? c0 : a.ncol - 1;
  long long fo, qo;
  {
    const long long ni = a.ni, nj = a.nj;
    const long long rest = col / ni, ci = col - rest * ni;
    const long long ct = rest / nj, cj = rest - ct * nj;
    const long long at = a.pg.at(a.i1 + (int)ci, a.j1 + (int)cj);
    fo = ct * a.sFt + at;
    qo = ct * a.sQt + at;
  }
  const float* __restrict__ dpc = a.dp + fo;
  const long long sk = a.sFk, sq = a.sQk;
  const float floor_v = a.iv == 1 ? (float)a.q_min : 0.f;
  auto ckp = [&](int c, int h) -> float& { return ck[(c * (FP + 1) + h) * RC_THREADS + tid]; };
  ColSched sc{akh, akl, bkh, bkl, FF{0.f, 0.f}};

  for (int f0 = 0; f0 < a.nfield; f0 += FP) {
    const float* Q[FP];
    float* Q2[FP];
    bool st[FP];
#pragma unroll
    for (int h = 0; h < FP; ++h) {
      const int f = min(f0 + h, a.nfield - 1);
      Q[h] = a.q_in + qo + f * a.sQq;
      Q2[h] = a.q_out + qo + f * a.sQqo;
      st[h] = real && f0 + h < a.nfield;
    }
    // -------------------------------------------------------- pass A
    float y[FP], qa[FP], qb[FP], cp, dpa, dpb;  // row k-1: y, q, cp, dp; qb, dpb: row k-2
    FF pe{akh[0], akl[0]};
    {
      const float d0 = dpc[0], d1 = dpc[sk];
      const float g = __fdividef(d1, d0);
      const float rg = __fdividef(1.f, g + 1.f);
      const float wa = fmaf(2.f, g, 3.f) * g * rg;
      const float rd = __fdividef(1.f, g);
      cp = (g + 1.f) * rd;
#pragma unroll
      for (int h = 0; h < FP; ++h) {
        qa[h] = Q[h][0];
        qb[h] = qa[h];
        y[h] = fmaf(wa, qa[h], rg * Q[h][sq]) * rd;
      }
      dpa = d0;
      dpb = d0;
      pe = ff_addf(pe, d0);
    }
    for (int c = 0; c < nch; ++c) {
      const int s = c == 0 ? 0 : r0 + (c - 1) * C, n = c == 0 ? r0 : C;
      if (c > 0) {
#pragma unroll
        for (int h = 0; h < FP; ++h) ckp(c, h) = y[h];
        ckp(c, FP) = cp;
      }
      float dv[C], qv[FP][C];
#pragma unroll
      for (int i = 0; i < C; ++i) {
        const long long k = min(s + i, km - 1);
        dv[i] = dpc[k * sk];
#pragma unroll
        for (int h = 0; h < FP; ++h) qv[h][i] = Q[h][k * sq];
      }
#pragma unroll
      for (int i = 0; i < C; ++i) {
        if (i >= n) break;
        if (s + i == 0) continue;  // row 0 above
        const float d = __fdividef(dpa, dv[i]);
        const float rd = __fdividef(1.f, fmaf(2.f, d, 2.f) - cp);
        cp = d * rd;
#pragma unroll
        for (int h = 0; h < FP; ++h) {
          y[h] = fmaf(3.f, fmaf(d, qv[h][i], qa[h]), -y[h]) * rd;
          qb[h] = qa[h];
          qa[h] = qv[h][i];
        }
        dpb = dpa;
        dpa = dv[i];
        pe = ff_addf(pe, dv[i]);
      }
    }
    // bottom row km: the one-sided C1 condition (iv != -2)
    sc.ps = pe;
    PassB<FP> b;
    {
      const float gb = __fdividef(dpb, dpa);
      const float lo = gb + 1.f;
      const float rd = __fdividef(1.f, fmaf(-lo, cp, gb));
      const float rg = __fdividef(1.f, gb + 1.f);
      const float wa = fmaf(2.f, gb, 3.f) * gb * rg;
#pragma unroll
      for (int h = 0; h < FP; ++h) {
        const float ykm = fmaf(-lo, y[h], fmaf(wa, qa[h], rg * qb[h])) * rd;
        b.ar[h] = ykm;
        b.al1[h] = clamp_f(ykm, qb[h], qa[h]);
        b.D[h] = FF{0.f, 0.f};
        b.Dn[h] = FF{0.f, 0.f};
      }
    }
    b.p1 = pe;
    b.t = kn;
    b.p2 = sc.pe2(kn);
    b.p2n = b.p2;
    // -------------------------------------------------------- pass B
    const bool write_dp = f0 == 0 && real && a.dp_out != nullptr;
    for (int c = nch - 1; c >= 1; --c) {
      float yin[FP];
#pragma unroll
      for (int h = 0; h < FP; ++h) yin[h] = ckp(c, h);
      chunk_b<FP, false>(a, dpc, Q, Q2, st, write_dp, fo, r0 + (c - 1) * C, C, yin, ckp(c, FP), floor_v, sc, b);
    }
    {
      float yin[FP];
#pragma unroll
      for (int h = 0; h < FP; ++h) yin[h] = 0.f;
      chunk_b<FP, true>(a, dpc, Q, Q2, st, write_dp, fo, 0, r0, yin, 0.f, floor_v, sc, b);
    }
  }
}

}  // namespace

size_t remap_col_smem(int km, int kn) {
  const int nch = (km + RC_CHUNK - 1) / RC_CHUNK;
  return (size_t)nch * (RC_FIELDS + 1) * RC_THREADS * sizeof(float) + 4 * (size_t)(kn + 1) * sizeof(float);
}

bool remap_col_applies(const RemapArgs<float>& a, int kord) {
  return kord == 9 && a.scratch == nullptr && a.pe1 == nullptr && a.pe2 == nullptr && a.dp2 == nullptr &&
         a.iv >= -1 && a.iv <= 1 && a.km >= 2 * RC_CHUNK && a.km <= KMAX && a.kn >= 1 && a.kn <= KMAX &&
         a.ak != nullptr && a.bk != nullptr;
}

cudaError_t launch_remap_col(const RemapArgs<float>& a, cudaStream_t s) {
  const size_t smem = remap_col_smem(a.km, a.kn);
  const unsigned nb = (unsigned)((a.ncol + RC_THREADS - 1) / RC_THREADS);
  k_remap_col<RC_FIELDS><<<nb, RC_THREADS, smem, s>>>(a);
  return cudaGetLastError();
}

}  // namespace fv3g
