// fv3g_substep.cuh -- fused fv_tp_2d + flux-form update (one tracer_2d substep).
//
// Restates, GB300-first, the body of the substep loop of tracer_2d
// (fv_tracer2d.F90) and fv_tp_2d / xppm / yppm / copy_corners (tp_core.F90) of
// GFDL_atmos_cubed_sphere (absent submodule, .gitmodules:1-4).
//
// One CTA owns a 26 x 26 block of output cells of one (tile, level) and a
// 32 x 32 window (3-cell halo) of every tracer.  Per-level fields (Courant
// numbers, area and mass fluxes, 1/ra_x, 1/ra_y, dp ratios) are staged once
// in shared memory and shared by the CTA's warps; each warp advances one
// tracer at a time through three on-chip stages:
//   S1  lane = window column: inner y-PPM on q (corner blocks filled for a y
//       sweep) -> inner y flux and the advective update q_i;
//   S2  lane = window row: inner x-PPM on q (corners re-filled for an x sweep)
//       -> q_j, and on the 26 interior rows the outer x-PPM on q_i, combined
//       into the final x flux and its divergence;
//   S3  lane = window column (interior ones): outer y-PPM on q_j, final y
//       flux, and the flux-form update q <- (q dp1 + div F * rarea) / dp2
//       written to HBM.  The inner y flux of S1 stays in the lane's registers.
// Each lane marches its line with a register pipeline (slope -> interface ->
// edge deviations -> flux), so intermediate fluxes never leave the SM and q
// is read once and written once per substep.  Halo cells are gathered from
// the neighbouring tiles of the cube (or read from the caller's halo), and
// the cube-corner blocks are filled by the rotation of copy_corners at load.
//
// This header holds the kernel templates; fv3g_substep_h{1,5,8}.cu instantiate
// them once per hord, so the three compile in parallel.
#pragma once

#include <cstdio>
#include <type_traits>

#include "fv3g_pair.cuh"
#include "fv3g_stencil.cuh"

namespace fv3g {

template <typename T>
struct SmemLevel {
  T cy[NF][WIN];  // inner/outer y Courant [face j][window col]
  T yf[NF][WIN];  // yfx
  T cx[WIN][PF];  // [window row][face i]
  T xf[WIN][PF];
  T mx[TW][PF];   // 0.5*mfx [interior row][face i]
  T my[NF][TW];   // 0.5*mfy [face j][interior col]
  T area[WIN][PQ];
  T rrx[WIN][PF];  // 1/ra_x [window row][interior col]
  T rry[TW][WIN];  // 1/ra_y [interior row][window col]
  T dpa[TW][TW];   // dp1/rarea
  T ub[TW][TW];    // rarea/dp2
  T edx[2][4][WIN];  // edge CTAs: dxa at window columns e-2..e+1 of x edge A/B, per window row
  T edy[2][4][WIN];  // dya at window rows e-2..e+1 of y edge A/B, per window column
};

template <typename T>
struct SmemWarp {
  T q[WIN][PQ];   // tracer window; S2 overwrites each row with q_j (interior columns)
  T qi[TW][PQ];   // q_i; then q dp1/rarea + x-flux divergence (or the x fluxes)
};

// Per-warp shared memory; edge CTAs add the edge deviations of two lines,
// [2][slots][32] values: 8 slots (bl, br of the 4 cells beside one edge) when
// no window holds both edges of a direction, 16 when one can (a compute
// domain of at most 28 cells in x or y).
template <typename T>
__host__ __device__ constexpr size_t warp_smem_bytes(bool edges, bool two_edges) {
  return sizeof(SmemWarp<T>) + (edges ? 2 * (two_edges ? 16 : 8) * 32 * sizeof(T) : 0);
}

__host__ __device__ __forceinline__ bool windows_hold_two_edges(int is, int ie, int js, int je) {
  return ie - is + 1 <= WIN - 4 || je - js + 1 <= WIN - 4;
}

// Edge CTAs of FP64 and dual-number states keep 16 slots everywhere (their
// shared memory does not limit them; the fixed layout keeps their registers).
template <typename T>
__host__ __device__ __forceinline__ bool edge_slots16(int is, int ie, int js, int je) {
  return sizeof(T) != 4 || windows_hold_two_edges(is, ie, js, je);
}

template <typename T>
size_t substep_smem_bytes(int warps, bool edges, bool two_edges) {
  return sizeof(SmemLevel<T>) + warps * warp_smem_bytes<T>(edges, two_edges);
}

// Edge-ring CTAs of FP32 states run as k_substep_ring32, capped at 8 warps
// and 128 registers so that two 8-warp CTAs fit an SM; FP64 and dual-number
// ones keep 10 warps (ring_max_warps).

// ------------------------------------------------------- PPM line stream ---
// Deviations (bl, br) of the four cells e-2..e+1 around a cube-face edge at
// window face e, computed once per line from shared memory and kept there
// (o[c*OS] = bl of cell e-2+c, o[(4+c)*OS] = br; lane-strided, OS = 32 values
// or, for one value of a pair of tracers, 64).  `east`: the
// tile interior lies below face e (the high edge of the tile).  The edge value
// is the mean of the two one-sided, dxa-weighted linear extrapolations.
//   hord 8: the edge value is clamped to the two cells beside it; the next
//     interface inward is s15 q + s11 q' -+ s14 dm' from the two cells on that
//     side (q' the one further in); the halo cell's outer interface uses the
//     same form from the halo side, so both tiles sharing the edge compute one
//     face value; the interface after that stays unlimited; CW84 on the three
//     cells at the edge.
//   hord 1 / 5: interfaces e-1 and e+1 are one-sided c1 q'' + c2 q' + c3 q
//     values, the edge value unlimited.
// Only cells 2..29 of a window feed its fluxes.
constexpr double kS11 = 11.0 / 14.0, kS14 = 4.0 / 7.0, kS15 = 3.0 / 14.0;
constexpr double kC1 = -2.0 / 14.0, kC2 = 11.0 / 14.0, kC3 = 5.0 / 14.0;

template <typename T, int HORD, class EX>
__device__ __forceinline__ T generic_bl(int c, EX&& x) {
  if (HORD == 8) {
    T dm0 = vl_slope(x(c - 2), x(c - 1), x(c)), dm1 = vl_slope(x(c - 1), x(c), x(c + 1));
    T al = T(0.5) * (x(c - 1) + x(c)) + (dm0 - dm1) * T(1.0 / 3.0);
    T xt = T(2) * dm1;
    return -tsign(tmin(tabs(xt), tabs(al - x(c))), xt);
  }
  return T(7.0 / 12.0) * (x(c - 1) + x(c)) - T(1.0 / 12.0) * (x(c - 2) + x(c + 1)) - x(c);
}

template <typename T, int HORD, class EX>
__device__ __forceinline__ T generic_br(int c, EX&& x) {
  if (HORD == 8) {
    T dm0 = vl_slope(x(c - 1), x(c), x(c + 1)), dm1 = vl_slope(x(c), x(c + 1), x(c + 2));
    T al = T(0.5) * (x(c) + x(c + 1)) + (dm0 - dm1) * T(1.0 / 3.0);
    T xt = T(2) * dm0;
    return tsign(tmin(tabs(xt), tabs(al - x(c))), xt);
  }
  return T(7.0 / 12.0) * (x(c) + x(c + 1)) - T(1.0 / 12.0) * (x(c - 1) + x(c + 2)) - x(c);
}

template <typename T, int HORD, int OS = 32, class EX, class ED>
__device__ __noinline__ void edge_devs(int e, bool east, EX x, ED ed, T* o) {
  if (e == NO_EDGE) return;
  bool need[4];
  for (int c = 0; c < 4; ++c) need[c] = (e - 2 + c >= 2 && e - 2 + c <= 29);
  T b[4] = {T(0), T(0), T(0), T(0)}, r[4] = {T(0), T(0), T(0), T(0)};
  auto dm = [&](int c) { return vl_slope(x(c - 1), x(c), x(c + 1)); };
  T a0 = T(0);
  if (need[1] || need[2]) {
    T d2 = ed(e - 2), d1 = ed(e - 1), d0 = ed(e), d3 = ed(e + 1);
    T xl = ((T(2) * d1 + d2) * x(e - 1) - d1 * x(e - 2)) / (d2 + d1);
    T xr = ((T(2) * d0 + d3) * x(e) - d0 * x(e + 1)) / (d0 + d3);
    a0 = T(0.5) * (xl + xr);
    if (HORD == 8) a0 = clamp2(a0, x(e - 1), x(e));
  }
  if (need[1]) r[1] = a0 - x(e - 1);
  if (need[2]) b[2] = a0 - x(e);
  if (HORD == 8) {
    if (!east) {
      T ap = T(0);
      if (need[2] || need[3]) ap = T(kS15) * x(e) + T(kS11) * x(e + 1) - T(kS14) * dm(e + 1);
      if (need[0]) { b[0] = generic_bl<T, HORD>(e - 2, x); r[0] = generic_br<T, HORD>(e - 2, x); }
      if (need[1]) b[1] = T(kS14) * dm(e - 2) + T(kS11) * (x(e - 2) - x(e - 1));
      if (need[2]) r[2] = ap - x(e);
      if (need[3]) {
        b[3] = ap - x(e + 1);
        r[3] = T(0.5) * (x(e + 1) + x(e + 2)) + (dm(e + 1) - dm(e + 2)) * T(1.0 / 3.0) - x(e + 1);
      }
      for (int c = 1; c < 4; ++c) cw84(b[c], r[c]);
    } else {
      T am = T(0);
      if (need[0] || need[1]) am = T(kS15) * x(e - 1) + T(kS11) * x(e - 2) + T(kS14) * dm(e - 2);
      if (need[0]) {
        b[0] = T(0.5) * (x(e - 3) + x(e - 2)) + (dm(e - 3) - dm(e - 2)) * T(1.0 / 3.0) - x(e - 2);
        r[0] = am - x(e - 2);
      }
      if (need[1]) b[1] = am - x(e - 1);
      if (need[2]) r[2] = T(kS11) * (x(e + 1) - x(e)) - T(kS14) * dm(e + 1);
      if (need[3]) { b[3] = generic_bl<T, HORD>(e + 1, x); r[3] = generic_br<T, HORD>(e + 1, x); }
      for (int c = 0; c < 3; ++c) cw84(b[c], r[c]);
    }
  } else {
    if (need[0] || need[1]) {
      const T aM = T(kC1) * x(e - 3) + T(kC2) * x(e - 2) + T(kC3) * x(e - 1);
      r[0] = aM - x(e - 2);
      b[1] = aM - x(e - 1);
    }
    if (need[2] || need[3]) {
      const T aP = T(kC3) * x(e) + T(kC2) * x(e + 1) + T(kC1) * x(e + 2);
      r[2] = aP - x(e);
      b[3] = aP - x(e + 1);
    }
    if (need[0]) b[0] = generic_bl<T, HORD>(e - 2, x);
    if (need[3]) r[3] = generic_br<T, HORD>(e + 1, x);
  }
  for (int c = 0; c < 4; ++c) { o[c * OS] = b[c]; o[(4 + c) * OS] = r[c]; }
}

// A line of 32 window cells x[0..31] marched with a rolling register window;
// face f separates cells f-1 and f, and faces 3..29 are the CTA tile's.
// Before step m the state holds x[m-3..m-1] (xa, xb, xc), dm[m-2] and al[m-2]
// (hord 8) and the right deviation and b0 = bl + br of cell m-3; step(x[m])
// finalises cell m-2 and returns the flux through face m-2 (valid for m >= 5).
//   hord 8: dm = monotonized central slope (clamp form), al = interface value,
//           |edge deviation| <= |2 dm| with the sign of dm (Lin 2004);
//   hord 1 / 5: fourth-order interfaces, unlimited, and the 2-dx filter: the
//           face takes the first-order upwind value when neither cell beside it
//           passes bl br < 0 (hord 5) or |lim_fac b0| < |bl - br| (hord 1);
//   flux  = x_up + w1 d_up - w2 b0_up with w1 = 1-|c|, w2 = |c| w1 and the
//           upwind cell's deviation at the face (CW84 parabola integral).
template <typename T>
__device__ __forceinline__ T dm_clamp(T xm, T x0, T xp) {
  const T xt = T(0.25) * (xp - xm);
  return copysign_t(tmin3(tabs(xt), tmax3(xm, x0, xp) - x0, x0 - tmin3(xm, x0, xp)), xt);
}

// Steps of a line whose cell m-2 lies next to a cube-face edge: bit m of
// mask, for the two edges at window faces eA and eB (warp-uniform).
struct EdgeSel {
  unsigned mask;
  int eA, eB;
  int sb;  // first slot of edge B: 8 when a window can hold both edges, else 0
};
__device__ __forceinline__ EdgeSel edge_sel(int eA, int eB, int sb) {
  auto bits = [](int e) { return (e >= 0 && e < 32) ? (0xFu << e) : 0u; };
  return EdgeSel{bits(eA) | bits(eB), eA, eB, sb};
}

template <typename T, int HORD>
struct Line {
  T xa, xb, xc, dmb, alb, pbr, pb0;
  T lim;     // hord 1: lim_fac
  bool psm;  // hord 1 / 5: cell m-3 passes the 2-dx filter test

  __device__ __forceinline__ void init(T lim_fac) {
    xa = xb = xc = dmb = alb = pbr = pb0 = T(0);
    lim = lim_fac;
    psm = true;
  }

  // ed: this lane's edge deviations (lane-strided slots: edge A bl0..3 br0..3, then edge B from slot sb)
  template <bool EDGES>
  __device__ __forceinline__ T step(int m, T x, T c, const T* ed, const EdgeSel& es) {
    T alc, bl, br;
    if (HORD == 8) {
      const T dmc = dm_clamp(xb, xc, x);                      // dm[m-1]
      alc = T(0.5) * (xb + xc) + (dmb - dmc) * T(1.0 / 3.0);  // al[m-1]
      const T xt = dmb + dmb;                                 // cell m-2
      const T axt = tabs(xt);
      bl = copysign_t(tmin(axt, tabs(alb - xb)), -xt);
      br = copysign_t(tmin(axt, tabs(alc - xb)), xt);
      dmb = dmc;
    } else {
      alc = T(7.0 / 12.0) * (xb + xc) - T(1.0 / 12.0) * (xa + x);
      bl = alb - xb;
      br = alc - xb;
    }
    if (EDGES && ((es.mask >> m) & 1u)) {  // cell m-2 is cell e-2+d of an edge
      const int dA = m - es.eA;
      const int slot = (unsigned)dA < 4u ? dA : es.sb + (m - es.eB);
      bl = ed[slot * 32];
      br = ed[(slot + 4) * 32];
    }
    const T b0 = bl + br;
    const T a = tabs(c);
    const T w1 = T(1) - a, w2 = a * w1;
    T fl_l = (xa + w1 * pbr) - w2 * pb0;  // upwind cell on the left (c > 0)
    T fl_r = (xb + w1 * bl) - w2 * b0;
    if (HORD != 8) {
      // 2-dx filter: first-order upwind flux between two extrema
      const bool sm = (HORD == 5) ? (bl * br < T(0)) : (tabs(lim * b0) < tabs(bl - br));
      if (!(sm || psm)) {
        fl_l = xa;
        fl_r = xb;
      }
      psm = sm;
    }
    const T fl = c > T(0) ? fl_l : fl_r;
    xa = xb;
    xb = xc;
    xc = x;
    alb = alc;
    pbr = br;
    pb0 = b0;
    return fl;
  }
};

// Two FP32 hord-8 lines marched in lockstep as packed pairs (two tracers of
// one line, or two lines of one tracer that see the same faces), value for
// value the march of Line<float, 8>:
// before step m the state holds x[m-3..m-1] (xa, xb, xc), the slope of cell
// m-2 (dmb, as magnitude mb and sign sb) and its interface al (alb), and the
// right deviation and b0 of cell m-3; step(x[m]) finalises cell m-2 and
// returns the flux through face m-2 (valid for m >= 5).
struct PairLine {
  F2 xa, xb, xc, dmb, mb, sb, alb, pbr, pb0;

  __device__ __forceinline__ void init() {
    xa = xb = xc = dmb = mb = alb = pbr = pb0 = bc(0.f);
    sb = bc(1.f);
  }

  // ed: the pair's edge-deviation slots (lane-strided pairs); or, for two
  // lines with separate slots, edx for the first value and edy for the second
  template <bool EDGES>
  __device__ __forceinline__ F2 step(int m, F2 x, float c, const F2* ed, const EdgeSel& es) {
    return step2<EDGES, true>(m, x, c, ed, nullptr, nullptr, es);
  }
  template <bool EDGES, bool PAIRED_SLOTS>
  __device__ __forceinline__ F2 step2(int m, F2 x, float c, const F2* ed, const float* edx, const float* edy,
                                      const EdgeSel& es) {
    // monotonized central slope of cell m-1 (half increments), |dm| and sign
    const F2 xt = mul2(sub2(x, xb), bc(0.25f));
    const F2 mag = min3_2(abs2(xt), sub2(max3_2(xb, xc, x), xc), sub2(xc, min3_2(xb, xc, x)));
    const F2 sg = sign2(xt);
    const F2 dmc = mul2(mag, sg);
    const F2 alc = fma2(sub2(dmb, dmc), bc(1.f / 3.f), mul2(bc(0.5f), add2(xb, xc)));  // al[m-1]
    // cell m-2: edge deviations at most |2 dm| with the sign of dm (Lin 2004)
    const F2 two = add2(mb, mb);
    F2 bl = mul2(min2(two, abs2(sub2(alb, xb))), neg2(sb));
    F2 br = mul2(min2(two, abs2(sub2(alc, xb))), sb);
    dmb = dmc;
    mb = mag;
    sb = sg;
    if (EDGES && ((es.mask >> m) & 1u)) {  // cell m-2 is cell e-2+d of an edge
      const int dA = m - es.eA;
      const int slot = (unsigned)dA < 4u ? dA : es.sb + (m - es.eB);
      if (PAIRED_SLOTS) {
        bl = ed[slot * 32];
        br = ed[(slot + 4) * 32];
      } else {
        bl = F2{edx[slot * 32], edy[slot * 32]};
        br = F2{edx[(slot + 4) * 32], edy[(slot + 4) * 32]};
      }
    }
    const F2 b0 = add2(bl, br);
    const float a = fabsf(c);
    const float w1 = 1.f - a, w2 = a * w1;
    const F2 fl_l = fma2(bc(-w2), pb0, fma2(bc(w1), pbr, xa));  // upwind cell on the left (c > 0)
    const F2 fl_r = fma2(bc(-w2), b0, fma2(bc(w1), bl, xb));
    const F2 fl = c > 0.f ? fl_l : fl_r;
    xa = xb;
    xb = xc;
    xc = x;
    alb = alc;
    pbr = br;
    pb0 = b0;
    return fl;
  }
};

// One element of a plane, its indices clamped into the plane, into shared
// memory by an asynchronous copy (copy_async).
template <typename T>
__device__ __forceinline__ void stage_ld(T* dst, const T* base, const PlaneGeom& pg, int i, int j) {
  i = min(max(i, pg.isd), pg.isd + pg.pitch - 1);
  j = min(max(j, pg.jsd), pg.jsd + pg.rows - 1);
  copy_async(dst, base + pg.at(i, j));
}

// ------------------------------------------------------------ the kernel ---
// One tracer of one CTA tile through the three stages (see file header).
template <typename T, int HORD, bool FLUXES, bool EDGES>
__device__ __forceinline__ void advance_tracer(const AdvArgs<T>& a, SmemLevel<T>& L, SmemWarp<T>& S, int t, int k,
                                               T* eds, int iq, int i0, int j0, int ni, int nj, int lane, int exA,
                                               int exB, int eyA, int eyB, bool corner_block,
                                               long long efo, long long efe, int nslot) {
  const PlaneGeom& pg = a.pg;
  const int n = a.npx - 1;
  // Cube-corner halo blocks of the window, which copy_corners fills by a
  // rotation that depends on the sweep direction (1 = x, 2 = y).
  auto corner_cells = [&](int dir) {
    const int i = i0 - 3 + lane;
#pragma unroll 1
    for (int r = 0; r < WIN; ++r) {
      const int j = j0 - 3 + r;
      const bool oi = (i < 1) || (i > a.npx - 1), oj = (j < 1) || (j > a.npy - 1);
      if (oi && oj) S.q[r][lane] = load_q(a, t, iq, k, i, j, dir);
    }
  };
  // ------------------------------------------ window load (y-sweep corners)
  // The planes hold their halo strips (caller-filled, or k_cube_halo); cells
  // beyond the plane are clamped and feed only discarded outputs.
  auto load_window = [&](const T* base) {
    const int ic = min(max(i0 - 3 + lane, pg.isd), pg.isd + pg.pitch - 1);
    const T* src = base + t * a.sQt + iq * a.sQq + k * a.sQk + (ic - pg.isd);
    const int jhi = pg.jsd + pg.rows - 1;
    // every row in flight (asynchronous copies wait for nothing in the loop and hold no registers), then
    // one wait for them all: the corner cells written next must land after the copies
#pragma unroll 8
    for (int r = 0; r < WIN; ++r) {
      const int jr = min(max(j0 - 3 + r, pg.jsd), jhi);
      copy_async(&S.q[r][lane], src + (long long)(jr - pg.jsd) * pg.pitch);
    }
    stage_wait();
  };
  load_window(a.q_in);
  if (corner_block) corner_cells(2);
  __syncwarp();

  T fyr[NF];  // inner y flux of this lane's column at faces 3..29 (S1 -> S3)
  const int sb = nslot - 8;
  const EdgeSel esx = edge_sel(exA, exB, sb), esy = edge_sel(eyA, eyB, sb);
  // edge deviations of the lines in flight: eds[line][nslot][32], lines 0 (and 1 in S2)
  T* const ed0 = eds + lane;
  T* const ed1 = eds + nslot * 32 + lane;
  // ------------------------------------------------ S1: inner y, q_i ------
  {
    const int w = lane;
    const T* qcol = &S.q[0][w];
    if (EDGES) {
      auto ex = [qcol](int m) { return qcol[m * PQ]; };
      auto edA = [&L, w, eyA](int m) { return L.edy[0][m - eyA + 2][w]; };
      auto edB = [&L, w, eyB](int m) { return L.edy[1][m - eyB + 2][w]; };
      edge_devs<T, HORD>(eyA, false, ex, edA, ed0);
      edge_devs<T, HORD>(eyB, true, ex, edB, ed0 + sb * 32);
    }
    Line<T, HORD> ln;
    ln.init(T(a.lim_fac));
#pragma unroll
    for (int m = 0; m < 5; ++m) ln.template step<EDGES>(m, qcol[m * PQ], T(0), ed0, esy);
    fyr[0] = ln.template step<EDGES>(5, qcol[5 * PQ], L.cy[0][w], ed0, esy);
    T fyy_prev = L.yf[0][w] * fyr[0];
#pragma unroll
    for (int m = 6; m < WIN; ++m) {
      const int f = m - 2;
      const T xrow = ln.xa;  // cell row f-1 = m-3
      fyr[f - 3] = ln.template step<EDGES>(m, qcol[m * PQ], L.cy[f - 3][w], ed0, esy);
      const T fyy = L.yf[f - 3][w] * fyr[f - 3];
      S.qi[f - 4][w] = (xrow * L.area[f - 1][w] + fyy_prev - fyy) * L.rry[f - 4][w];
      fyy_prev = fyy;
    }
  }
  __syncwarp();

  // -------------------------------------- corner blocks for the x sweeps
  if (a.q_in_x != nullptr) {  // separate input of the x sweeps (adjoint assembly)
    load_window(a.q_in_x);
    __syncwarp();
  } else if (corner_block) {
    corner_cells(1);
    __syncwarp();
  }

  // ---------- S2: inner x -> q_j (into the q row); outer x on q_i -> P -----
  {
    const int r = lane;
    const bool outer = (r >= 3) && (r < 29);
    const int ro = outer ? r - 3 : 0;
    T* qrow = &S.q[r][0];
    T* qirow = &S.qi[ro][0];
    if (EDGES) {
      auto exi = [qrow](int m) { return qrow[m]; };
      auto exo = [qirow](int m) { return qirow[m]; };
      auto edA = [&L, r, exA](int m) { return L.edx[0][m - exA + 2][r]; };
      auto edB = [&L, r, exB](int m) { return L.edx[1][m - exB + 2][r]; };
      edge_devs<T, HORD>(exA, false, exi, edA, ed0);
      edge_devs<T, HORD>(exB, true, exi, edB, ed0 + sb * 32);
      if (outer) {
        edge_devs<T, HORD>(exA, false, exo, edA, ed1);
        edge_devs<T, HORD>(exB, true, exo, edB, ed1 + sb * 32);
      }
    }
    const bool efw = EDGES && a.cube && a.eflux != nullptr && outer && ro < nj;
    if constexpr (std::is_same<T, float>::value && HORD == 8 && !FLUXES) {
      // FP32 hord 8: the inner line (q) and the outer one (q_i) of this row see
      // the same faces, so they march as one packed pair (x: inner, y: outer)
      PairLine lp;
      lp.init();
      auto pstep = [&](int m, float c) {
        return lp.template step2<EDGES, false>(m, F2{qrow[m], qirow[m]}, c, nullptr, ed0, ed1, esx);
      };
#pragma unroll
      for (int m = 0; m < 5; ++m) pstep(m, 0.f);
      F2 fr = pstep(5, L.cx[r][0]);  // face 3: (inner flux fx2, outer flux fo)
      float fxx_prev = L.xf[r][0] * fr.x;
      float F_prev = (fr.y + fr.x) * L.mx[ro][0];
      if (efw && i0 == 1) a.eflux[efo + iq * (long long)n + (j0 + ro - 1)] = -F_prev;
      // interior CTAs unroll the march fully (the line's rolling state then needs no register moves:
      // 76 registers against 86); the edge-ring CTAs, at their 128-register cap, by two
#pragma unroll(EDGES ? 2 : WIN)
      for (int m = 6; m < WIN; ++m) {
        const int f = m - 2;
        const float xcol = lp.xa.x;  // q at window column f-1 of this row
        fr = pstep(m, L.cx[r][f - 3]);
        const float fxx = L.xf[r][f - 3] * fr.x;
        qrow[f - 4] = (xcol * L.area[r][f - 1] + fxx_prev - fxx) * L.rrx[r][f - 4];
        fxx_prev = fxx;
        const float F = (fr.y + fr.x) * L.mx[ro][f - 3];
        if (outer) qirow[f - 4] = xcol * L.dpa[ro][f - 4] + (F_prev - F);
        if (efw && i0 + f - 3 == a.npx) a.eflux[efo + efe + iq * (long long)n + (j0 + ro - 1)] = F;
        F_prev = F;
      }
    } else {
      Line<T, HORD> li, lo;
      li.init(T(a.lim_fac));
      lo.init(T(a.lim_fac));
#pragma unroll
      for (int m = 0; m < 5; ++m) {
        li.template step<EDGES>(m, qrow[m], T(0), ed0, esx);
        lo.template step<EDGES>(m, qirow[m], T(0), ed1, esx);
      }
      // face 3
      T c = L.cx[r][0];
      T fx2 = li.template step<EDGES>(5, qrow[5], c, ed0, esx);
      T fo = lo.template step<EDGES>(5, qirow[5], c, ed1, esx);
      T fxx_prev = L.xf[r][0] * fx2;
      T F_prev = (fo + fx2) * L.mx[ro][0];
      if (FLUXES && outer) qirow[0] = F_prev;
      if (efw && i0 == 1) a.eflux[efo + iq * (long long)n + (j0 + ro - 1)] = -F_prev;
#pragma unroll 2
      for (int m = 6; m < WIN; ++m) {
        const int f = m - 2;
        const T xcol = li.xa;  // q at window column f-1 of this row
        c = L.cx[r][f - 3];
        fx2 = li.template step<EDGES>(m, qrow[m], c, ed0, esx);
        fo = lo.template step<EDGES>(m, qirow[m], c, ed1, esx);
        const T fxx = L.xf[r][f - 3] * fx2;
        // q_j of window column f-1 (interior column f-4); column m-6 of this row is consumed
        qrow[f - 4] = (xcol * L.area[r][f - 1] + fxx_prev - fxx) * L.rrx[r][f - 4];
        fxx_prev = fxx;
        const T F = (fo + fx2) * L.mx[ro][f - 3];
        if (outer) {
          if (FLUXES) qirow[f - 3] = F;  // column f-3 was consumed at step f-3
          else qirow[f - 4] = xcol * L.dpa[ro][f - 4] + (F_prev - F);  // q dp1/rarea + x divergence
        }
        if (efw && i0 + f - 3 == a.npx) a.eflux[efo + efe + iq * (long long)n + (j0 + ro - 1)] = F;
        F_prev = F;
      }
    }
  }
  __syncwarp();

  // ---------------------------- S3: outer y on q_j, update / write -------
  if (lane >= 3 && lane < 3 + TW) {
    const int c = lane - 3;  // interior column
    const T* qjcol = &S.q[0][c];
    if (EDGES) {
      auto ex = [qjcol](int m) { return qjcol[m * PQ]; };
      auto edA = [&L, c, eyA](int m) { return L.edy[0][m - eyA + 2][c + 3]; };
      auto edB = [&L, c, eyB](int m) { return L.edy[1][m - eyB + 2][c + 3]; };
      edge_devs<T, HORD>(eyA, false, ex, edA, ed0);
      edge_devs<T, HORD>(eyB, true, ex, edB, ed0 + sb * 32);
    }
    const int ig = i0 + c;
    const bool valid_c = c < ni;
    const bool efw = EDGES && a.cube && a.eflux != nullptr && valid_c;
    T* qo = a.q_out + t * a.sQt + iq * a.sQq + k * a.sQk + pg.at(ig, j0);
    T* fyo = FLUXES ? a.fy_out + (long long)(k * a.nq + iq) * a.sFlux + pg.at(ig, j0) : nullptr;
    Line<T, HORD> ln;
    ln.init(T(a.lim_fac));
#pragma unroll
    for (int m = 0; m < 5; ++m) ln.template step<EDGES>(m, qjcol[m * PQ], T(0), ed0, esy);
    T Fprev = (ln.template step<EDGES>(5, qjcol[5 * PQ], L.cy[0][c + 3], ed0, esy) + fyr[0]) * L.my[0][c];
    if (FLUXES && valid_c) fyo[0] = Fprev;
    if (efw && j0 == 1) a.eflux[efo + 2 * efe + iq * (long long)n + (ig - 1)] = -Fprev;
#pragma unroll
    for (int m = 6; m < WIN; ++m) {
      const int f = m - 2;
      const T F = (ln.template step<EDGES>(m, qjcol[m * PQ], L.cy[f - 3][c + 3], ed0, esy) + fyr[f - 3]) *
                  L.my[f - 3][c];
      const int ir = f - 4;  // interior row between faces f-1 and f
      if (FLUXES) {
        if (valid_c && f - 3 <= nj) fyo[(long long)(f - 3) * pg.pitch] = F;
      } else if (ir < nj && valid_c) {
        qo[(long long)ir * pg.pitch] = (S.qi[ir][c] + Fprev - F) * L.ub[ir][c];
      }
      if (efw && j0 + f - 3 == a.npy) a.eflux[efo + 3 * efe + iq * (long long)n + (ig - 1)] = F;
      Fprev = F;
    }
  }
  if (FLUXES) {  // x fluxes staged in qi by S2
    __syncwarp();
    T* fxo = a.fx_out + (long long)(k * a.nq + iq) * a.sFlux;
    for (int e = lane; e < TW * NF; e += 32) {
      const int ir = e / NF, f = e % NF;
      if (ir < nj && f <= ni) fxo[pg.at(i0 + f, j0 + ir)] = S.qi[ir][f];
    }
  }
  __syncwarp();
}

// Interior CTAs (no cube-face edge in their window) and edge CTAs run as two
// instantiations: the edge code path costs registers the interior one does
// not need.  Interior CTAs cover the rectangle [bx0, bx0+nbxi) x [by0,
// by0+nbyi) of CTA tiles; edge CTAs enumerate the ring around it row by row.
// CTA tile of a substep launch: interior CTAs cover the rectangle [bx0,
// bx0+nbxi) x [by0, by0+nbyi) of CTA tiles; edge CTAs enumerate the ring
// around it row by row.  Returns the tile's first cell (i0, j0) and size.
struct TileCtx {
  int t, k, i0, j0, ni, nj, exA, exB, eyA, eyB;
  bool corner_block;
};

template <typename T, bool EDGES>
__device__ __forceinline__ TileCtx tile_of(const AdvArgs<T>& a, const BlockMap& bm) {
  TileCtx c;
  c.t = blockIdx.z;
  c.k = blockIdx.y;
  int bx, by;
  {
    const int e = blockIdx.x;
    if (!EDGES) {
      bx = bm.bx0 + e % bm.nbxi;
      by = bm.by0 + e / bm.nbxi;
    } else {
      const int top = bm.by0 * bm.nbx, nside = bm.nbx - bm.nbxi, mid = nside * bm.nbyi;
      if (e < top) {
        by = e / bm.nbx;
        bx = e % bm.nbx;
      } else if (e < top + mid) {
        const int r = e - top, sx = r % nside;
        by = bm.by0 + r / nside;
        bx = sx < bm.bx0 ? sx : sx + bm.nbxi;
      } else {
        const int r = e - top - mid;
        by = bm.by0 + bm.nbyi + r / bm.nbx;
        bx = r % bm.nbx;
      }
    }
  }
  c.i0 = a.is + bx * TW;
  c.j0 = a.js + by * TW;
  c.ni = min(TW, a.ie - c.i0 + 1);
  c.nj = min(TW, a.je - c.j0 + 1);
  // window faces of cube-face edges (x: west/east, y: south/north)
  c.exA = EDGES ? window_edge_lo(a.is, c.i0, a.nested) : NO_EDGE;
  c.exB = EDGES ? window_edge_hi(a.ie, a.npx, c.i0, a.nested) : NO_EDGE;
  c.eyA = EDGES ? window_edge_lo(a.js, c.j0, a.nested) : NO_EDGE;
  c.eyB = EDGES ? window_edge_hi(a.je, a.npy, c.j0, a.nested) : NO_EDGE;
  c.corner_block = !a.nested && a.corners != 0 && ((c.i0 - 3 < 1) || (c.i0 + 28 > a.npx - 1)) &&
                   ((c.j0 - 3 < 1) || (c.j0 + 28 > a.npy - 1));
  return c;
}

// One element of a plane field (clamped into the plane, as ld_field) into
// shared memory: FP32 and FP64 values by an asynchronous copy (cp.async, no
// register round trip, many in flight per thread), other types by a load.

// Per-level fields of a CTA tile into shared memory (Courant numbers, area
// and mass fluxes, 1/ra_x, 1/ra_y, dp ratios; edge metrics for edge CTAs);
// writes dp2 of the tile's cells.  Ends with a CTA barrier.
// Phase 1 copies every raw window asynchronously (the windows of dp1 and
// rarea into dpa and ub, a caller's ra_x / ra_y into rrx / rry); phase 2
// forms the derived values from shared memory with the same arithmetic as
// the field expressions; phase 3 halves the mass fluxes.
template <typename T, bool EDGES>
__device__ __forceinline__ void stage_level(const AdvArgs<T>& a, SmemLevel<T>& L, const TileCtx& tc) {
  const PlaneGeom& pg = a.pg;
  const int t = tc.t, k = tc.k, i0 = tc.i0, j0 = tc.j0, ni = tc.ni, nj = tc.nj;
  const int exA = tc.exA, exB = tc.exB, eyA = tc.eyA, eyB = tc.eyB;
  const long long fo = t * a.sFt + k * a.sFk;
  const T* cx = a.cx + fo;
  const T* cy = a.cy + fo;
  const T* xf = a.xfx + fo;
  const T* yf = a.yfx + fo;
  const T* mx = a.mfx + fo;
  const T* my = a.mfy + fo;
  const T* area = a.area + t * a.sMt;
  const T* rarea = a.rarea + t * a.sMt;
  const T* dp1 = a.dp1 ? a.dp1 + fo : nullptr;
  T* dp2o = a.dp2 ? a.dp2 + fo : nullptr;
  // ---- phase 1: raw windows
  for (int e = threadIdx.x; e < NF * WIN; e += blockDim.x) {
    const int f = e / WIN, w = e % WIN;
    stage_ld(&L.cy[f][w], cy, pg, i0 - 3 + w, j0 + f);
    stage_ld(&L.yf[f][w], yf, pg, i0 - 3 + w, j0 + f);
  }
  for (int e = threadIdx.x; e < WIN * NF; e += blockDim.x) {
    const int r = e / NF, f = e % NF;
    stage_ld(&L.cx[r][f], cx, pg, i0 + f, j0 - 3 + r);
    stage_ld(&L.xf[r][f], xf, pg, i0 + f, j0 - 3 + r);
  }
  for (int e = threadIdx.x; e < TW * NF; e += blockDim.x) {
    const int r = e / NF, f = e % NF;
    stage_ld(&L.mx[r][f], mx, pg, i0 + f, j0 + r);
    const int ff = e / TW, c = e % TW;
    stage_ld(&L.my[ff][c], my, pg, i0 + c, j0 + ff);
  }
  for (int e = threadIdx.x; e < WIN * WIN; e += blockDim.x) {
    const int r = e / WIN, w = e % WIN;
    stage_ld(&L.area[r][w], area, pg, i0 - 3 + w, j0 - 3 + r);
  }
  if (a.ra_x || a.ra_y) {
    for (int e = threadIdx.x; e < WIN * TW; e += blockDim.x) {
      const int r = e / TW, c = e % TW;
      if (a.ra_x) stage_ld(&L.rrx[r][c], a.ra_x, pg, i0 + c, j0 - 3 + r);
      const int r2 = e / WIN, w = e % WIN;
      if (a.ra_y) stage_ld(&L.rry[r2][w], a.ra_y, pg, i0 - 3 + w, j0 + r2);
    }
  }
  if (dp1 != nullptr) {
    for (int e = threadIdx.x; e < TW * TW; e += blockDim.x) {
      const int r = e / TW, c = e % TW;
      stage_ld(&L.dpa[r][c], dp1, pg, i0 + c, j0 + r);
      stage_ld(&L.ub[r][c], rarea, pg, i0 + c, j0 + r);
    }
  }
  if (EDGES) {  // metrics of the one-sided edge values: dxa across x edges, dya across y edges
    const T* dxa = a.dxa + t * a.sMt;
    const T* dya = a.dya + t * a.sMt;
    for (int e = threadIdx.x; e < 2 * 4 * WIN; e += blockDim.x) {
      const int side = e / (4 * WIN), m = (e / WIN) % 4, w = e % WIN;
      const int ex = side ? exB : exA, ey = side ? eyB : eyA;
      if (ex == NO_EDGE) L.edx[side][m][w] = T(1);
      else stage_ld(&L.edx[side][m][w], dxa, pg, i0 - 3 + ex - 2 + m, j0 - 3 + w);
      if (ey == NO_EDGE) L.edy[side][m][w] = T(1);
      else stage_ld(&L.edy[side][m][w], dya, pg, i0 - 3 + w, j0 - 3 + ey - 2 + m);
    }
  }
  stage_wait();
  __syncthreads();
  // ---- phase 2: derived values
  for (int e = threadIdx.x; e < WIN * TW; e += blockDim.x) {
    const int r = e / TW, c = e % TW;
    L.rrx[r][c] = T(1) / (a.ra_x ? L.rrx[r][c] : L.area[r][c + 3] + L.xf[r][c] - L.xf[r][c + 1]);
    const int r2 = e / WIN, w = e % WIN;
    L.rry[r2][w] = T(1) / (a.ra_y ? L.rry[r2][w] : L.area[r2 + 3][w] + L.yf[r2][w] - L.yf[r2 + 1][w]);
  }
  if (dp1 != nullptr) {
    for (int e = threadIdx.x; e < TW * TW; e += blockDim.x) {
      const int r = e / TW, c = e % TW;
      const T d1 = L.dpa[r][c], ra = L.ub[r][c];
      const T d2 = d1 + (L.mx[r][c] - L.mx[r][c + 1] + L.my[r][c] - L.my[r + 1][c]) * ra;
      L.dpa[r][c] = d1 / ra;
      L.ub[r][c] = ra / d2;
      if (r < nj && c < ni) {
        if (dp2o != nullptr) dp2o[pg.at(i0 + c, j0 + r)] = d2;
        if (!(d2 > T(0))) raise_error(a.err, FV3G_E_DELP);
      }
    }
  }
  __syncthreads();
  // ---- phase 3: 0.5 mfx, 0.5 mfy
  for (int e = threadIdx.x; e < TW * NF; e += blockDim.x) {
    const int r = e / NF, f = e % NF;
    L.mx[r][f] = T(0.5) * L.mx[r][f];
    const int ff = e / TW, c = e % TW;
    L.my[ff][c] = T(0.5) * L.my[ff][c];
  }
  __syncthreads();
}

template <typename T, int HORD, bool FLUXES, bool EDGES>
__device__ __forceinline__ void substep_body(const AdvArgs<T>& a, const BlockMap& bm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemLevel<T>& L = *reinterpret_cast<SmemLevel<T>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, W = blockDim.x >> 5;
  const bool two = EDGES && edge_slots16<T>(a.is, a.ie, a.js, a.je);
  unsigned char* wbase = smem_raw + sizeof(SmemLevel<T>) + warp * warp_smem_bytes<T>(EDGES, two);
  SmemWarp<T>& S = *reinterpret_cast<SmemWarp<T>*>(wbase);
  T* eds = reinterpret_cast<T*>(wbase + sizeof(SmemWarp<T>));
  const TileCtx tc = tile_of<T, EDGES>(a, bm);
  stage_level<T, EDGES>(a, L, tc);
  const int t = tc.t, k = tc.k, i0 = tc.i0, j0 = tc.j0, ni = tc.ni, nj = tc.nj;
  const int exA = tc.exA, exB = tc.exB, eyA = tc.eyA, eyB = tc.eyB;
  const int n = a.npx - 1;
  const bool corner_block = tc.corner_block;
  // edge-flux index (((t*4 + e)*npz + k)*nq + iq)*n + s = efo + e*efe + iq*n + s
  const long long efe = (long long)a.npz * a.nq * n;
  const long long efo = (((long long)t * 4) * a.npz + k) * a.nq * n;

  for (int iq = warp; iq < a.nq; iq += W)
    advance_tracer<T, HORD, FLUXES, EDGES>(a, L, S, t, k, eds, iq, i0, j0, ni, nj, lane, exA, exB, eyA, eyB,
                                           corner_block, efo, efe, two ? 16 : 8);
}

template <typename T, int HORD, bool FLUXES, bool EDGES>
__global__ void __launch_bounds__(320) k_substep(const AdvArgs<T> a, const BlockMap bm) {
  substep_body<T, HORD, FLUXES, EDGES>(a, bm);
}

template <int HORD, bool FLUXES>
__global__ void __launch_bounds__(256, 2) k_substep_ring32(const AdvArgs<float> a, const BlockMap bm) {
  substep_body<float, HORD, FLUXES, true>(a, bm);
}

template <typename T, int HORD, bool FLUXES>
static int launch_one(const AdvArgs<T>& a, int warps, cudaStream_t s) {
  const BlockMap bm = block_map(a.is, a.ie, a.js, a.je, a.npx, a.npy, a.nested);
  const int nint = bm.nbxi * bm.nbyi, nring = bm.nbx * bm.nby - nint;
  const int nt = adv_tiles(a);
  // edge-ring CTAs may run narrower (and at most ring_max_warps wide)
  const int wr = std::min(a.warps_ring > 0 ? a.warps_ring : warps, ring_max_warps((int)sizeof(T)));
  const bool two = edge_slots16<T>(a.is, a.ie, a.js, a.je);
  if (nint > 0) {
    dim3 grid(nint, a.npz, nt);
    k_substep<T, HORD, FLUXES, false><<<grid, 32 * warps, substep_smem_bytes<T>(warps, false, false), s>>>(a, bm);
    FV3G_CUDA(cudaGetLastError());
  }
  if (nring > 0) {
    dim3 grid(nring, a.npz, nt);
    if constexpr (sizeof(T) == 4)
      k_substep_ring32<HORD, FLUXES><<<grid, 32 * wr, substep_smem_bytes<T>(wr, true, two), s>>>(a, bm);
    else
      k_substep<T, HORD, FLUXES, true><<<grid, 32 * wr, substep_smem_bytes<T>(wr, true, two), s>>>(a, bm);
    FV3G_CUDA(cudaGetLastError());
  }
  return 0;
}

// Largest warps per CTA whose shared memory fits in 227 KB (at most 10).
template <typename T>
static int max_warps() {
  int w = 10;
  while (w > 1 && substep_smem_bytes<T>(w, true, true) > 227 * 1024) --w;
  return w;
}

template <typename T, int HORD, bool FLUXES, bool EDGES>
static cudaError_t set_smem_attr() {
  const int mx = (int)substep_smem_bytes<T>(max_warps<T>(), EDGES, true);
  if constexpr (EDGES && sizeof(T) == 4)
    return cudaFuncSetAttribute(k_substep_ring32<HORD, FLUXES>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
  else
    return cudaFuncSetAttribute(k_substep<T, HORD, FLUXES, EDGES>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

template <typename T, int HORD>
static void set_attrs_tl(cudaError_t& err) {
  cudaError_t es[] = {set_smem_attr<T, HORD, true, false>(), set_smem_attr<T, HORD, true, true>()};
  for (cudaError_t e : es)
    if (e != cudaSuccess && err == cudaSuccess) err = e;
}

template <typename T, int HORD>
static void set_attrs(cudaError_t& err) {
  cudaError_t es[] = {set_smem_attr<T, HORD, false, false>(), set_smem_attr<T, HORD, false, true>(),
                      set_smem_attr<T, HORD, true, false>(), set_smem_attr<T, HORD, true, true>()};
  for (cudaError_t e : es)
    if (e != cudaSuccess && err == cudaSuccess) err = e;
}

template <typename T, int HORD>
int launch_substep_hord(const AdvArgs<T>& a, bool flux_mode, int warps, cudaStream_t s) {
  const int mw = max_warps<T>(), mr = std::min(mw, ring_max_warps((int)sizeof(T)));
  if (warps < 1 || warps > mw || a.warps_ring < 0 || a.warps_ring > mr)
    return set_error(FV3G_E_ARG,
                     "this precision supports 1..%d advection warps per CTA and 1..%d per edge-ring CTA (got %d, %d)",
                     mw, mr, warps, a.warps_ring);
  return flux_mode ? launch_one<T, HORD, true>(a, warps, s) : launch_one<T, HORD, false>(a, warps, s);
}

template <int HORD>
int launch_substep_tl_hord(const AdvArgs<Dual<double>>& a, cudaStream_t s) {
  return launch_one<Dual<double>, HORD, true>(a, 1, s);
}

template <int HORD>
void prepare_substep_hord(cudaError_t& err) {
  set_attrs<float, HORD>(err);
  set_attrs<double, HORD>(err);
  set_attrs_tl<Dual<double>, HORD>(err);
}

}  // namespace fv3g

#define FV3G_SUBSTEP_INSTANTIATE(H)                                                                       \
  namespace fv3g {                                                                                       \
  template int launch_substep_hord<float, H>(const AdvArgs<float>&, bool, int, cudaStream_t);            \
  template int launch_substep_hord<double, H>(const AdvArgs<double>&, bool, int, cudaStream_t);          \
  template int launch_substep_tl_hord<H>(const AdvArgs<Dual<double>>&, cudaStream_t);                     \
  template void prepare_substep_hord<H>(cudaError_t&);                                                   \
  }
