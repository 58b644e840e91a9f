// fv3g_advect.cu -- fused fv_tp_2d + flux-form update (one tracer_2d substep).
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
//   S3  lane = interior column: outer y-PPM on q_j, final y flux, and the
//       flux-form update q <- (q dp1 + div F * rarea) / dp2 written to HBM.
// Each lane marches its line with a register pipeline (slope -> interface ->
// edge deviations -> flux), so intermediate fluxes never leave the SM and q
// is read once and written once per substep.  Halo cells are gathered from
// the neighbouring tiles of the cube (or read from the caller's halo), and
// the cube-corner blocks are filled by the rotation of copy_corners at load.
#include <cstdio>
#include <algorithm>
#include <mutex>
#include <type_traits>

#include "fv3g_internal.cuh"

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
  T ua[TW][TW];    // dp1/dp2
  T ub[TW][TW];    // rarea/dp2
};

template <typename T>
struct SmemWarp {
  T q[WIN][PQ];   // tracer window
  T qi[TW][PQ];   // q_i; later the x-flux divergence (or x fluxes)
  T qj[WIN][PF];  // q_j [window row][interior col]
  T fy2[NF][TW];  // inner y flux [face][interior col]
};

size_t substep_smem_bytes(bool fp64, int warps) {
  return fp64 ? sizeof(SmemLevel<double>) + warps * sizeof(SmemWarp<double>)
              : sizeof(SmemLevel<float>) + warps * sizeof(SmemWarp<float>);
}

// ----------------------------------------------------------- halo source ---
// Rotate a cube-corner halo cell (tile indices) into the halo strip that a
// sweep in direction dir (1 = x, 2 = y) continues: about the corner point,
// +90 deg maps (u,v) -> (-v,u) and -90 deg maps (u,v) -> (v,-u).
__device__ __forceinline__ void corner_rotate(int& i, int& j, int npx, int npy, int dir) {
  const int su = (i < 1) ? -1 : 1, sv = (j < 1) ? -1 : 1;
  const int cx2 = (su < 0) ? 1 : 2 * npx - 1;  // doubled corner coordinates
  const int cy2 = (sv < 0) ? 1 : 2 * npy - 1;
  const int U = 2 * i - cx2, V = 2 * j - cy2;
  const bool plus = (dir == 1) ? (su == -sv) : (su == sv);
  const int U2 = plus ? -V : V, V2 = plus ? U : -U;
  i = (U2 + cx2) / 2;
  j = (V2 + cy2) / 2;
}

// Interior cell of the neighbouring tile that tile t's edge-halo cell (i, j) is.
__device__ __forceinline__ void cube_source(const Topo& tp, int n, int& t, int& i, int& j) {
  int e, d, s;
  if (i < 1) { e = EW; d = 1 - i; s = j - 1; }
  else if (i > n) { e = EE; d = i - n; s = j - 1; }
  else if (j < 1) { e = ES; d = 1 - j; s = i - 1; }
  else { e = EN; d = j - n; s = i - 1; }
  const int nt = tp.nbr[t][e], ne = tp.nedge[t][e];
  const int sb = tp.rev[t][e] ? n - 1 - s : s;
  switch (ne) {
    case EW: i = d; j = sb + 1; break;
    case EE: i = n + 1 - d; j = sb + 1; break;
    case ES: i = sb + 1; j = d; break;
    default: i = sb + 1; j = n + 1 - d; break;
  }
  t = nt;
}

template <typename T>
__device__ __forceinline__ T load_q(const AdvArgs<T>& a, int t, int iq, int k, int i, int j, int dir) {
  const int n = a.npx - 1;
  const bool out_i = (i < 1) || (i > a.npx - 1), out_j = (j < 1) || (j > a.npy - 1);
  if (out_i && out_j && !a.nested) {
    const int bit = (i < 1 ? 0 : 1) + (j < 1 ? 0 : 2);
    if (a.corners & (1 << bit)) corner_rotate(i, j, a.npx, a.npy, dir);
  }
  if (a.cube && (i < 1 || i > n || j < 1 || j > n) && !(((i < 1) || (i > n)) && ((j < 1) || (j > n))))
    cube_source(a.topo, n, t, i, j);
  // stay inside the data domain; clamped cells feed only discarded outputs
  i = min(max(i, a.pg.isd), a.pg.isd + a.pg.pitch - 1);
  j = min(max(j, a.pg.jsd), a.pg.jsd + a.pg.rows - 1);
  return a.q_in[t * a.sQt + iq * a.sQq + k * a.sQk + a.pg.at(i, j)];
}

template <typename T>
__device__ __forceinline__ T ld_field(const T* base, const PlaneGeom& pg, int i, int j) {
  i = min(max(i, pg.isd), pg.isd + pg.pitch - 1);
  j = min(max(j, pg.jsd), pg.jsd + pg.rows - 1);
  return base[pg.at(i, j)];
}

// ------------------------------------------------------- PPM line stream ---
// Deviations (bl, br) of the four cells e-2..e+1 around a cube-face edge at
// window face e, computed once per line from shared memory: the edge value is
// the mean of the two one-sided, dxa-weighted linear extrapolations; the two
// neighbouring interfaces use one-sided third-order values (see the oracle's
// xppm/yppm restatement).  Only cells 2..29 of a window feed its fluxes.
template <typename T>
struct EdgeDev {
  int e;  // window face of the edge, NO_EDGE if none
  T bl0, bl1, bl2, bl3, br0, br1, br2, br3;
};

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

template <typename T, int HORD, class EX, class ED>
__device__ __noinline__ void edge_devs_impl(int e, EX x, ED ed, T* o) {
  // o[0..3] = bl of cells e-2..e+1, o[4..7] = br
  const bool need0 = (e - 2 >= 2 && e - 2 <= 29), need1 = (e - 1 >= 2 && e - 1 <= 29);
  const bool need2 = (e >= 2 && e <= 29), need3 = (e + 1 >= 2 && e + 1 <= 29);
  T aM = T(0), a0 = T(0), aP = T(0);
  if (need0 || need1) {
    aM = T(-1.0 / 6.0) * x(e - 3) + T(5.0 / 6.0) * x(e - 2) + T(1.0 / 3.0) * x(e - 1);
    if (HORD == 8) aM = clamp2(aM, x(e - 2), x(e - 1));
  }
  if (need1 || need2) {
    T d2 = ed(e - 2), d1 = ed(e - 1), d0 = ed(e), d3 = ed(e + 1);
    T xl = ((T(2) * d1 + d2) * x(e - 1) - d1 * x(e - 2)) / (d2 + d1);
    T xr = ((T(2) * d0 + d3) * x(e) - d0 * x(e + 1)) / (d0 + d3);
    a0 = T(0.5) * (xl + xr);
    if (HORD == 8) a0 = clamp2(a0, x(e - 1), x(e));
  }
  if (need2 || need3) {
    aP = T(1.0 / 3.0) * x(e) + T(5.0 / 6.0) * x(e + 1) - T(1.0 / 6.0) * x(e + 2);
    if (HORD == 8) aP = clamp2(aP, x(e), x(e + 1));
  }
  T b[4] = {T(0), T(0), T(0), T(0)}, r[4] = {T(0), T(0), T(0), T(0)};
  if (need0) { b[0] = generic_bl<T, HORD>(e - 2, x); r[0] = aM - x(e - 2); }
  if (need1) { b[1] = aM - x(e - 1); r[1] = a0 - x(e - 1); }
  if (need2) { b[2] = a0 - x(e); r[2] = aP - x(e); }
  if (need3) { b[3] = aP - x(e + 1); r[3] = generic_br<T, HORD>(e + 1, x); }
  if (HORD == 8)
    for (int c = 0; c < 4; ++c) cw84(b[c], r[c]);
  for (int c = 0; c < 4; ++c) { o[c] = b[c]; o[4 + c] = r[c]; }
}

template <typename T, int HORD, class EX, class ED>
__device__ __forceinline__ EdgeDev<T> edge_devs(int e, EX&& x, ED&& ed) {
  EdgeDev<T> d;
  d.e = e;
  if (e == NO_EDGE) return d;
  T o[8];
  edge_devs_impl<T, HORD>(e, x, ed, o);
  d.bl0 = o[0]; d.bl1 = o[1]; d.bl2 = o[2]; d.bl3 = o[3];
  d.br0 = o[4]; d.br1 = o[5]; d.br2 = o[6]; d.br3 = o[7];
  return d;
}

// A line of 32 window cells x[0..31] marched with a rolling register window;
// face f separates cells f-1 and f, and faces 3..29 are the CTA tile's.
// Before step m the state holds x[m-3..m-1], dm[m-2], al[m-2] and the
// deviations of cell m-3; step(x[m]) finalises cell m-2 and returns the flux
// through face m-2 (meaningful for m >= 5).
template <typename T, int HORD>
struct Line {
  T xa = T(0), xb = T(0), xc = T(0), dmb = T(0), alb = T(0), pbl = T(0), pbr = T(0);

  __device__ __forceinline__ static void splice(int c, const EdgeDev<T>& E, T& bl, T& br) {
    const int d = c - (E.e - 2);
    if (E.e != NO_EDGE && d >= 0 && d <= 3) {
      bl = d == 0 ? E.bl0 : d == 1 ? E.bl1 : d == 2 ? E.bl2 : E.bl3;
      br = d == 0 ? E.br0 : d == 1 ? E.br1 : d == 2 ? E.br2 : E.br3;
    }
  }

  // consume x[m]; return the flux through face m-2 for Courant number c
  __device__ __forceinline__ T step(int m, T x, T c, const EdgeDev<T>& E0, const EdgeDev<T>& E1) {
    T alc, bl, br;
    if (HORD == 8) {
      const T dmc = vl_slope(xb, xc, x);                      // dm[m-1]
      alc = T(0.5) * (xb + xc) + (dmb - dmc) * T(1.0 / 3.0);  // al[m-1]
      const T xt = T(2) * dmb, axt = tabs(xt);                // cell m-2
      bl = -tsign(tmin(axt, tabs(alb - xb)), xt);
      br = tsign(tmin(axt, tabs(alc - xb)), xt);
      dmb = dmc;
    } else {
      alc = T(7.0 / 12.0) * (xb + xc) - T(1.0 / 12.0) * (xa + x);
      bl = alb - xb;
      br = alc - xb;
    }
    splice(m - 2, E0, bl, br);
    splice(m - 2, E1, bl, br);
    const T fl = ppm_flux(c, xa, pbl, pbr, xb, bl, br);
    xa = xb;
    xb = xc;
    xc = x;
    alb = alc;
    pbl = bl;
    pbr = br;
    return fl;
  }
};

// ------------------------------------------------------------ the kernel ---
template <typename T, int HORD, bool FLUXES>
__global__ void __launch_bounds__(256) k_substep(const AdvArgs<T> a) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemLevel<T>& L = *reinterpret_cast<SmemLevel<T>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, W = blockDim.x >> 5;
  SmemWarp<T>& S = reinterpret_cast<SmemWarp<T>*>(smem_raw + sizeof(SmemLevel<T>))[warp];

  const int t = blockIdx.z, k = blockIdx.y;
  const int nbx = (a.ie - a.is + TW) / TW;
  const int i0 = a.is + (blockIdx.x % nbx) * TW, j0 = a.js + (blockIdx.x / nbx) * TW;
  const int ni = min(TW, a.ie - i0 + 1), nj = min(TW, a.je - j0 + 1);
  const PlaneGeom& pg = a.pg;
  const int n = a.npx - 1;

  // window faces of cube-face edges (x: west/east, y: south/north)
  auto inwin = [](int e) { return (e >= 1 && e <= 31) ? e : NO_EDGE; };
  const int exA = (!a.nested && a.is == 1) ? inwin(1 - i0 + 3) : NO_EDGE;
  const int exB = (!a.nested && a.ie + 1 == a.npx) ? inwin(a.npx - i0 + 3) : NO_EDGE;
  const int eyA = (!a.nested && a.js == 1) ? inwin(1 - j0 + 3) : NO_EDGE;
  const int eyB = (!a.nested && a.je + 1 == a.npy) ? inwin(a.npy - j0 + 3) : NO_EDGE;

  // ---------------------------------------------- per-level staging -------
  {
    const long long fo = t * a.sFt + k * a.sFk;
    const T* cx = a.cx + fo;
    const T* cy = a.cy + fo;
    const T* xf = a.xfx + fo;
    const T* yf = a.yfx + fo;
    const T* mx = a.mfx + fo;
    const T* my = a.mfy + fo;
    const T* area = a.area + t * a.sMt;
    const T* rarea = a.rarea + t * a.sMt;
    for (int e = threadIdx.x; e < NF * WIN; e += blockDim.x) {
      const int f = e / WIN, w = e % WIN;
      L.cy[f][w] = ld_field(cy, pg, i0 - 3 + w, j0 + f);
      L.yf[f][w] = ld_field(yf, pg, i0 - 3 + w, j0 + f);
    }
    for (int e = threadIdx.x; e < WIN * NF; e += blockDim.x) {
      const int r = e / NF, f = e % NF;
      L.cx[r][f] = ld_field(cx, pg, i0 + f, j0 - 3 + r);
      L.xf[r][f] = ld_field(xf, pg, i0 + f, j0 - 3 + r);
    }
    for (int e = threadIdx.x; e < TW * NF; e += blockDim.x) {
      const int r = e / NF, f = e % NF;
      L.mx[r][f] = T(0.5) * ld_field(mx, pg, i0 + f, j0 + r);
      const int ff = e / TW, c = e % TW;
      L.my[ff][c] = T(0.5) * ld_field(my, pg, i0 + c, j0 + ff);
    }
    for (int e = threadIdx.x; e < WIN * WIN; e += blockDim.x) {
      const int r = e / WIN, w = e % WIN;
      L.area[r][w] = ld_field(area, pg, i0 - 3 + w, j0 - 3 + r);
    }
    for (int e = threadIdx.x; e < WIN * TW; e += blockDim.x) {
      const int r = e / TW, c = e % TW;
      const int i = i0 + c, j = j0 - 3 + r;
      L.rrx[r][c] = T(1) / (a.ra_x ? ld_field(a.ra_x, pg, i, j)
                                   : ld_field(area, pg, i, j) + ld_field(xf, pg, i, j) - ld_field(xf, pg, i + 1, j));
      const int r2 = e / WIN, w = e % WIN;
      const int i2 = i0 - 3 + w, j2 = j0 + r2;
      L.rry[r2][w] = T(1) / (a.ra_y ? ld_field(a.ra_y, pg, i2, j2)
                                    : ld_field(area, pg, i2, j2) + ld_field(yf, pg, i2, j2) - ld_field(yf, pg, i2, j2 + 1));
    }
    const T* dp1 = a.dp1 ? a.dp1 + fo : nullptr;
    T* dp2o = a.dp2 ? a.dp2 + fo : nullptr;
    for (int e = threadIdx.x; dp1 != nullptr && e < TW * TW; e += blockDim.x) {
      const int r = e / TW, c = e % TW;
      const int i = i0 + c, j = j0 + r;
      const T ra = ld_field(rarea, pg, i, j);
      const T d1 = ld_field(dp1, pg, i, j);
      const T d2 = d1 + (ld_field(mx, pg, i, j) - ld_field(mx, pg, i + 1, j) + ld_field(my, pg, i, j) -
                         ld_field(my, pg, i, j + 1)) * ra;
      L.ua[r][c] = d1 / d2;
      L.ub[r][c] = ra / d2;
      if (r < nj && c < ni && dp2o != nullptr) dp2o[pg.at(i, j)] = d2;
    }
  }
  __syncthreads();

  const bool corner_block = !a.nested && a.corners != 0 &&
                            ((i0 - 3 < 1) || (i0 + 28 > a.npx - 1)) && ((j0 - 3 < 1) || (j0 + 28 > a.npy - 1));
  const bool inside = i0 - 3 >= 1 && i0 + 28 <= n && j0 - 3 >= 1 && j0 + 28 <= n;
  const bool fast = (!a.cube || inside) && !corner_block;
  // edge-flux index (((t*4 + e)*npz + k)*nq + iq)*n + s = efo + e*efe + iq*n + s
  const long long efe = (long long)a.npz * a.nq * n;
  const long long efo = (((long long)t * 4) * a.npz + k) * a.nq * n;

  for (int iq = warp; iq < a.nq; iq += W) {
    // ------------------------------------------ window load (y-sweep corners)
    {
      const int i = i0 - 3 + lane;
      const T* qp = a.q_in + t * a.sQt + iq * a.sQq + k * a.sQk;
#pragma unroll 4
      for (int r = 0; r < WIN; ++r) {
        const int j = j0 - 3 + r;
        S.q[r][lane] = fast ? ld_field(qp, pg, i, j) : load_q(a, t, iq, k, i, j, 2);
      }
    }
    __syncwarp();

    // ------------------------------------------------ S1: inner y, q_i ------
    {
      const int w = lane;
      const T* qcol = &S.q[0][w];
      auto ex = [qcol](int m) { return qcol[m * PQ]; };
      const int ig = i0 - 3 + w;
      const T* dya = a.dya + t * a.sMt;
      auto ed = [dya, pg, ig, j0](int m) { return ld_field(dya, pg, ig, j0 - 3 + m); };
      const EdgeDev<T> EA = edge_devs<T, HORD>(eyA, ex, ed), EB = edge_devs<T, HORD>(eyB, ex, ed);
      Line<T, HORD> ln;
      T fyy_prev = T(0);
#pragma unroll 1
      for (int m = 0; m < WIN; ++m) {
        const int f = m - 2;  // window face of the flux produced now
        const T c = (m >= 5) ? L.cy[f - 3][w] : T(0);
        const T xm1 = ln.xb;  // x[m-2] before the step: the cell below face m-2... (row f-1 = m-3 after)
        (void)xm1;
        const T xrow = ln.xa;  // x[m-3]: row f-1, whose faces are f-1 and f
        const T fy = ln.step(m, qcol[m * PQ], c, EA, EB);
        if (m >= 5) {
          const T fyy = L.yf[f - 3][w] * fy;
          if (w >= 3 && w < 29) S.fy2[f - 3][w - 3] = fy;
          if (m >= 6) {
            const int r = f - 1;
            S.qi[r - 3][w] = (xrow * L.area[r][w] + fyy_prev - fyy) * L.rry[r - 3][w];
          }
          fyy_prev = fyy;
        }
      }
    }
    __syncwarp();

    // -------------------------------------- corner blocks for the x sweeps
    if (corner_block) {
      const int i = i0 - 3 + lane;
#pragma unroll 1
      for (int r = 0; r < WIN; ++r) {
        const int j = j0 - 3 + r;
        const bool oi = (i < 1) || (i > a.npx - 1), oj = (j < 1) || (j > a.npy - 1);
        if (oi && oj) S.q[r][lane] = load_q(a, t, iq, k, i, j, 1);
      }
      __syncwarp();
    }

    // ------------------------------ S2: inner x -> q_j; outer x on q_i -------
    {
      const int r = lane;
      const bool outer = (r >= 3) && (r < 29);
      const int ro = outer ? r - 3 : 0;
      const T* qrow = &S.q[r][0];
      T* qirow = &S.qi[ro][0];
      auto exi = [qrow](int m) { return qrow[m]; };
      auto exo = [qirow](int m) { return qirow[m]; };
      const T* dxa = a.dxa + t * a.sMt;
      const int jg = j0 - 3 + r;
      auto ed = [dxa, pg, i0, jg](int m) { return ld_field(dxa, pg, i0 - 3 + m, jg); };
      const EdgeDev<T> IA = edge_devs<T, HORD>(exA, exi, ed), IB = edge_devs<T, HORD>(exB, exi, ed);
      EdgeDev<T> OA, OB;
      OA.e = NO_EDGE;
      OB.e = NO_EDGE;
      if (outer) {
        OA = edge_devs<T, HORD>(exA, exo, ed);
        OB = edge_devs<T, HORD>(exB, exo, ed);
      }
      Line<T, HORD> li, lo;
      T fxx_prev = T(0), F_prev = T(0);
      const bool efw = a.cube && a.eflux != nullptr && outer && ro < nj;
#pragma unroll 1
      for (int m = 0; m < WIN; ++m) {
        const int f = m - 2;
        const T c = (m >= 5) ? L.cx[r][f - 3] : T(0);
        const T xcol = li.xa;  // x[m-3]: column f-1
        const T fx2 = li.step(m, qrow[m], c, IA, IB);
        const T fo = lo.step(m, qirow[m], c, OA, OB);
        if (m >= 5) {
          const T fxx = L.xf[r][f - 3] * fx2;
          if (m >= 6) {
            const int cc = f - 1;  // window column with both faces
            if (cc >= 3 && cc < 29) S.qj[r][cc - 3] = (xcol * L.area[r][cc] + fxx_prev - fxx) * L.rrx[r][cc - 3];
          }
          fxx_prev = fxx;
          if (outer) {
            const T F = (fo + fx2) * L.mx[ro][f - 3];
            if (FLUXES) {
              qirow[f - 3] = F;  // column f-3 was consumed at step f-3
            } else if (m >= 6) {
              qirow[f - 4] = F_prev - F;  // divergence of interior column f-4
            }
            if (efw) {
              const int fi = i0 + f - 3;  // tile face index
              if (fi == 1) a.eflux[efo + iq * (long long)n + (j0 + ro - 1)] = -F;
              else if (fi == a.npx) a.eflux[efo + efe + iq * (long long)n + (j0 + ro - 1)] = F;
            }
            F_prev = F;
          }
        }
      }
    }
    __syncwarp();

    // ---------------------------- S3: outer y on q_j, update / write -------
    if (lane < TW) {
      const int c = lane;
      const T* qjcol = &S.qj[0][c];
      auto ex = [qjcol](int m) { return qjcol[m * PF]; };
      const T* dya = a.dya + t * a.sMt;
      const int ig = i0 + c;
      auto ed = [dya, pg, ig, j0](int m) { return ld_field(dya, pg, ig, j0 - 3 + m); };
      const EdgeDev<T> EA = edge_devs<T, HORD>(eyA, ex, ed), EB = edge_devs<T, HORD>(eyB, ex, ed);
      Line<T, HORD> ln;
      T* qo = a.q_out + t * a.sQt + iq * a.sQq + k * a.sQk;
      T* fyo = FLUXES ? a.fy_out + (long long)(k * a.nq + iq) * a.sFlux : nullptr;
      T Fprev = T(0);
      const bool efw = a.cube && a.eflux != nullptr && c < ni;
#pragma unroll 1
      for (int m = 0; m < WIN; ++m) {
        const int f = m - 2;
        const T cc = (m >= 5) ? L.cy[f - 3][c + 3] : T(0);
        const T fo = ln.step(m, qjcol[m * PF], cc, EA, EB);
        if (m >= 5) {
          const T F = (fo + S.fy2[f - 3][c]) * L.my[f - 3][c];
          const int fj = j0 + f - 3;  // tile face index
          if (FLUXES) {
            if (c < ni && f - 3 <= nj) fyo[pg.at(ig, fj)] = F;
          } else if (m >= 6) {
            const int ir = f - 4;  // interior row with faces f-1, f
            if (ir < nj && c < ni) {
              const T qn = S.q[ir + 3][c + 3] * L.ua[ir][c] + (S.qi[ir][c] + Fprev - F) * L.ub[ir][c];
              qo[pg.at(ig, j0 + ir)] = qn;
            }
          }
          if (efw) {
            if (fj == 1) a.eflux[efo + 2 * efe + iq * (long long)n + (ig - 1)] = -F;
            else if (fj == a.npy) a.eflux[efo + 3 * efe + iq * (long long)n + (ig - 1)] = F;
          }
          Fprev = F;
        }
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
}

// ------------------------------------------------ tile-edge reconciliation ---
// Every shared tile-edge face carries one flux: the one computed by the tile
// the flow leaves (the upwind tile; the lower-numbered tile when the Courant
// number is zero).  The downwind tile's edge cell was updated with its own
// value; add the difference times rarea/dp2.  Cells at tile corners collect
// both of their edges in the W/E threads.
template <typename T>
__device__ __forceinline__ T edge_correction(const AdvArgs<T>& a, int n, int t, int e, int s, int k, int iq) {
  const int j = s + 1, i = s + 1;
  const T* cx = a.cx + t * a.sFt + k * a.sFk;
  const T* cy = a.cy + t * a.sFt + k * a.sFk;
  T cin;
  switch (e) {
    case EW: cin = cx[a.pg.at(1, j)]; break;
    case EE: cin = -cx[a.pg.at(n + 1, j)]; break;
    case ES: cin = cy[a.pg.at(i, 1)]; break;
    default: cin = -cy[a.pg.at(i, n + 1)]; break;
  }
  const int nt = a.topo.nbr[t][e], ne = a.topo.nedge[t][e];
  if (!(cin > T(0) || (cin == T(0) && nt < t))) return T(0);
  const int sb = a.topo.rev[t][e] ? n - 1 - s : s;
  const T own = a.eflux[((((long long)nt * 4 + ne) * a.npz + k) * a.nq + iq) * n + sb];
  const T mine = a.eflux[((((long long)t * 4 + e) * a.npz + k) * a.nq + iq) * n + s];
  return own + mine;
}

template <typename T>
__global__ void k_edge_fix(const AdvArgs<T> a, int n) {
  const long long tot = (long long)6 * 4 * n;
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= tot) return;
  const int s = (int)(id % n), e = (int)((id / n) % 4), t = (int)(id / (4 * n));
  const int k = blockIdx.y / a.nq, iq = blockIdx.y % a.nq;
  if ((e == ES || e == EN) && (s == 0 || s == n - 1)) return;  // corner cells: W/E threads
  int i, j;
  switch (e) {
    case EW: i = 1; j = s + 1; break;
    case EE: i = n; j = s + 1; break;
    case ES: i = s + 1; j = 1; break;
    default: i = s + 1; j = n; break;
  }
  T corr = edge_correction(a, n, t, e, s, k, iq);
  if (e == EW || e == EE) {
    const int sc = (e == EW) ? 0 : n - 1;
    if (s == 0) corr += edge_correction(a, n, t, ES, sc, k, iq);
    if (s == n - 1) corr += edge_correction(a, n, t, EN, sc, k, iq);
  }
  if (corr == T(0)) return;
  const long long p = a.pg.at(i, j);
  const T ra = a.rarea[t * a.sMt + p];
  const T d2 = a.dp2[t * a.sFt + k * a.sFk + p];
  T* qo = a.q_out + t * a.sQt + iq * a.sQq + k * a.sQk;
  qo[p] += corr * (ra / d2);
}

// ------------------------------------------------------------- prologue ---
// Area fluxes from Courant numbers with the upwind metric, then scaling of
// cx, cy, xfx, yfx, mfx, mfy by 1/nsplt (tracer_2d before its substep loop).
template <typename T>
__global__ void k_area_flux(T* cx, T* cy, T* xfx, T* yfx, T* mfx, T* mfy, const T* dxa, const T* dya,
                            const T* dx, const T* dy, const T* sin_sg, long long sFt, long long sFk,
                            long long sMt, long long sSin, PlaneGeom pg, int is, int ie, int js, int je, T frac) {
  const int t = blockIdx.z, k = blockIdx.y;
  const int nid = pg.pitch;  // loop over the data-domain rectangle of faces
  const int ni = ie - is + 1 + 2 * NG + 1, nj = je - js + 1 + 2 * NG + 1;
  const long long fo = t * sFt + k * sFk;
  const long long mo = t * sMt;
  const T* s_w = sin_sg + t * sMt * 0 + (long long)t * 4 * sSin;  // slots W, S, E, N
  const T* s_s = s_w + sSin;
  const T* s_e = s_w + 2 * sSin;
  const T* s_n = s_w + 3 * sSin;
  (void)nid;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ni * nj; e += gridDim.x * blockDim.x) {
    const int i = pg.isd + e % ni, j = pg.jsd + e / ni;
    const long long p = pg.at(i, j);
    // x faces: i in is..ie+1, rows jsd..jed
    if (i >= is && i <= ie + 1 && j <= je + NG) {
      const T c = cx[fo + p];
      T v;
      if (c > T(0)) v = c * dxa[mo + pg.at(i - 1, j)] * dy[mo + p] * s_e[pg.at(i - 1, j)];
      else v = c * dxa[mo + p] * dy[mo + p] * s_w[p];
      xfx[fo + p] = v * frac;
      cx[fo + p] = c * frac;
      if (j >= js && j <= je) mfx[fo + p] *= frac;
    }
    // y faces: j in js..je+1, cols isd..ied
    if (j >= js && j <= je + 1 && i <= ie + NG) {
      const T c = cy[fo + p];
      T v;
      if (c > T(0)) v = c * dya[mo + pg.at(i, j - 1)] * dx[mo + p] * s_n[pg.at(i, j - 1)];
      else v = c * dya[mo + p] * dx[mo + p] * s_s[p];
      yfx[fo + p] = v * frac;
      cy[fo + p] = c * frac;
      if (i >= is && i <= ie) mfy[fo + p] *= frac;
    }
  }
}

template <typename T>
__global__ void k_max_courant(const T* cx, const T* cy, long long sFt, long long sFk, PlaneGeom pg, int is, int ie,
                              int js, int je, unsigned int* out) {
  const int t = blockIdx.z, k = blockIdx.y;
  const int ni = ie - is + 1, nj = je - js + 1;
  float m = 0.f;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ni * nj; e += gridDim.x * blockDim.x) {
    const int i = is + e % ni, j = js + e / ni;
    const long long p = t * sFt + k * sFk + pg.at(i, j);
    m = fmaxf(m, fmaxf(fabsf((float)cx[p]), fabsf((float)cy[p])));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// ------------------------------------------------------------ launchers ---
template <typename T, int HORD, bool FLUXES>
static int launch_one(const AdvArgs<T>& a, int warps, cudaStream_t s) {
  const size_t smem = substep_smem_bytes(sizeof(T) == 8, warps);
  const int nbx = (a.ie - a.is + TW) / TW, nby = (a.je - a.js + TW) / TW;
  dim3 grid(nbx * nby, a.npz, a.cube ? 6 : 1);
  k_substep<T, HORD, FLUXES><<<grid, 32 * warps, smem, s>>>(a);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

template <typename T, int HORD, bool FLUXES>
static cudaError_t set_smem_attr() {
  const int mx = (int)std::min<size_t>(substep_smem_bytes(sizeof(T) == 8, sizeof(T) == 8 ? 5 : 8), 227 * 1024);
  return cudaFuncSetAttribute(k_substep<T, HORD, FLUXES>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
}

// Raise the dynamic shared-memory limit of every advection kernel once per
// process (before any stream capture).
int prepare_kernels() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    cudaError_t es[] = {set_smem_attr<float, 5, false>(),  set_smem_attr<float, 5, true>(),
                        set_smem_attr<float, 8, false>(),  set_smem_attr<float, 8, true>(),
                        set_smem_attr<double, 5, false>(), set_smem_attr<double, 5, true>(),
                        set_smem_attr<double, 8, false>(), set_smem_attr<double, 8, true>()};
    for (cudaError_t e : es)
      if (e != cudaSuccess && err == cudaSuccess) err = e;
  });
  return err == cudaSuccess ? 0 : cuda_error(err, "cudaFuncSetAttribute(k_substep)");
}

template <typename T>
int launch_substep(const AdvArgs<T>& a, int hord, bool flux_mode, int warps, cudaStream_t s) {
  {
    int prc = prepare_kernels();
    if (prc) return prc;
  }
  if (warps < 1 || warps > 8) return set_error(FV3G_E_ARG, "warps per CTA must be 1..8 (got %d)", warps);
  if (sizeof(T) == 8 && substep_smem_bytes(true, warps) > 227 * 1024)
    return set_error(FV3G_E_ARG, "FP64 advection supports at most %d warps per CTA", 5);
  if (hord == 8) return flux_mode ? launch_one<T, 8, true>(a, warps, s) : launch_one<T, 8, false>(a, warps, s);
  if (hord == 5) return flux_mode ? launch_one<T, 5, true>(a, warps, s) : launch_one<T, 5, false>(a, warps, s);
  return set_error(FV3G_E_UNSUPPORTED, "hord %d not implemented (5 and 8 are)", hord);
}

template <typename T>
int launch_edge_fix(const AdvArgs<T>& a, int n, cudaStream_t s) {
  const long long tot = (long long)6 * 4 * n;
  dim3 grid((unsigned)((tot + 127) / 128), a.npz * a.nq);
  k_edge_fix<T><<<grid, 128, 0, s>>>(a, n);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

template <typename T>
int launch_area_flux(T* cx, T* cy, T* xfx, T* yfx, T* mfx, T* mfy, const T* dxa, const T* dya, const T* dx,
                     const T* dy, const T* sin_sg, long long sFt, long long sFk, long long sMt, long long sSin,
                     PlaneGeom pg, int is, int ie, int js, int je, int ntiles, int npz, T frac, cudaStream_t s) {
  const int ncell = (ie - is + 2 + 2 * NG) * (je - js + 2 + 2 * NG);
  dim3 grid((ncell + 255) / 256, npz, ntiles);
  k_area_flux<T><<<grid, 256, 0, s>>>(cx, cy, xfx, yfx, mfx, mfy, dxa, dya, dx, dy, sin_sg, sFt, sFk, sMt, sSin,
                                      pg, is, ie, js, je, frac);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

template <typename T>
int launch_max_courant(const T* cx, const T* cy, long long sFt, long long sFk, PlaneGeom pg, int is, int ie, int js,
                       int je, int ntiles, int npz, unsigned int* d_out, cudaStream_t s) {
  const int ncell = (ie - is + 1) * (je - js + 1);
  dim3 grid(std::min((ncell + 255) / 256, 64), npz, ntiles);
  k_max_courant<T><<<grid, 256, 0, s>>>(cx, cy, sFt, sFk, pg, is, ie, js, je, d_out);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

#define FV3G_INST(T)                                                                                          \
  template int launch_substep<T>(const AdvArgs<T>&, int, bool, int, cudaStream_t);                          \
  template int launch_edge_fix<T>(const AdvArgs<T>&, int, cudaStream_t);                                     \
  template int launch_area_flux<T>(T*, T*, T*, T*, T*, T*, const T*, const T*, const T*, const T*, const T*, \
                                   long long, long long, long long, long long, PlaneGeom, int, int, int, int, int, \
                                   int, T, cudaStream_t);                                                    \
  template int launch_max_courant<T>(const T*, const T*, long long, long long, PlaneGeom, int, int, int, int, int, \
                                     int, unsigned int*, cudaStream_t);
FV3G_INST(float)
FV3G_INST(double)
#undef FV3G_INST

}  // namespace fv3g
