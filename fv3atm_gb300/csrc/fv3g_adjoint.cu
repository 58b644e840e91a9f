// fv3g_adjoint.cu -- the linearised transport step (fv3g_adjoint.cuh): face
// weights of the PPM sweeps on the trajectory, the tangent-linear substep,
// the hand-written adjoint substep (transposed gathers, corner and halo
// transposes) and the reverse sweep of the kord-4 column remap.
#include <algorithm>

#include "fv3g_adjoint.cuh"
#include "fv3g_dual.cuh"
#include "fv3g_profile.cuh"
#include "fv3g_remap.cuh"
#include "fv3g_stencil.cuh"

namespace fv3g {
namespace {

using D2 = Dual<double>;

// one-sided interface weights at cube-face edges (Putman & Lin 2007)
constexpr double kS11 = 11.0 / 14.0, kS14 = 4.0 / 7.0, kS15 = 3.0 / 14.0;  // hord 8
constexpr double kC1 = -2.0 / 14.0, kC2 = 11.0 / 14.0, kC3 = 5.0 / 14.0;   // hord 1 / 5

// ------------------------------------------------------- face-local PPM ---
// Flux through face f (between cells f-1 and f) of one line, read through
// X(m) for the cells m = f-3..f+2 it depends on, with the cell widths DX(m)
// along the line (one-sided edge values) and the face's Courant number c.
// eLo / eHi: the line's cube-face edge faces (tile interior above eLo, below
// eHi) or NO_EDGE.  The same scheme as the substep kernel's lines:
//   hord 8: monotonized central slopes, interfaces from them, the Lin (2004)
//           limit of the edge deviations; at a cube-face edge the edge value
//           (mean of the two one-sided extrapolations) clamped to the two
//           cells beside it, the next interfaces inward one-sided, the one
//           beyond unlimited, then CW84 on the three edge cells;
//   hord 1 / 5: fourth-order interfaces, one-sided three-cell interfaces
//           beside a cube-face edge and the unlimited edge value; the face
//           takes the first-order upwind value unless a cell beside it
//           passes bl br < 0 (hord 5) or |lim_fac (bl + br)| < |bl - br|
//           (hord 1).
template <typename T, class XF, class DF>
__device__ T ppm_face(int hord, double lim_fac, int f, const XF& X, const DF& DX, double c, int eLo, int eHi) {
  auto edge_mean = [&](int e) -> T {
    const T d2 = T(DX(e - 2)), d1 = T(DX(e - 1)), d0 = T(DX(e)), d3 = T(DX(e + 1));
    const T xl = ((T(2) * d1 + d2) * X(e - 1) - d1 * X(e - 2)) / (d2 + d1);
    const T xr = ((T(2) * d0 + d3) * X(e) - d0 * X(e + 1)) / (d0 + d3);
    return T(0.5) * (xl + xr);
  };
  auto in = [f](int m) { return m == f - 1 || m == f; };
  T bl[2], br[2];  // deviations of cells f-1 and f
  bool smt[2] = {true, true};
  if (hord == 8) {
    // the forms of the substep kernel, so that exact ties (flat lines) take
    // its one-sided derivatives: its line march (clamped slopes, copysign)
    // away from cube-face edges, the generic cell values of its edge windows
    // (cells e-2 .. e+1 of an edge e) beside them
    auto DM = [&](int m) -> T { return vl_slope(X(m - 1), X(m), X(m + 1)); };
    auto AL = [&](int g) -> T { return T(0.5) * (X(g - 1) + X(g)) + (DM(g - 1) - DM(g)) * T(1.0 / 3.0); };
    auto DMC = [&](int m) -> T {
      const T xm = X(m - 1), x0 = X(m), xp = X(m + 1);
      const T xt = T(0.25) * (xp - xm);
      return copysign_t(tmin3(tabs(xt), tmax3(xm, x0, xp) - x0, x0 - tmin3(xm, x0, xp)), xt);
    };
    auto ALC = [&](int g) -> T { return T(0.5) * (X(g - 1) + X(g)) + (DMC(g - 1) - DMC(g)) * T(1.0 / 3.0); };
    auto window = [&](int m) {
      return (eLo != NO_EDGE && m >= eLo - 2 && m <= eLo + 1) || (eHi != NO_EDGE && m >= eHi - 2 && m <= eHi + 1);
    };
    for (int h = 0; h < 2; ++h) {
      const int m = f - 1 + h;
      if (window(m)) {
        const T xt = T(2) * DM(m);
        bl[h] = -tsign(tmin(tabs(xt), tabs(AL(m) - X(m))), xt);
        br[h] = tsign(tmin(tabs(xt), tabs(AL(m + 1) - X(m))), xt);
      } else {
        const T dmm = DMC(m);
        const T xt = dmm + dmm;
        const T axt = tabs(xt);
        bl[h] = copysign_t(tmin(axt, tabs(ALC(m) - X(m))), -xt);
        br[h] = copysign_t(tmin(axt, tabs(ALC(m + 1) - X(m))), xt);
      }
    }
    auto setl = [&](int m, T v) { if (in(m)) bl[m - f + 1] = v; };
    auto setr = [&](int m, T v) { if (in(m)) br[m - f + 1] = v; };
    auto cw = [&](int m) { if (in(m)) cw84(bl[m - f + 1], br[m - f + 1]); };
    if (eLo != NO_EDGE) {
      const int e = eLo;
      const bool cL = in(e - 1), c0 = in(e), cR = in(e + 1);
      if (cL || c0 || cR) {
        T a0 = T(0), ap = T(0);
        if (cL || c0) a0 = clamp2(edge_mean(e), X(e - 1), X(e));
        if (c0 || cR) ap = T(kS15) * X(e) + T(kS11) * X(e + 1) - T(kS14) * DM(e + 1);
        if (cL) {
          setl(e - 1, T(kS14) * DM(e - 2) + T(kS11) * (X(e - 2) - X(e - 1)));
          setr(e - 1, a0 - X(e - 1));
        }
        if (c0) {
          setl(e, a0 - X(e));
          setr(e, ap - X(e));
        }
        if (cR) {
          setl(e + 1, ap - X(e + 1));
          setr(e + 1, AL(e + 2) - X(e + 1));
        }
        cw(e - 1);
        cw(e);
        cw(e + 1);
      }
    }
    if (eHi != NO_EDGE) {
      const int e = eHi;
      const bool cL2 = in(e - 2), cL = in(e - 1), c0 = in(e);
      if (cL2 || cL || c0) {
        T am = T(0), a0 = T(0);
        if (cL2 || cL) am = T(kS15) * X(e - 1) + T(kS11) * X(e - 2) + T(kS14) * DM(e - 2);
        if (cL || c0) a0 = clamp2(edge_mean(e), X(e - 1), X(e));
        if (cL2) {
          setl(e - 2, AL(e - 2) - X(e - 2));
          setr(e - 2, am - X(e - 2));
        }
        if (cL) {
          setl(e - 1, am - X(e - 1));
          setr(e - 1, a0 - X(e - 1));
        }
        if (c0) {
          setl(e, a0 - X(e));
          setr(e, T(kS11) * (X(e + 1) - X(e)) - T(kS14) * DM(e + 1));
        }
        cw(e - 2);
        cw(e - 1);
        cw(e);
      }
    }
  } else {
    auto AL = [&](int g) -> T {
      for (int side = 1; side >= 0; --side) {  // the high edge's one-sided values take precedence
        const int e = side ? eHi : eLo;
        if (e == NO_EDGE) continue;
        if (g == e - 1) return T(kC1) * X(e - 3) + T(kC2) * X(e - 2) + T(kC3) * X(e - 1);
        if (g == e) return edge_mean(e);
        if (g == e + 1) return T(kC3) * X(e) + T(kC2) * X(e + 1) + T(kC1) * X(e + 2);
      }
      return T(7.0 / 12.0) * (X(g - 1) + X(g)) - T(1.0 / 12.0) * (X(g - 2) + X(g + 1));
    };
    for (int h = 0; h < 2; ++h) {
      const int m = f - 1 + h;
      bl[h] = AL(m) - X(m);
      br[h] = AL(m + 1) - X(m);
      if (hord == 5) smt[h] = value_of(bl[h]) * value_of(br[h]) < 0.0;
      else smt[h] = fabs(lim_fac * value_of(bl[h] + br[h])) < fabs(value_of(bl[h] - br[h]));
    }
  }
  const bool high = hord == 8 || smt[0] || smt[1];
  const double ac = fabs(c), w1 = 1.0 - ac, w2 = ac * w1;
  if (c > 0.0) return high ? (X(f - 1) + T(w1) * br[0]) - T(w2) * (bl[0] + br[0]) : X(f - 1);
  return high ? (X(f) + T(w1) * bl[1]) - T(w2) * (bl[1] + br[1]) : X(f);
}

// The six weights of face f's flux on cells f-3..f+2 (one forward-mode pass
// per cell) and the flux value.
template <class XV, class DF>
__device__ __forceinline__ double face_weights(int hord, double lim_fac, int f, const XV& xv, const DF& DX, double c,
                                               int eLo, int eHi, double* w, long long ws) {
  double val = 0.0;
#pragma unroll 1
  for (int s = 0; s < 6; ++s) {
    const int ms = f - 3 + s;
    auto X = [&](int m) -> D2 { return D2(xv(m), m == ms ? 1.0 : 0.0); };
    const D2 r = ppm_face<D2>(hord, lim_fac, f, X, DX, c, eLo, eHi);
    w[s * ws] = r.d;
    val = r.v;
  }
  return val;
}

// ------------------------------------------------------- plane indexing ---
struct Cell {
  int pl, t, k;  // plane, tile, level
  int i, j;      // tile indices
  long long p;   // offset in the plane
  long long q0, lev, met;  // plane offsets: q-shaped arrays, per-level fields, metrics
};

__device__ __forceinline__ bool cell_of(const LinArgs& a, Cell& c) {
  c.p = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c.p >= a.P) return false;
  c.pl = blockIdx.y;
  c.i = a.pg.isd + (int)(c.p % a.pg.pitch);
  c.j = a.pg.jsd + (int)(c.p / a.pg.pitch);
  if (c.i > a.ied || c.j > a.jed) return false;  // plane padding: never read
  const int per_tile = a.nq * a.npz;
  c.t = c.pl / per_tile;
  c.k = c.pl % a.npz;
  c.q0 = (long long)c.pl * a.P;
  c.lev = ((long long)c.t * a.npz + c.k) * a.P;
  c.met = (long long)c.t * a.P;
  return true;
}

__device__ __forceinline__ bool in_rng(int v, int lo, int hi) { return v >= lo && v <= hi; }
__device__ __forceinline__ bool inside_data(const LinArgs& a, int i, int j) {
  return in_rng(i, a.isd, a.ied) && in_rng(j, a.jsd, a.jed);
}
// a cell of a copy_corners block that the sweeps fill
__device__ __forceinline__ bool corner_cell(const LinArgs& a, int i, int j) {
  const bool oi = i < 1 || i > a.npx - 1, oj = j < 1 || j > a.npy - 1;
  if (!(oi && oj)) return false;
  const int bit = (i < 1 ? 0 : 1) + (j < 1 ? 0 : 2);
  return (a.corners >> bit) & 1;
}

__device__ __forceinline__ double ra_y(const LinArgs& a, const Cell& c, int i, int j) {
  const PlaneGeom& pg = a.pg;
  if (a.ra_y) return a.ra_y[c.lev + pg.at(i, j)];
  return a.area[c.met + pg.at(i, j)] + a.yfx[c.lev + pg.at(i, j)] - a.yfx[c.lev + pg.at(i, j + 1)];
}
__device__ __forceinline__ double ra_x(const LinArgs& a, const Cell& c, int i, int j) {
  const PlaneGeom& pg = a.pg;
  if (a.ra_x) return a.ra_x[c.lev + pg.at(i, j)];
  return a.area[c.met + pg.at(i, j)] + a.xfx[c.lev + pg.at(i, j)] - a.xfx[c.lev + pg.at(i + 1, j)];
}

// face ranges of the four sweeps
__device__ __forceinline__ bool yi_face(const LinArgs& a, int i, int j) {  // inner y: every column
  return in_rng(j, a.js, a.je + 1) && in_rng(i, a.isd, a.ied);
}
__device__ __forceinline__ bool xi_face(const LinArgs& a, int i, int j) {  // inner x: every row
  return in_rng(i, a.is, a.ie + 1) && in_rng(j, a.jsd, a.jed);
}
__device__ __forceinline__ bool xo_face(const LinArgs& a, int i, int j) {  // outer x: compute rows
  return in_rng(i, a.is, a.ie + 1) && in_rng(j, a.js, a.je);
}
__device__ __forceinline__ bool yo_face(const LinArgs& a, int i, int j) {  // outer y: compute columns
  return in_rng(j, a.js, a.je + 1) && in_rng(i, a.is, a.ie);
}

// ---------------------------------------------------------- trajectory ---
// The two corner-filled copies of the halo-filled input (copy_corners for x
// and for y sweeps).
__global__ void k_lin_corners(const LinArgs a, const double* q, double* c1, double* c2) {
  Cell c;
  if (!cell_of(a, c)) return;
  const double* qp = q + c.q0;
  if (corner_cell(a, c.i, c.j)) {
    int i1 = c.i, j1 = c.j, i2 = c.i, j2 = c.j;
    corner_rotate(i1, j1, a.npx, a.npy, 1);
    corner_rotate(i2, j2, a.npx, a.npy, 2);
    c1[c.q0 + c.p] = inside_data(a, i1, j1) ? qp[a.pg.at(i1, j1)] : 0.0;
    c2[c.q0 + c.p] = inside_data(a, i2, j2) ? qp[a.pg.at(i2, j2)] : 0.0;
  } else {
    c1[c.q0 + c.p] = qp[c.p];
    c2[c.q0 + c.p] = qp[c.p];
  }
}

// Inner sweeps: y faces for every column of the data domain on the dir-2
// copy, x faces for every row on the dir-1 copy: weights and flux values.
__global__ void k_lin_inner(const LinArgs a, const LinTraj tr) {
  Cell c;
  if (!cell_of(a, c)) return;
  const long long ws = (long long)a.nt * a.nq * a.npz * a.P;
  const PlaneGeom& pg = a.pg;
  double fy = 0.0, fx = 0.0;
  if (yi_face(a, c.i, c.j)) {
    const double* line = tr.qc2 + c.q0;
    const int i = c.i;
    auto xv = [&](int m) { return line[pg.at(i, m)]; };
    auto dx = [&](int m) { return a.dya[c.met + pg.at(i, m)]; };
    fy = face_weights(a.hord, a.lim_fac, c.j, xv, dx, a.cy[c.lev + c.p], a.es, a.en, tr.wyi + c.q0 + c.p, ws);
  } else {
    for (int s = 0; s < 6; ++s) tr.wyi[s * ws + c.q0 + c.p] = 0.0;
  }
  if (xi_face(a, c.i, c.j)) {
    const double* line = tr.qc1 + c.q0;
    const int j = c.j;
    auto xv = [&](int m) { return line[pg.at(m, j)]; };
    auto dx = [&](int m) { return a.dxa[c.met + pg.at(m, j)]; };
    fx = face_weights(a.hord, a.lim_fac, c.i, xv, dx, a.cx[c.lev + c.p], a.ew, a.ee, tr.wxi + c.q0 + c.p, ws);
  } else {
    for (int s = 0; s < 6; ++s) tr.wxi[s * ws + c.q0 + c.p] = 0.0;
  }
  tr.fy2[c.q0 + c.p] = fy;
  tr.fx2[c.q0 + c.p] = fx;
}

// Inner updates: q_i = (q area + yfx fy2 - yfx' fy2') / ra_y on the compute
// rows of every column, q_j likewise along x on the compute columns of every
// row.  The same form maps the tangents.
__global__ void k_lin_mid(const LinArgs a, const double* c1, const double* c2, const double* fx2, const double* fy2,
                          double* qi, double* qj) {
  Cell c;
  if (!cell_of(a, c)) return;
  const int i = c.i, j = c.j;
  const PlaneGeom& pg = a.pg;
  double vi = 0.0, vj = 0.0;
  if (in_rng(j, a.js, a.je)) {
    const double y0 = a.yfx[c.lev + pg.at(i, j)], y1 = a.yfx[c.lev + pg.at(i, j + 1)];
    vi = (c2[c.q0 + c.p] * a.area[c.met + c.p] + y0 * fy2[c.q0 + pg.at(i, j)] - y1 * fy2[c.q0 + pg.at(i, j + 1)]) /
         ra_y(a, c, i, j);
  }
  if (in_rng(i, a.is, a.ie)) {
    const double x0 = a.xfx[c.lev + pg.at(i, j)], x1 = a.xfx[c.lev + pg.at(i + 1, j)];
    vj = (c1[c.q0 + c.p] * a.area[c.met + c.p] + x0 * fx2[c.q0 + pg.at(i, j)] - x1 * fx2[c.q0 + pg.at(i + 1, j)]) /
         ra_x(a, c, i, j);
  }
  qi[c.q0 + c.p] = vi;
  qj[c.q0 + c.p] = vj;
}

// Outer sweeps: x faces of the compute rows on q_i, y faces of the compute
// columns on q_j: weights.
__global__ void k_lin_outer(const LinArgs a, const LinTraj tr) {
  Cell c;
  if (!cell_of(a, c)) return;
  const long long ws = (long long)a.nt * a.nq * a.npz * a.P;
  const PlaneGeom& pg = a.pg;
  if (xo_face(a, c.i, c.j)) {
    const double* line = tr.qi + c.q0;
    const int j = c.j;
    auto xv = [&](int m) { return line[pg.at(m, j)]; };
    auto dx = [&](int m) { return a.dxa[c.met + pg.at(m, j)]; };
    face_weights(a.hord, a.lim_fac, c.i, xv, dx, a.cx[c.lev + c.p], a.ew, a.ee, tr.wxo + c.q0 + c.p, ws);
  } else {
    for (int s = 0; s < 6; ++s) tr.wxo[s * ws + c.q0 + c.p] = 0.0;
  }
  if (yo_face(a, c.i, c.j)) {
    const double* line = tr.qj + c.q0;
    const int i = c.i;
    auto xv = [&](int m) { return line[pg.at(i, m)]; };
    auto dx = [&](int m) { return a.dya[c.met + pg.at(i, m)]; };
    face_weights(a.hord, a.lim_fac, c.j, xv, dx, a.cy[c.lev + c.p], a.es, a.en, tr.wyo + c.q0 + c.p, ws);
  } else {
    for (int s = 0; s < 6; ++s) tr.wyo[s * ws + c.q0 + c.p] = 0.0;
  }
}

// ------------------------------------------------------- tangent-linear ---
// Inner-sweep flux tangents from the corner-filled tangents.
__global__ void k_tl_inner(const LinArgs a, const LinTraj tr, const double* t1, const double* t2, double* fx2,
                           double* fy2) {
  Cell c;
  if (!cell_of(a, c)) return;
  const long long ws = (long long)a.nt * a.nq * a.npz * a.P;
  const PlaneGeom& pg = a.pg;
  double fy = 0.0, fx = 0.0;
  if (yi_face(a, c.i, c.j))
    for (int s = 0; s < 6; ++s) fy += tr.wyi[s * ws + c.q0 + c.p] * t2[c.q0 + pg.at(c.i, c.j - 3 + s)];
  if (xi_face(a, c.i, c.j))
    for (int s = 0; s < 6; ++s) fx += tr.wxi[s * ws + c.q0 + c.p] * t1[c.q0 + pg.at(c.i - 3 + s, c.j)];
  fy2[c.q0 + c.p] = fy;
  fx2[c.q0 + c.p] = fx;
}

// The substep's update of a compute cell from the outer-sweep flux tangents
// (computed here for the cell's four faces) and the inner ones.
__global__ void k_tl_update(const LinArgs a, const LinTraj tr, const double* dq, const double* ti, const double* tj,
                            const double* fx2, const double* fy2, double* out) {
  Cell c;
  if (!cell_of(a, c)) return;
  const long long ws = (long long)a.nt * a.nq * a.npz * a.P;
  const int i = c.i, j = c.j;
  const PlaneGeom& pg = a.pg;
  if (!in_rng(i, a.is, a.ie) || !in_rng(j, a.js, a.je)) {
    out[c.q0 + c.p] = 0.0;
    return;
  }
  auto FX = [&](int f) {
    const long long pf = pg.at(f, j);
    double fo = 0.0;
    for (int s = 0; s < 6; ++s) fo += tr.wxo[s * ws + c.q0 + pf] * ti[c.q0 + pg.at(f - 3 + s, j)];
    return (fo + fx2[c.q0 + pf]) * (0.5 * a.mfx[c.lev + pf]);
  };
  auto FY = [&](int f) {
    const long long pf = pg.at(i, f);
    double fo = 0.0;
    for (int s = 0; s < 6; ++s) fo += tr.wyo[s * ws + c.q0 + pf] * tj[c.q0 + pg.at(i, f - 3 + s)];
    return (fo + fy2[c.q0 + pf]) * (0.5 * a.mfy[c.lev + pf]);
  };
  const double div = FX(i) - FX(i + 1) + FY(j) - FY(j + 1);
  out[c.q0 + c.p] = (dq[c.q0 + c.p] * a.dp1[c.lev + c.p] + div * a.rarea[c.met + c.p]) / a.dp2[c.lev + c.p];
}

// ------------------------------------------------------------- adjoint ---
// Outer-sweep flux adjoints of the substep: with t = q_ad rarea / dp2 on the
// compute cells, FX_ad(f) = t(f) - t(f-1), and both x sweeps' fluxes enter
// FX with 0.5 mfx.
__global__ void k_ad_faces(const LinArgs a, const double* qa, double* gx, double* gy) {
  Cell c;
  if (!cell_of(a, c)) return;
  const int i = c.i, j = c.j;
  const PlaneGeom& pg = a.pg;
  auto tt = [&](int ii, int jj) -> double {
    if (!in_rng(ii, a.is, a.ie) || !in_rng(jj, a.js, a.je)) return 0.0;
    const long long p = pg.at(ii, jj);
    return qa[c.q0 + p] * a.rarea[c.met + p] / a.dp2[c.lev + p];
  };
  double vx = 0.0, vy = 0.0;
  if (xo_face(a, i, j)) vx = 0.5 * a.mfx[c.lev + c.p] * (tt(i, j) - tt(i - 1, j));
  if (yo_face(a, i, j)) vy = 0.5 * a.mfy[c.lev + c.p] * (tt(i, j) - tt(i, j - 1));
  gx[c.q0 + c.p] = vx;
  gy[c.q0 + c.p] = vy;
}

// The same from fv_tp_2d's flux adjoints: g = 0.5 w flux_ad.
__global__ void k_ad_flux_in(const LinArgs a, const double* fxa, const double* fya, double* gx, double* gy) {
  Cell c;
  if (!cell_of(a, c)) return;
  gx[c.q0 + c.p] = xo_face(a, c.i, c.j) ? 0.5 * a.mfx[c.lev + c.p] * fxa[c.q0 + c.p] : 0.0;
  gy[c.q0 + c.p] = yo_face(a, c.i, c.j) ? 0.5 * a.mfy[c.lev + c.p] * fya[c.q0 + c.p] : 0.0;
}

// Outer sweeps transposed: the adjoints of q_i (compute rows, every column)
// and of q_j (compute columns, every row), each cell summing the faces whose
// stencils hold it.
__global__ void k_ad_outer(const LinArgs a, const LinTraj tr, const double* gx, const double* gy, double* ai,
                           double* aj) {
  Cell c;
  if (!cell_of(a, c)) return;
  const long long ws = (long long)a.nt * a.nq * a.npz * a.P;
  const int i = c.i, j = c.j;
  const PlaneGeom& pg = a.pg;
  double vi = 0.0, vj = 0.0;
  if (in_rng(j, a.js, a.je))
    for (int f = max(a.is, i - 2); f <= min(a.ie + 1, i + 3); ++f) {
      const long long pf = pg.at(f, j);
      vi += tr.wxo[(i - f + 3) * ws + c.q0 + pf] * gx[c.q0 + pf];
    }
  if (in_rng(i, a.is, a.ie))
    for (int f = max(a.js, j - 2); f <= min(a.je + 1, j + 3); ++f) {
      const long long pf = pg.at(i, f);
      vj += tr.wyo[(j - f + 3) * ws + c.q0 + pf] * gy[c.q0 + pf];
    }
  ai[c.q0 + c.p] = vi;
  aj[c.q0 + c.p] = vj;
}

// Inner updates transposed, flux part: the adjoints of the inner-sweep
// fluxes (their direct share of FX, FY plus their terms in q_i, q_j).
__global__ void k_ad_mid(const LinArgs a, const double* ai, const double* aj, const double* gx, const double* gy,
                         double* fx2, double* fy2) {
  Cell c;
  if (!cell_of(a, c)) return;
  const int i = c.i, j = c.j;
  const PlaneGeom& pg = a.pg;
  double vy = 0.0, vx = 0.0;
  if (yi_face(a, i, j)) {
    double s = 0.0;
    if (j <= a.je) s += ai[c.q0 + pg.at(i, j)] / ra_y(a, c, i, j);
    if (j - 1 >= a.js) s -= ai[c.q0 + pg.at(i, j - 1)] / ra_y(a, c, i, j - 1);
    vy = a.yfx[c.lev + c.p] * s + (in_rng(i, a.is, a.ie) ? gy[c.q0 + c.p] : 0.0);
  }
  if (xi_face(a, i, j)) {
    double s = 0.0;
    if (i <= a.ie) s += aj[c.q0 + pg.at(i, j)] / ra_x(a, c, i, j);
    if (i - 1 >= a.is) s -= aj[c.q0 + pg.at(i - 1, j)] / ra_x(a, c, i - 1, j);
    vx = a.xfx[c.lev + c.p] * s + (in_rng(j, a.js, a.je) ? gx[c.q0 + c.p] : 0.0);
  }
  fy2[c.q0 + c.p] = vy;
  fx2[c.q0 + c.p] = vx;
}

// Inner sweeps transposed: the adjoints of the two corner-filled copies
// (their area terms in q_i, q_j plus the gathered stencil terms).
__global__ void k_ad_inner(const LinArgs a, const LinTraj tr, const double* ai, const double* aj, const double* fx2,
                           const double* fy2, double* a1, double* a2) {
  Cell c;
  if (!cell_of(a, c)) return;
  const long long ws = (long long)a.nt * a.nq * a.npz * a.P;
  const int i = c.i, j = c.j;
  const PlaneGeom& pg = a.pg;
  double v1 = 0.0, v2 = 0.0;
  if (in_rng(j, a.js, a.je)) v2 = ai[c.q0 + c.p] * a.area[c.met + c.p] / ra_y(a, c, i, j);
  for (int f = max(a.js, j - 2); f <= min(a.je + 1, j + 3); ++f) {
    const long long pf = pg.at(i, f);
    v2 += tr.wyi[(j - f + 3) * ws + c.q0 + pf] * fy2[c.q0 + pf];
  }
  if (in_rng(i, a.is, a.ie)) v1 = aj[c.q0 + c.p] * a.area[c.met + c.p] / ra_x(a, c, i, j);
  for (int f = max(a.is, i - 2); f <= min(a.ie + 1, i + 3); ++f) {
    const long long pf = pg.at(f, j);
    v1 += tr.wxi[(i - f + 3) * ws + c.q0 + pf] * fx2[c.q0 + pf];
  }
  a1[c.q0 + c.p] = v1;
  a2[c.q0 + c.p] = v2;
}

// The input's adjoint before the corner (and halo) transposes: the substep's
// direct term dp1/dp2 on the compute cells (qa, when given) plus both
// copies' adjoints off the filled corner blocks; added to out when acc.
__global__ void k_ad_collect(const LinArgs a, const double* qa, const double* a1, const double* a2, double* out,
                             int acc) {
  Cell c;
  if (!cell_of(a, c)) return;
  double v = 0.0;
  if (qa && in_rng(c.i, a.is, a.ie) && in_rng(c.j, a.js, a.je))
    v = qa[c.q0 + c.p] * a.dp1[c.lev + c.p] / a.dp2[c.lev + c.p];
  if (!corner_cell(a, c.i, c.j)) v += a1[c.q0 + c.p] + a2[c.q0 + c.p];
  out[c.q0 + c.p] = acc ? out[c.q0 + c.p] + v : v;
}

// copy_corners transposed: each filled corner-block cell's adjoint moves to
// the halo-strip cell it was rotated from (one thread per plane and corner;
// the 72 rotation targets of a plane are distinct, so no two threads meet).
__global__ void k_ad_corners(const LinArgs a, const double* a1, const double* a2, double* out) {
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nplanes = (long long)a.nt * a.nq * a.npz;
  if (id >= nplanes * 4) return;
  const long long q0 = (id / 4) * a.P;
  const int corner = (int)(id % 4);
  if (!((a.corners >> corner) & 1)) return;
  const int ib = (corner & 1) ? a.npx : 1 - NG, jb = (corner & 2) ? a.npy : 1 - NG;
  for (int dj = 0; dj < NG; ++dj)
    for (int di = 0; di < NG; ++di) {
      const int i = ib + di, j = jb + dj;
      if (!inside_data(a, i, j)) continue;
      const long long p = a.pg.at(i, j);
      int i1 = i, j1 = j, i2 = i, j2 = j;
      corner_rotate(i1, j1, a.npx, a.npy, 1);
      corner_rotate(i2, j2, a.npx, a.npy, 2);
      if (inside_data(a, i1, j1)) out[q0 + a.pg.at(i1, j1)] += a1[q0 + p];
      if (inside_data(a, i2, j2)) out[q0 + a.pg.at(i2, j2)] += a2[q0 + p];
    }
}

// Cube halo transposed: every interior cell within NG of a tile edge adds the
// adjoints of the halo cells of the neighbouring tiles that copy it; halo
// cells leave with zero.
__global__ void k_ad_halo(const LinArgs a, const double* in, double* out) {
  Cell c;
  if (!cell_of(a, c)) return;
  const int n = a.n, i = c.i, j = c.j;
  if (i < 1 || i > n || j < 1 || j > n) {
    out[c.q0 + c.p] = 0.0;
    return;
  }
  double v = in[c.q0 + c.p];
  const long long per_tile = (long long)a.nq * a.npz;
  const long long within = c.pl - (long long)c.t * per_tile;  // tracer and level inside the tile
  for (int e = 0; e < 4; ++e) {
    int d, sb;
    switch (e) {
      case EW: d = i; sb = j - 1; break;
      case EE: d = n + 1 - i; sb = j - 1; break;
      case ES: d = j; sb = i - 1; break;
      default: d = n + 1 - j; sb = i - 1; break;
    }
    if (d > NG) continue;
    const int u = a.topo.nbr[c.t][e], fe = a.topo.nedge[c.t][e];
    const int su = a.topo.rev[u][fe] ? n - 1 - sb : sb;
    int hi, hj;
    switch (fe) {
      case EW: hi = 1 - d; hj = su + 1; break;
      case EE: hi = n + d; hj = su + 1; break;
      case ES: hi = su + 1; hj = 1 - d; break;
      default: hi = su + 1; hj = n + d; break;
    }
    v += in[((long long)u * per_tile + within) * a.P + a.pg.at(hi, hj)];
  }
  out[c.q0 + c.p] = v;
}

// del-2 damping fluxes transposed (fluxes d6 (q(m-1) - q(m)) through the
// compute faces): q_ad(m) += d6(m+1) F_ad(m+1) - d6(m) F_ad(m) along x and y.
__global__ void k_ad_damp(const LinArgs a, const double* fxa, const double* fya, const double* d6x,
                          const double* d6y, double* out) {
  Cell c;
  if (!cell_of(a, c)) return;
  const int i = c.i, j = c.j;
  const PlaneGeom& pg = a.pg;
  double v = 0.0;
  if (d6x && in_rng(j, a.js, a.je)) {
    if (xo_face(a, i + 1, j)) v += d6x[pg.at(i + 1, j)] * fxa[c.q0 + pg.at(i + 1, j)];
    if (xo_face(a, i, j)) v -= d6x[pg.at(i, j)] * fxa[c.q0 + pg.at(i, j)];
  }
  if (d6y && in_rng(i, a.is, a.ie)) {
    if (yo_face(a, i, j + 1)) v += d6y[pg.at(i, j + 1)] * fya[c.q0 + pg.at(i, j + 1)];
    if (yo_face(a, i, j)) v -= d6y[pg.at(i, j)] * fya[c.q0 + pg.at(i, j)];
  }
  out[c.q0 + c.p] += v;
}

dim3 plane_grid(const LinArgs& a) {
  return dim3((unsigned)((a.P + 127) / 128), (unsigned)(a.nt * a.nq * a.npz));
}

// ------------------------------------------------ remap reverse (kord 4) ---
// One column's source means, slopes, interfaces, the overlap schedule and
// the adjoints, in local memory.
struct ColumnAd {
  double q[KMAX], h[KMAX], d[KMAX], a[KMAX + 1];
  double qa[KMAX], da[KMAX], aa[KMAX + 1];
  double pl[KMAX], pr[KMAX], p6[KMAX];  // adjoints of the layer parabolas (left, right edge, curvature)
  double x[KMAX + 1];
  unsigned char L[KMAX + 1];
};

// d pmean(l, r, s6, x1, x2) / d(l, r, s6), pmean the mean of the layer's
// parabola over the fraction [x1, x2]
__device__ __forceinline__ void pmean_grad(double x1, double x2, double g, double& gl, double& gr, double& g6) {
  const double m = 0.5 * (x1 + x2);
  gl += g * (1.0 - m);
  gr += g * m;
  g6 += g * (m - (x2 * x2 + x1 * x2 + x1 * x1) * (1.0 / 3.0));
}

// Reverse of one column: pe1(k) (k = 0..km) source interface pressures,
// pe2(k) target ones, G2(k2) the target adjoints; leaves the source
// adjoints in C.qa.  C.q holds the source means.
template <class PE1, class PE2, class G2>
__device__ void column_ad4(ColumnAd& C, int km, int kn, int iv, double floor_v, double qs, const PE1& pe1,
                           const PE2& pe2, const G2& g2) {
  // thicknesses and the overlap schedule, as the forward kernel forms them
  {
    double p1 = pe1(0);
    for (int k = 0; k < km; ++k) {
      const double p2 = pe1(k + 1);
      C.h[k] = p2 - p1;
      p1 = p2;
    }
    int k1 = 0;
    double lo = pe1(0), hi = pe1(1);
    for (int k2 = 0; k2 <= kn; ++k2) {
      const double p = pe2(k2);
      while (k1 < km - 1 && hi <= p) {
        ++k1;
        lo = hi;
        hi = pe1(k1 + 1);
      }
      C.L[k2] = (unsigned char)k1;
      C.x[k2] = (p - lo) / (hi - lo);
    }
  }
  auto qf = [&](int k) -> double { return C.q[min(max(k, 0), km - 1)]; };
  auto hf = [&](int k) -> double { return C.h[min(max(k, 0), km - 1)]; };
  for (int k = 0; k < km; ++k) C.d[k] = ppm_slope_f<double>(k, km, qf, hf);
  for (int u = 0; u <= km; ++u)
    C.a[u] = ppm_interface<double>(u, km, iv, qs, u >= 1 ? C.d[u - 1] : 0.0, u < km ? C.d[u] : 0.0, qf, hf);
  for (int k = 0; k < km; ++k) C.qa[k] = C.da[k] = C.pl[k] = C.pr[k] = C.p6[k] = 0.0;
  for (int u = 0; u <= km; ++u) C.aa[u] = 0.0;

  // integration, reversed
  int Lt = C.L[0];
  double Xt = C.x[0];
  for (int k2 = 0; k2 < kn; ++k2) {
    const int Lb = C.L[k2 + 1];
    const double Xb = C.x[k2 + 1];
    const double g = g2(k2);
    const bool inside = (Lb == Lt) || (Lb == Lt + 1 && Xb == 0.0);
    if (inside) {
      if (Xt == 0.0 && (Lb == Lt + 1 || Xb == 1.0)) C.qa[Lt] += g;
      else pmean_grad(Xt, Lb == Lt ? Xb : 1.0, g, C.pl[Lt], C.pr[Lt], C.p6[Lt]);
    } else {
      const double ma = g / (pe2(k2 + 1) - pe2(k2));
      if (Xt == 0.0) C.qa[Lt] += ma * C.h[Lt];
      else pmean_grad(Xt, 1.0, ma * (C.h[Lt] * (1.0 - Xt)), C.pl[Lt], C.pr[Lt], C.p6[Lt]);
      for (int m = Lt + 1; m < Lb; ++m) C.qa[m] += ma * C.h[m];
      if (Xb >= 1.0) C.qa[Lb] += ma * (C.h[Lb] * Xb);
      else if (Xb > 0.0) pmean_grad(0.0, Xb, ma * (C.h[Lb] * Xb), C.pl[Lb], C.pr[Lb], C.p6[Lb]);
    }
    Lt = Lb;
    Xt = Xb;
  }

  // layer parabolas, reversed: local derivatives of the profile with respect
  // to its inputs (neighbour means, the layer's edges and slope)
  for (int k = 0; k < km; ++k) {
    if (C.pl[k] == 0.0 && C.pr[k] == 0.0 && C.p6[k] == 0.0) continue;
    const bool inner = k >= 2 && k <= km - 3;
    for (int s = 0; s < 8; ++s) {
      if (!inner && (s == 0 || s == 1 || s == 3 || s == 4)) continue;
      auto in = [&](int which, double v) { return D2(v, which == s ? 1.0 : 0.0); };
      const double qk = C.q[k];
      const Profile<D2> P = layer_profile<D2, 4>(
          k, km, in(0, inner ? C.q[k - 2] : qk), in(1, inner ? C.q[k - 1] : qk), in(2, qk),
          in(3, inner ? C.q[k + 1] : qk), in(4, inner ? C.q[k + 2] : qk), in(5, C.a[k]), in(6, C.a[k + 1]),
          in(7, C.d[k]), iv, D2(floor_v));
      const double g = C.pl[k] * P.l.d + C.pr[k] * P.r.d + C.p6[k] * P.s6.d;
      if (s <= 4) C.qa[k - 2 + s] += g;
      else if (s == 5) C.aa[k] += g;
      else if (s == 6) C.aa[k + 1] += g;
      else C.da[k] += g;
    }
  }

  // interfaces, reversed: each reads the means of at most three layers and
  // the slopes of the two beside it
  for (int u = 0; u <= km; ++u) {
    const double g = C.aa[u];
    if (g == 0.0) continue;
    int lo, hi;
    if (km == 2) { lo = 0; hi = 1; }
    else if (u <= 1) { lo = 0; hi = 2; }
    else if (u >= km - 1) { lo = km - 3; hi = km - 1; }
    else { lo = u - 1; hi = u; }
    const bool inner = km > 2 && u >= 2 && u <= km - 2;
    for (int s = lo; s <= hi + (inner ? 2 : 0); ++s) {
      const int sq = s <= hi ? s : -1;            // seeded mean
      const int sd = s > hi ? s - hi - 1 : -1;    // seeded slope: 0 left (layer u-1), 1 right (layer u)
      auto qd = [&](int k) -> D2 {
        const int kk = min(max(k, 0), km - 1);
        return D2(C.q[kk], kk == sq ? 1.0 : 0.0);
      };
      auto hd = [&](int k) -> D2 { return D2(C.h[min(max(k, 0), km - 1)]); };
      const D2 dml(u >= 1 ? C.d[u - 1] : 0.0, sd == 0 ? 1.0 : 0.0);
      const D2 dmr(u < km ? C.d[u] : 0.0, sd == 1 ? 1.0 : 0.0);
      const D2 r = ppm_interface<D2>(u, km, iv, D2(qs), dml, dmr, qd, hd);
      if (sq >= 0) C.qa[sq] += g * r.d;
      else if (sd == 0) C.da[u - 1] += g * r.d;
      else C.da[u] += g * r.d;
    }
  }

  // slopes, reversed
  for (int k = 1; k <= km - 2; ++k) {
    const double g = C.da[k];
    if (g == 0.0) continue;
    for (int s = -1; s <= 1; ++s) {
      const D2 r = ppm_slope(D2(C.q[k - 1], s == -1 ? 1.0 : 0.0), D2(C.q[k], s == 0 ? 1.0 : 0.0),
                             D2(C.q[k + 1], s == 1 ? 1.0 : 0.0), D2(C.h[k - 1]), D2(C.h[k]), D2(C.h[k + 1]));
      C.qa[k + s] += g * r.d;
    }
  }
}

// Every interior column and tracer of the state (thread per column and
// tracer): pressures from ptop = ak[0] and the running sum of dp, targets
// ak + bk ps.
__global__ void __launch_bounds__(64) k_remap_ad_state(const double* q, const double* dp, const double* ak,
                                                       const double* bk, const double* q2_ad, double* q_ad,
                                                       PlaneGeom pg, long long P, int n, int nt, int nq, int km,
                                                       int kn, int iv, double floor_v) {
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ncol = (long long)nt * n * n;
  if (id >= ncol * nq) return;
  const int iq = (int)(id / ncol);
  const long long col = id % ncol;
  const int t = (int)(col / ((long long)n * n));
  const int rem = (int)(col % ((long long)n * n));
  const int i = 1 + rem % n, j = 1 + rem / n;
  const long long p = pg.at(i, j);
  ColumnAd C;
  const long long qb = ((long long)t * nq + iq) * km * P + p;
  for (int k = 0; k < km; ++k) C.q[k] = q[qb + (long long)k * P];
  const double* dpc = dp + (long long)t * km * P + p;
  double ps = ak[0];
  for (int k = 0; k < km; ++k) ps += dpc[(long long)k * P];
  // pe1 as the forward kernel accumulates it (ptop, then + dp layer by layer)
  double pe1v[KMAX + 1];
  pe1v[0] = ak[0];
  for (int k = 0; k < km; ++k) pe1v[k + 1] = pe1v[k] + dpc[(long long)k * P];
  auto pe1 = [&](int k) { return pe1v[k]; };
  auto pe2 = [&](int k) { return ak[k] + bk[k] * ps; };
  const long long ob = ((long long)t * nq + iq) * kn * P + p;
  auto g2 = [&](int k2) { return q2_ad[ob + (long long)k2 * P]; };
  column_ad4(C, km, kn, iv, floor_v, 0.0, pe1, pe2, g2);
  for (int k = 0; k < km; ++k) q_ad[qb + (long long)k * P] = C.qa[k];
}

// One row of drop-in columns, [level][column] layout.
__global__ void __launch_bounds__(64) k_remap_ad_rows(const double* q1, const double* pe1, const double* pe2,
                                                      const double* qs, const double* q2_ad, double* q1_ad, int ncol,
                                                      int km, int kn, int iv) {
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  ColumnAd C;
  for (int k = 0; k < km; ++k) C.q[k] = q1[(long long)k * ncol + col];
  auto p1 = [&](int k) { return pe1[(long long)k * ncol + col]; };
  auto p2 = [&](int k) { return pe2[(long long)k * ncol + col]; };
  auto g2 = [&](int k2) { return q2_ad[(long long)k2 * ncol + col]; };
  column_ad4(C, km, kn, iv, 0.0, qs ? qs[col] : 0.0, p1, p2, g2);
  for (int k = 0; k < km; ++k) q1_ad[(long long)k * ncol + col] += C.qa[k];
}

}  // namespace

namespace {
__global__ void k_pack_dual2(Dual<double>* out, const double* v, const double* d, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = Dual<double>(v[i], d ? d[i] : 0.0);
}
__global__ void k_unpack_tangent(const Dual<double>* in, double* d, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    d[i] = in[i].d;
}
unsigned blocks_for(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 8 * 152); }
}  // namespace

int lin_pack_dual(Dual<double>* out, const double* v, const double* d, long long n, cudaStream_t s) {
  k_pack_dual2<<<blocks_for(n), 256, 0, s>>>(out, v, d, n);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

int lin_unpack_tangent(const Dual<double>* in, double* d, long long n, cudaStream_t s) {
  k_unpack_tangent<<<blocks_for(n), 256, 0, s>>>(in, d, n);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

int lin_trajectory(const LinArgs& a, const double* q, const LinTraj& tr, cudaStream_t s) {
  const dim3 g = plane_grid(a);
  k_lin_corners<<<g, 128, 0, s>>>(a, q, tr.qc1, tr.qc2);
  k_lin_inner<<<g, 128, 0, s>>>(a, tr);
  k_lin_mid<<<g, 128, 0, s>>>(a, tr.qc1, tr.qc2, tr.fx2, tr.fy2, tr.qi, tr.qj);
  k_lin_outer<<<g, 128, 0, s>>>(a, tr);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

int lin_substep_tl(const LinArgs& a, const LinTraj& tr, const LinWork& w, const double* dq, double* dq_out,
                   cudaStream_t s) {
  const dim3 g = plane_grid(a);
  k_lin_corners<<<g, 128, 0, s>>>(a, dq, w.a1, w.a2);
  k_tl_inner<<<g, 128, 0, s>>>(a, tr, w.a1, w.a2, w.fx2, w.fy2);
  k_lin_mid<<<g, 128, 0, s>>>(a, w.a1, w.a2, w.fx2, w.fy2, w.ai, w.aj);
  k_tl_update<<<g, 128, 0, s>>>(a, tr, dq, w.ai, w.aj, w.fx2, w.fy2, dq_out);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

int lin_substep_ad(const LinArgs& a, const LinTraj& tr, const LinWork& w, const double* q_ad_out, double* q_ad_in,
                   cudaStream_t s) {
  const dim3 g = plane_grid(a);
  k_ad_faces<<<g, 128, 0, s>>>(a, q_ad_out, w.gx, w.gy);
  k_ad_outer<<<g, 128, 0, s>>>(a, tr, w.gx, w.gy, w.ai, w.aj);
  k_ad_mid<<<g, 128, 0, s>>>(a, w.ai, w.aj, w.gx, w.gy, w.fx2, w.fy2);
  k_ad_inner<<<g, 128, 0, s>>>(a, tr, w.ai, w.aj, w.fx2, w.fy2, w.a1, w.a2);
  // the collected adjoint goes through gx (free after k_ad_mid) before the halo transpose
  k_ad_collect<<<g, 128, 0, s>>>(a, q_ad_out, w.a1, w.a2, w.gx, 0);
  const long long nc = (long long)a.nt * a.nq * a.npz * 4;
  k_ad_corners<<<(unsigned)((nc + 127) / 128), 128, 0, s>>>(a, w.a1, w.a2, w.gx);
  k_ad_halo<<<g, 128, 0, s>>>(a, w.gx, q_ad_in);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

int lin_fluxes_ad(const LinArgs& a, const LinTraj& tr, const LinWork& w, const double* fx_ad, const double* fy_ad,
                  const double* d6x, const double* d6y, double* q_ad, cudaStream_t s) {
  const dim3 g = plane_grid(a);
  k_ad_flux_in<<<g, 128, 0, s>>>(a, fx_ad, fy_ad, w.gx, w.gy);
  k_ad_outer<<<g, 128, 0, s>>>(a, tr, w.gx, w.gy, w.ai, w.aj);
  k_ad_mid<<<g, 128, 0, s>>>(a, w.ai, w.aj, w.gx, w.gy, w.fx2, w.fy2);
  k_ad_inner<<<g, 128, 0, s>>>(a, tr, w.ai, w.aj, w.fx2, w.fy2, w.a1, w.a2);
  k_ad_collect<<<g, 128, 0, s>>>(a, nullptr, w.a1, w.a2, q_ad, 1);
  const long long nc = (long long)a.nt * a.nq * a.npz * 4;
  k_ad_corners<<<(unsigned)((nc + 127) / 128), 128, 0, s>>>(a, w.a1, w.a2, q_ad);
  if (d6x || d6y) k_ad_damp<<<g, 128, 0, s>>>(a, fx_ad, fy_ad, d6x, d6y, q_ad);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

LinArgs lin_state_args(const PlaneGeom& pg, long long P, int n, int nt, int nq, int npz, int hord, double lim_fac,
                       const Topo& topo) {
  LinArgs a{};
  a.pg = pg;
  a.P = P;
  a.is = 1; a.ie = n; a.js = 1; a.je = n;
  a.isd = 1 - NG; a.ied = n + NG; a.jsd = 1 - NG; a.jed = n + NG;
  a.npx = n + 1; a.npy = n + 1;
  a.ew = 1; a.ee = n + 1; a.es = 1; a.en = n + 1;
  a.corners = 15;
  a.n = n; a.nt = nt; a.nq = nq; a.npz = npz;
  a.hord = hord;
  a.lim_fac = lim_fac;
  a.topo = topo;
  return a;
}

int lin_remap_ad(const double* q, const double* dp, const double* ak, const double* bk, const double* q2_ad,
                 double* q_ad, PlaneGeom pg, long long P, int n, int nt, int nq, int km, int kn, int iv,
                 double q_min, int kord, cudaStream_t s) {
  if (kord != 4) return set_error(FV3G_E_UNSUPPORTED, "the hand-written remap adjoint is kord 4 (got %d)", kord);
  if (km < 3 || km > KMAX || kn < 1 || kn > KMAX)
    return set_error(FV3G_E_ARG, "remap adjoint supports 3..%d layers (km=%d, kn=%d)", KMAX, km, kn);
  const long long nthr = (long long)nt * n * n * nq;
  k_remap_ad_state<<<(unsigned)((nthr + 63) / 64), 64, 0, s>>>(q, dp, ak, bk, q2_ad, q_ad, pg, P, n, nt, nq, km, kn,
                                                               iv, iv == 1 ? q_min : 0.0);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

int lin_remap_ad_rows(const double* q1, const double* pe1, const double* pe2, const double* qs, const double* q2_ad,
                      double* q1_ad, int ncol, int km, int kn, int iv, int kord, cudaStream_t s) {
  if (kord != 4) return set_error(FV3G_E_UNSUPPORTED, "the hand-written remap adjoint is kord 4 (got %d)", kord);
  if (km < 3 || km > KMAX || kn < 1 || kn > KMAX)
    return set_error(FV3G_E_ARG, "remap adjoint supports 3..%d layers (km=%d, kn=%d)", KMAX, km, kn);
  k_remap_ad_rows<<<(unsigned)((ncol + 63) / 64), 64, 0, s>>>(q1, pe1, pe2, qs, q2_ad, q1_ad, ncol, km, kn, iv);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

}  // namespace fv3g
