// fv3_oracle.cpp -- FP64 CPU restatement of the FV3 tracer-transport path.
//
// TEST INFRASTRUCTURE ONLY (the oracle the CUDA path is compared with).  See fv3_oracle.h
// for the method references and the parity status (unpinned: the upstream
// Fortran is an empty submodule in the reference tree, .gitmodules:1-4).
//
// The PPM core is a template on the tracer scalar type so that the same code,
// instantiated with a dual number, yields the tangent-linear model with every
// limiter branch frozen at the trajectory.
#include "fv3_oracle.h"

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

namespace {

// ---------------------------------------------------------------- scalars ---
struct Dual {  // value + tangent; comparisons act on the value only
  double v, d;
  Dual() : v(0), d(0) {}
  Dual(double a) : v(a), d(0) {}
  Dual(double a, double b) : v(a), d(b) {}
};
inline Dual operator+(Dual a, Dual b) { return {a.v + b.v, a.d + b.d}; }
inline Dual operator-(Dual a, Dual b) { return {a.v - b.v, a.d - b.d}; }
inline Dual operator-(Dual a) { return {-a.v, -a.d}; }
inline Dual operator*(Dual a, Dual b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
inline Dual operator/(Dual a, Dual b) { return {a.v / b.v, (a.d * b.v - a.v * b.d) / (b.v * b.v)}; }
inline double val(double a) { return a; }
inline double val(const Dual& a) { return a.v; }
// Op-counting scalar (for the flop ceiling of the measurement): every +, -,
// *, / on it and every min / max / sign transfer is tallied in g_ops; a
// negation and |.| are free (operand modifiers on the GPU).  Counting runs
// are single-threaded.
struct OpTally {
  unsigned long long add = 0, mul = 0, div = 0, cmp = 0;
};
OpTally g_ops;
struct Cnt {
  double v;
  Cnt() : v(0) {}
  Cnt(double a) : v(a) {}
};
inline Cnt operator+(Cnt a, Cnt b) { ++g_ops.add; return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { ++g_ops.add; return Cnt(a.v - b.v); }
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
inline Cnt operator*(Cnt a, Cnt b) { ++g_ops.mul; return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { ++g_ops.div; return Cnt(a.v / b.v); }
inline double val(const Cnt& a) { return a.v; }
inline Cnt tmin(Cnt a, Cnt b) { ++g_ops.cmp; return b.v < a.v ? b : a; }
inline Cnt tmax(Cnt a, Cnt b) { ++g_ops.cmp; return b.v > a.v ? b : a; }
inline Cnt tabs(Cnt a) { return a.v < 0 ? Cnt(-a.v) : a; }
inline Cnt tsign(Cnt a, Cnt b) { ++g_ops.cmp; return b.v < 0 ? Cnt(-std::fabs(a.v)) : Cnt(std::fabs(a.v)); }
// ops done on the values of T (limiter tests), tallied for the counting scalar only
template <class T> inline void tally(int, int, int) {}
template <> inline void tally<Cnt>(int add, int mul, int cmp) {
  g_ops.add += add;
  g_ops.mul += mul;
  g_ops.cmp += cmp;
}

template <class T> inline T tmin(T a, T b) { return val(b) < val(a) ? b : a; }
template <class T> inline T tmax(T a, T b) { return val(b) > val(a) ? b : a; }
template <class T> inline T tabs(T a) { return val(a) < 0 ? -a : a; }
// magnitude of a with the sign of b (b == 0 counts as positive)
template <class T> inline T tsign(T a, T b) {
  T m = tabs(a);
  return val(b) < 0 ? -m : m;
}

// ------------------------------------------------------------ array views ---
template <class T>
struct View2 {  // Fortran-style (i,j) view with explicit lower bounds, i fastest
  T* p;
  int ilo, jlo, ni;
  T& operator()(int i, int j) const { return p[(ptrdiff_t)(i - ilo) + (ptrdiff_t)(j - jlo) * ni]; }
};
template <class T> View2<T> v2(T* p, int ilo, int ihi, int jlo) { return View2<T>{p, ilo, jlo, ihi - ilo + 1}; }

// ------------------------------------------------------------ PPM on a line ---
// Colella & Woodward (1984) eq. 1.10 in perturbation form: bl = aL - q,
// br = aR - q.  Flatten a cell that is a local extremum; otherwise move the
// edge value on the overshooting side so that the parabola's extremum sits on
// the opposite edge.
template <class T> inline void cw84(T& bl, T& br) {
  tally<T>(3, 4, 3);  // bl br, 3 (br - bl)(bl + br), (br - bl)^2, the tests and the -2 factor
  if (val(bl) * val(br) >= 0.0) {
    bl = T(0.0);
    br = T(0.0);
    return;
  }
  double t = 3.0 * (val(br) - val(bl)) * (val(bl) + val(br));
  double d2 = (val(br) - val(bl)) * (val(br) - val(bl));
  if (-t > d2) {
    bl = T(-2.0) * br;
  } else if (t > d2) {
    br = T(-2.0) * bl;
  }
}

template <class T> inline T clamp2(T a, T x0, T x1) {  // a into [min(x0,x1), max(x0,x1)]
  T lo = tmin(x0, x1), hi = tmax(x0, x1);
  return tmin(tmax(a, lo), hi);
}

// Fluxes at faces f in [flo, fhi] (face f separates cells f-1 and f).
// x(m) for m in [flo-3, fhi+2] via xs(m) = x[m - (flo-3)]; c[f - flo];
// dxa(m) in the same indexing as x.  eW / eE: the tile-edge face at the low
// end (tile interior above it) / high end (interior below), or kNoEdge.
//   hord 8: monotonized central slope dm, interface al, Lin (2004) limit of
//           the edge deviations to |2 dm|;
//   hord 5: fourth-order interfaces (7/12, -1/12), no limiter, and a 2-dx
//           filter: the parabola's correction is dropped (first-order upwind
//           flux) when both cells beside the face are extrema (bl br >= 0);
//   hord 1: hord 5 with the filter test |lim_fac b0| < |bl - br| (lim_fac 1
//           is hord 5's test, lim_fac 3 the stricter hord-6 one).
constexpr int kNoEdge = -1000000;
constexpr double kS11 = 11.0 / 14.0, kS14 = 4.0 / 7.0, kS15 = 3.0 / 14.0;    // hord 8 edge values
constexpr double kC1 = -2.0 / 14.0, kC2 = 11.0 / 14.0, kC3 = 5.0 / 14.0;    // hord < 8 edge values

template <class T>
void ppm_line(int hord, double lim_fac, const T* x, const double* c, const double* dxa, int flo, int fhi, int eW,
              int eE, T* flux) {
  const int m0 = flo - 3;  // first cell index held in x
  const int ncell = fhi - flo + 6;
  auto X = [&](int m) -> const T& { return x[m - m0]; };
  auto DX = [&](int m) -> double { return dxa[m - m0]; };
  std::vector<T> bl(ncell), br(ncell), al(ncell + 1);
  std::vector<char> smt(ncell, 1);
  auto BL = [&](int m) -> T& { return bl[m - m0]; };
  auto BR = [&](int m) -> T& { return br[m - m0]; };
  auto AL = [&](int f) -> T& { return al[f - m0]; };
  const int lo = flo - 1, hi = fhi;  // cells whose bl/br feed a flux
  auto in_cells = [&](int m) { return m >= lo && m <= hi; };
  auto in_faces = [&](int f) { return f >= lo && f <= hi + 1; };
  // Edge value at a cube-face edge e (Putman & Lin 2007): the mean of the two
  // one-sided, dxa-weighted linear extrapolations from either face.
  auto edge_mean = [&](int e) -> T {
    T extL = ((2.0 * DX(e - 1) + DX(e - 2)) * X(e - 1) - DX(e - 1) * X(e - 2)) / (DX(e - 2) + DX(e - 1));
    T extR = ((2.0 * DX(e) + DX(e + 1)) * X(e) - DX(e) * X(e + 1)) / (DX(e) + DX(e + 1));
    return T(0.5) * (extL + extR);
  };

  if (hord == 8) {
    std::vector<T> dm(ncell);
    auto DM = [&](int m) -> T& { return dm[m - m0]; };
    for (int m = flo - 2; m <= fhi + 1; ++m) {
      // monotonized central slope in half-increment form (Lin et al. 1994)
      T xt = T(0.25) * (X(m + 1) - X(m - 1));
      T smax = tmax(tmax(X(m - 1), X(m)), X(m + 1)) - X(m);
      T smin = X(m) - tmin(tmin(X(m - 1), X(m)), X(m + 1));
      DM(m) = tsign(tmin(tmin(tabs(xt), smax), smin), xt);
    }
    for (int f = flo - 1; f <= fhi + 1; ++f)
      AL(f) = T(0.5) * (X(f - 1) + X(f)) + (DM(f - 1) - DM(f)) * T(1.0 / 3.0);
    for (int m = lo; m <= hi; ++m) {
      // Lin (2004) constraint: |edge deviation| <= |2 dm|, same sign as dm
      T xt = T(2.0) * DM(m);
      BL(m) = -tsign(tmin(tabs(xt), tabs(AL(m) - X(m))), xt);
      BR(m) = tsign(tmin(tabs(xt), tabs(AL(m + 1) - X(m))), xt);
    }
    // Cube-face edges: the edge value clamped to the two cells beside it; the
    // next interfaces inward take a one-sided value from two cells and the
    // slope of the second (s15 q + s11 q' -+ s14 dm'); the interface beyond
    // is left unlimited; then the CW84 constraint on the three edge cells.
    // The same one-sided value serves a halo cell's outer edge, so the two
    // tiles sharing an edge compute the same face values.
    auto set = [&](int m, bool left, T v) {
      if (in_cells(m)) (left ? BL(m) : BR(m)) = v;
    };
    if (eW != kNoEdge) {
      const int e = eW;
      T a0 = clamp2(edge_mean(e), X(e - 1), X(e));
      set(e - 1, true, T(kS14) * DM(e - 2) + T(kS11) * (X(e - 2) - X(e - 1)));
      set(e - 1, false, a0 - X(e - 1));
      set(e, true, a0 - X(e));
      T ap = T(kS15) * X(e) + T(kS11) * X(e + 1) - T(kS14) * DM(e + 1);
      set(e, false, ap - X(e));
      set(e + 1, true, ap - X(e + 1));
      if (in_cells(e + 1)) BR(e + 1) = AL(e + 2) - X(e + 1);
      for (int m = e - 1; m <= e + 1; ++m)
        if (in_cells(m)) cw84(BL(m), BR(m));
    }
    if (eE != kNoEdge) {
      const int e = eE;
      if (in_cells(e - 2)) BL(e - 2) = AL(e - 2) - X(e - 2);
      T am = T(kS15) * X(e - 1) + T(kS11) * X(e - 2) + T(kS14) * DM(e - 2);
      set(e - 2, false, am - X(e - 2));
      set(e - 1, true, am - X(e - 1));
      T a0 = clamp2(edge_mean(e), X(e - 1), X(e));
      set(e - 1, false, a0 - X(e - 1));
      set(e, true, a0 - X(e));
      set(e, false, T(kS11) * (X(e + 1) - X(e)) - T(kS14) * DM(e + 1));
      for (int m = e - 2; m <= e; ++m)
        if (in_cells(m)) cw84(BL(m), BR(m));
    }
  } else {
    for (int f = lo; f <= hi + 1; ++f)
      AL(f) = T(7.0 / 12.0) * (X(f - 1) + X(f)) - T(1.0 / 12.0) * (X(f - 2) + X(f + 1));
    // Cube-face edges: one-sided three-cell interfaces next to the edge
    // (c1, c2, c3) and the edge value itself, unlimited.
    for (int e : {eW, eE}) {
      if (e == kNoEdge) continue;
      if (in_faces(e - 1)) AL(e - 1) = T(kC1) * X(e - 3) + T(kC2) * X(e - 2) + T(kC3) * X(e - 1);
      if (in_faces(e)) AL(e) = edge_mean(e);
      if (in_faces(e + 1)) AL(e + 1) = T(kC3) * X(e) + T(kC2) * X(e + 1) + T(kC1) * X(e + 2);
    }
    for (int m = lo; m <= hi; ++m) {
      BL(m) = AL(m) - X(m);
      BR(m) = AL(m + 1) - X(m);
      if (hord == 5) smt[m - m0] = val(BL(m)) * val(BR(m)) < 0.0;
      else smt[m - m0] = std::fabs(lim_fac * val(BL(m) + BR(m))) < std::fabs(val(BL(m) - BR(m)));
      tally<T>(hord == 5 ? 0 : 2, 1, 1);
    }
  }

  // upwind integral of the sub-grid parabola over the swept fraction
  for (int f = flo; f <= fhi; ++f) {
    double cf = c[f - flo];
    const bool high = hord == 8 || smt[f - 1 - m0] || smt[f - m0];
    tally<T>(1, 0, 1);  // 1 -+ c and the upwind selection
    if (cf > 0.0) {
      T b0 = BL(f - 1) + BR(f - 1);
      flux[f - flo] = high ? X(f - 1) + T(1.0 - cf) * (BR(f - 1) - T(cf) * b0) : X(f - 1);
    } else {
      T b0 = BL(f) + BR(f);
      flux[f - flo] = high ? X(f) + T(1.0 + cf) * (BL(f) + T(cf) * b0) : X(f);
    }
  }
}

// ---------------------------------------------------------------- corners ---
// The ng x ng halo block at a cube corner has no cells of its own (three faces
// meet there).  For a sweep along x the block continues the rows of the halo
// strip beside it in y; for a sweep along y it continues the columns of the
// strip beside it in x.  Each corner cell takes the value found by rotating it
// by +-90 degrees about the cube-corner point into that strip.
template <class T>
void copy_corners_t(T* q, int npx, int npy, int dir, const orc_grid* g, const orc_bounds* bd) {
  if (g->nested) return;
  View2<T> Q = v2(q, bd->isd, bd->ied, bd->jsd);
  const int ng = bd->ng;
  struct Corner { int on; double cx, cy; int su, sv; };  // corner point and quadrant signs
  const Corner cs[4] = {
      {g->sw_corner, 0.5, 0.5, -1, -1},
      {g->se_corner, npx - 0.5, 0.5, +1, -1},
      {g->nw_corner, 0.5, npy - 0.5, -1, +1},
      {g->ne_corner, npx - 0.5, npy - 0.5, +1, +1},
  };
  for (const Corner& k : cs) {
    if (!k.on) continue;
    // source quadrant: same u-sign for x sweeps (the strip beside it in y),
    // same v-sign for y sweeps (the strip beside it in x)
    int tu = (dir == 1) ? k.su : -k.su;
    int tv = (dir == 1) ? -k.sv : k.sv;
    for (int a = 1; a <= ng; ++a)
      for (int b = 1; b <= ng; ++b) {
        double u = k.su * (a - 0.5), v = k.sv * (b - 0.5);
        double uu, vv;
        // rotation +90: (u,v)->(-v,u); rotation -90: (u,v)->(v,-u)
        if ((-v > 0) == (tu > 0) && (u > 0) == (tv > 0)) { uu = -v; vv = u; }
        else { uu = v; vv = -u; }
        int i = (int)std::lround(k.cx + u), j = (int)std::lround(k.cy + v);
        int is = (int)std::lround(k.cx + uu), js = (int)std::lround(k.cy + vv);
        Q(i, j) = Q(is, js);
      }
  }
}

// ---------------------------------------------------------------- sweeps ---
// x sweep: fluxes at faces [bd->is, bd->ie+1] for rows [j1, j2].
template <class T>
void xppm_t(T* flux /*(is:ie+1, j1:j2)*/, const T* q /*(isd:ied,jsd:jed)*/, const double* c /*(is:ie+1, clo..)*/,
            int cjlo, int hord, double lim_fac, int j1, int j2, int npx, const orc_grid* g, const orc_bounds* bd) {
  const int is = bd->is, ie = bd->ie;
  View2<const T> Q{q, bd->isd, bd->jsd, bd->ied - bd->isd + 1};
  View2<const double> C{c, is, cjlo, ie - is + 2};
  View2<const double> DXA{g->dxa, bd->isd, bd->jsd, bd->ied - bd->isd + 1};
  View2<T> F{flux, is, j1, ie - is + 2};
  int eW = (!g->nested && is == 1) ? 1 : kNoEdge;
  int eE = (!g->nested && ie + 1 == npx) ? npx : kNoEdge;
  std::vector<T> line(ie - is + 7), out(ie - is + 2);
  std::vector<double> cl(ie - is + 2), dl(ie - is + 7);
  for (int j = j1; j <= j2; ++j) {
    for (int m = is - 3; m <= ie + 3; ++m) { line[m - is + 3] = Q(m, j); dl[m - is + 3] = DXA(m, j); }
    for (int f = is; f <= ie + 1; ++f) cl[f - is] = C(f, j);
    ppm_line<T>(hord, lim_fac, line.data(), cl.data(), dl.data(), is, ie + 1, eW, eE, out.data());
    for (int f = is; f <= ie + 1; ++f) F(f, j) = out[f - is];
  }
}

// y sweep: fluxes at faces [bd->js, bd->je+1] for columns [i1, i2].
template <class T>
void yppm_t(T* flux /*(i1:i2, js:je+1)*/, const T* q, const double* c /*(cilo.., js:je+1)*/, int cilo,
            int cni, int hord, double lim_fac, int i1, int i2, int npy, const orc_grid* g, const orc_bounds* bd) {
  const int js = bd->js, je = bd->je;
  View2<const T> Q{q, bd->isd, bd->jsd, bd->ied - bd->isd + 1};
  View2<const double> C{c, cilo, js, cni};
  View2<const double> DYA{g->dya, bd->isd, bd->jsd, bd->ied - bd->isd + 1};
  View2<T> F{flux, i1, js, i2 - i1 + 1};
  int eS = (!g->nested && js == 1) ? 1 : kNoEdge;
  int eN = (!g->nested && je + 1 == npy) ? npy : kNoEdge;
  std::vector<T> line(je - js + 7), out(je - js + 2);
  std::vector<double> cl(je - js + 2), dl(je - js + 7);
  for (int i = i1; i <= i2; ++i) {
    for (int m = js - 3; m <= je + 3; ++m) { line[m - js + 3] = Q(i, m); dl[m - js + 3] = DYA(i, m); }
    for (int f = js; f <= je + 1; ++f) cl[f - js] = C(i, f);
    ppm_line<T>(hord, lim_fac, line.data(), cl.data(), dl.data(), js, je + 1, eS, eN, out.data());
    for (int f = js; f <= je + 1; ++f) F(i, f) = out[f - js];
  }
}

struct Dom {  // convenience sizes of one domain
  int is, ie, js, je, isd, ied, jsd, jed, nid, njd;
  size_t plane, nxf, nyf, nmx, nmy;
  explicit Dom(const orc_bounds* b)
      : is(b->is), ie(b->ie), js(b->js), je(b->je), isd(b->isd), ied(b->ied), jsd(b->jsd), jed(b->jed) {
    nid = ied - isd + 1;
    njd = jed - jsd + 1;
    plane = (size_t)nid * njd;
    nxf = (size_t)(ie - is + 2) * njd;           // cx, xfx
    nyf = (size_t)nid * (je - js + 2);           // cy, yfx
    nmx = (size_t)(ie - is + 2) * (je - js + 1); // mfx, fx
    nmy = (size_t)(ie - is + 1) * (je - js + 2); // mfy, fy
  }
};

// ---------------------------------------------------------- tracer damping ---
// deln_flux: del-2(nord+1) damping fluxes added to fx, fy.  nord = 0 is a del-2
// flux of the field (del6_v / del6_u times the difference across the face);
// every further order takes the flux divergence times rarea as the new field
// and differences it again with the opposite sign, so the added flux always
// damps.  copy_corners fills the field's cube-corner blocks before each
// direction when nord > 0.  With mass, the field is q and the face flux is
// scaled by damp times the face mean of mass; without, the field is damp q.
template <class T>
void deln_flux_t(int nord, int npx, int npy, double damp, const T* q, T* fx, T* fy, const orc_grid* g,
                 const orc_bounds* bd, const double* mass) {
  Dom d(bd);
  const int is = d.is, ie = d.ie, js = d.js, je = d.je, isd = d.isd, jsd = d.jsd, nid = d.nid;
  View2<const T> Q{q, isd, jsd, nid};
  View2<const double> RAREA{g->rarea, isd, jsd, nid};
  View2<const double> D6U{g->del6_u, isd, jsd, nid};      // (isd:ied, jsd:jed+1)
  View2<const double> D6V{g->del6_v, isd, jsd, nid + 1};  // (isd:ied+1, jsd:jed)
  std::vector<T> d2v(d.plane), fx2v((size_t)(nid + 1) * d.njd), fy2v((size_t)nid * (d.njd + 1));
  View2<T> D2{d2v.data(), isd, jsd, nid};
  View2<T> FX2{fx2v.data(), isd, jsd, nid + 1};
  View2<T> FY2{fy2v.data(), isd, jsd, nid};
  for (int j = js - 1 - nord; j <= je + 1 + nord; ++j)
    for (int i = is - 1 - nord; i <= ie + 1 + nord; ++i) D2(i, j) = mass ? Q(i, j) : T(damp) * Q(i, j);
  if (nord > 0) copy_corners_t<T>(d2v.data(), npx, npy, 1, g, bd);
  for (int j = js - nord; j <= je + nord; ++j)
    for (int i = is - nord; i <= ie + nord + 1; ++i) FX2(i, j) = T(D6V(i, j)) * (D2(i - 1, j) - D2(i, j));
  if (nord > 0) copy_corners_t<T>(d2v.data(), npx, npy, 2, g, bd);
  for (int j = js - nord; j <= je + nord + 1; ++j)
    for (int i = is - nord; i <= ie + nord; ++i) FY2(i, j) = T(D6U(i, j)) * (D2(i, j - 1) - D2(i, j));
  for (int n = 1; n <= nord; ++n) {
    const int nt = nord - n;
    for (int j = js - nt - 1; j <= je + nt + 1; ++j)
      for (int i = is - nt - 1; i <= ie + nt + 1; ++i)
        D2(i, j) = (FX2(i, j) - FX2(i + 1, j) + FY2(i, j) - FY2(i, j + 1)) * T(RAREA(i, j));
    copy_corners_t<T>(d2v.data(), npx, npy, 1, g, bd);
    for (int j = js - nt; j <= je + nt; ++j)
      for (int i = is - nt; i <= ie + nt + 1; ++i) FX2(i, j) = T(D6V(i, j)) * (D2(i, j) - D2(i - 1, j));
    copy_corners_t<T>(d2v.data(), npx, npy, 2, g, bd);
    for (int j = js - nt; j <= je + nt + 1; ++j)
      for (int i = is - nt; i <= ie + nt; ++i) FY2(i, j) = T(D6U(i, j)) * (D2(i, j) - D2(i, j - 1));
  }
  View2<T> FX{fx, is, js, ie - is + 2};
  View2<T> FY{fy, is, js, ie - is + 1};
  if (mass) {
    View2<const double> M{mass, isd, jsd, nid};
    const double damp2 = 0.5 * damp;
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie + 1; ++i) FX(i, j) = FX(i, j) + T(damp2 * (M(i - 1, j) + M(i, j))) * FX2(i, j);
    for (int j = js; j <= je + 1; ++j)
      for (int i = is; i <= ie; ++i) FY(i, j) = FY(i, j) + T(damp2 * (M(i, j - 1) + M(i, j))) * FY2(i, j);
  } else {
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie + 1; ++i) FX(i, j) = FX(i, j) + FX2(i, j);
    for (int j = js; j <= je + 1; ++j)
      for (int i = is; i <= ie; ++i) FY(i, j) = FY(i, j) + FY2(i, j);
  }
}

// damp = (damp_c da_min)^(nord+1), as a product
inline double damp_coefficient(double damp_c, double da_min, int nord) {
  const double b = damp_c * da_min;
  double r = b;
  for (int n = 0; n < nord; ++n) r *= b;
  return r;
}

// fv_tp_2d: Lin & Rood inner/outer operators.  q's corner halo is modified.
// Damping (deln_flux) is added when damp_c > 1e-4: with mass fluxes only if
// mass is given (mass-weighted), without them unweighted.
template <class T>
void fv_tp_2d_t(T* q, const double* crx, const double* cry, int npx, int npy, int hord, T* fx, T* fy,
                const double* xfx, const double* yfx, const orc_grid* g, const orc_bounds* bd,
                const double* ra_x, const double* ra_y, double lim_fac, const double* mfx, const double* mfy,
                const double* mass, int nord, double damp_c) {
  const int is = bd->is, ie = bd->ie, js = bd->js, je = bd->je;
  const int isd = bd->isd, ied = bd->ied, jsd = bd->jsd, jed = bd->jed;
  const int nid = ied - isd + 1;
  View2<T> Q{q, isd, jsd, nid};
  View2<const double> AREA{g->area, isd, jsd, nid};
  View2<const double> XFX{xfx, is, jsd, ie - is + 2};
  View2<const double> YFX{yfx, isd, js, nid};
  View2<const double> RAX{ra_x, is, jsd, ie - is + 1};
  View2<const double> RAY{ra_y, isd, js, nid};

  // inner y operator on every column of the data domain, then outer x
  copy_corners_t<T>(q, npx, npy, 2, g, bd);
  std::vector<T> fy2((size_t)nid * (je - js + 2));
  yppm_t<T>(fy2.data(), q, cry, isd, nid, hord, lim_fac, isd, ied, npy, g, bd);
  View2<T> FY2{fy2.data(), isd, js, nid};
  std::vector<T> qi((size_t)nid * (jed - jsd + 1));
  View2<T> QI{qi.data(), isd, jsd, nid};
  for (int j = js; j <= je; ++j)
    for (int i = isd; i <= ied; ++i)
      QI(i, j) = (Q(i, j) * T(AREA(i, j)) + T(YFX(i, j)) * FY2(i, j) - T(YFX(i, j + 1)) * FY2(i, j + 1)) /
                 T(RAY(i, j));
  xppm_t<T>(fx, qi.data(), crx, jsd, hord, lim_fac, js, je, npx, g, bd);

  // inner x operator on every row of the data domain, then outer y
  copy_corners_t<T>(q, npx, npy, 1, g, bd);
  std::vector<T> fx2((size_t)(ie - is + 2) * (jed - jsd + 1));
  xppm_t<T>(fx2.data(), q, crx, jsd, hord, lim_fac, jsd, jed, npx, g, bd);
  View2<T> FX2{fx2.data(), is, jsd, ie - is + 2};
  std::vector<T> qj((size_t)nid * (jed - jsd + 1));
  View2<T> QJ{qj.data(), isd, jsd, nid};
  for (int j = jsd; j <= jed; ++j)
    for (int i = is; i <= ie; ++i)
      QJ(i, j) = (Q(i, j) * T(AREA(i, j)) + T(XFX(i, j)) * FX2(i, j) - T(XFX(i + 1, j)) * FX2(i + 1, j)) /
                 T(RAX(i, j));
  yppm_t<T>(fy, qj.data(), cry, isd, nid, hord, lim_fac, is, ie, npy, g, bd);

  View2<T> FX{fx, is, js, ie - is + 2};
  View2<T> FY{fy, is, js, ie - is + 1};
  for (int j = js; j <= je; ++j)
    for (int i = is; i <= ie + 1; ++i) {
      double w = mfx ? View2<const double>{mfx, is, js, ie - is + 2}(i, j) : XFX(i, j);
      FX(i, j) = T(0.5) * (FX(i, j) + FX2(i, j)) * T(w);
    }
  for (int j = js; j <= je + 1; ++j)
    for (int i = is; i <= ie; ++i) {
      double w = mfy ? View2<const double>{mfy, is, js, ie - is + 1}(i, j) : YFX(i, j);
      FY(i, j) = T(0.5) * (FY(i, j) + FY2(i, j)) * T(w);
    }
  if (damp_c > 1e-4 && (mfx == nullptr || mass != nullptr))
    deln_flux_t<T>(nord, npx, npy, damp_coefficient(damp_c, g->da_min, nord), q, fx, fy, g, bd,
                   mfx ? mass : nullptr);
}

// --------------------------------------------------------- tracer_2d parts ---
struct Level {  // per-level work arrays of tracer_2d
  std::vector<double> xfx, yfx, rax, ray, dp2;
};

// Area fluxes from Courant numbers (upwind metric), as tracer_2d does.
void area_fluxes(const double* cx, const double* cy, double* xfx, double* yfx, const orc_grid* g,
                 const orc_bounds* bd) {
  const int is = bd->is, ie = bd->ie, js = bd->js, je = bd->je;
  const int isd = bd->isd, ied = bd->ied, jsd = bd->jsd, jed = bd->jed;
  const int nid = ied - isd + 1;
  View2<const double> DXA{g->dxa, isd, jsd, nid}, DYA{g->dya, isd, jsd, nid};
  View2<const double> DX{g->dx, isd, jsd, nid}, DY{g->dy, isd, jsd, nid + 1};
  const size_t plane = (size_t)nid * (jed - jsd + 1);
  auto SIN = [&](int i, int j, int s) { return g->sin_sg[(size_t)(s - 1) * plane + (i - isd) + (size_t)(j - jsd) * nid]; };
  View2<const double> CX{cx, is, jsd, ie - is + 2}, CY{cy, isd, js, nid};
  View2<double> XF{xfx, is, jsd, ie - is + 2}, YF{yfx, isd, js, nid};
  for (int j = jsd; j <= jed; ++j)
    for (int i = is; i <= ie + 1; ++i) {
      double c = CX(i, j);
      XF(i, j) = c > 0.0 ? c * DXA(i - 1, j) * DY(i, j) * SIN(i - 1, j, 3) : c * DXA(i, j) * DY(i, j) * SIN(i, j, 1);
    }
  for (int j = js; j <= je + 1; ++j)
    for (int i = isd; i <= ied; ++i) {
      double c = CY(i, j);
      YF(i, j) = c > 0.0 ? c * DYA(i, j - 1) * DX(i, j) * SIN(i, j - 1, 4) : c * DYA(i, j) * DX(i, j) * SIN(i, j, 2);
    }
}


double max_courant(const double* cx, const double* cy, const Dom& d, int npz) {
  double cmax = 0.0;
  for (int k = 0; k < npz; ++k) {
    View2<const double> CX{cx + k * d.nxf, d.is, d.jsd, d.ie - d.is + 2};
    View2<const double> CY{cy + k * d.nyf, d.isd, d.js, d.nid};
    for (int j = d.js; j <= d.je; ++j)
      for (int i = d.is; i <= d.ie; ++i) cmax = std::max(cmax, std::max(std::fabs(CX(i, j)), std::fabs(CY(i, j))));
  }
  return cmax;
}

void scale_fluxes(double* mfx, double* mfy, double* cx, double* cy, const Dom& d, int npz, double frac) {
  for (size_t n = 0; n < d.nxf * npz; ++n) cx[n] *= frac;
  for (size_t n = 0; n < d.nyf * npz; ++n) cy[n] *= frac;
  for (size_t n = 0; n < d.nmx * npz; ++n) mfx[n] *= frac;
  for (size_t n = 0; n < d.nmy * npz; ++n) mfy[n] *= frac;
}

// dp2, ra_x, ra_y of level k
void level_setup(Level& L, const double* dp1k, const double* mfxk, const double* mfyk, const orc_grid* g,
                 const Dom& d) {
  View2<const double> AREA{g->area, d.isd, d.jsd, d.nid}, RAREA{g->rarea, d.isd, d.jsd, d.nid};
  View2<const double> XF{L.xfx.data(), d.is, d.jsd, d.ie - d.is + 2}, YF{L.yfx.data(), d.isd, d.js, d.nid};
  View2<const double> MX{mfxk, d.is, d.js, d.ie - d.is + 2}, MY{mfyk, d.is, d.js, d.ie - d.is + 1};
  View2<const double> DP{dp1k, d.isd, d.jsd, d.nid};
  L.rax.assign((size_t)(d.ie - d.is + 1) * d.njd, 0.0);
  L.ray.assign((size_t)d.nid * (d.je - d.js + 1), 0.0);
  L.dp2.assign(d.plane, 0.0);
  View2<double> RX{L.rax.data(), d.is, d.jsd, d.ie - d.is + 1}, RY{L.ray.data(), d.isd, d.js, d.nid};
  View2<double> D2{L.dp2.data(), d.isd, d.jsd, d.nid};
  for (int j = d.js; j <= d.je; ++j)
    for (int i = d.is; i <= d.ie; ++i)
      D2(i, j) = DP(i, j) + (MX(i, j) - MX(i + 1, j) + MY(i, j) - MY(i, j + 1)) * RAREA(i, j);
  for (int j = d.jsd; j <= d.jed; ++j)
    for (int i = d.is; i <= d.ie; ++i) RX(i, j) = AREA(i, j) + XF(i, j) - XF(i + 1, j);
  for (int j = d.js; j <= d.je; ++j)
    for (int i = d.isd; i <= d.ied; ++i) RY(i, j) = AREA(i, j) + YF(i, j) - YF(i, j + 1);
}

// flux-form update of the compute domain
void flux_update(double* qk, const double* dp1k, const Level& L, const double* fx, const double* fy,
                 const orc_grid* g, const Dom& d) {
  View2<double> Q{qk, d.isd, d.jsd, d.nid};
  View2<const double> DP{dp1k, d.isd, d.jsd, d.nid}, D2{L.dp2.data(), d.isd, d.jsd, d.nid};
  View2<const double> RAREA{g->rarea, d.isd, d.jsd, d.nid};
  View2<const double> FX{fx, d.is, d.js, d.ie - d.is + 2}, FY{fy, d.is, d.js, d.ie - d.is + 1};
  for (int j = d.js; j <= d.je; ++j)
    for (int i = d.is; i <= d.ie; ++i)
      Q(i, j) = (Q(i, j) * DP(i, j) + (FX(i, j) - FX(i + 1, j) + FY(i, j) - FY(i, j + 1)) * RAREA(i, j)) / D2(i, j);
}

// ------------------------------------------------------------------ remap ---
// Column reconstruction: the sub-grid parabola (aL, aR, a6) of every source
// layer, in the two families of fv_mapz.
//
// kord >= 7 (cs_profile).  Interface values come from the C1 ("cubic-spline")
// condition: the sub-grid parabolas of adjacent layers have equal slopes at
// their shared interface, which on layers of thickness h_{k-1}, h_k gives
//   a_{k-1} + 2(1+d) a_k + d a_{k+1} = 3 (q_{k-1} + d q_k),   d = h_{k-1}/h_k.
// The top and bottom rows require the outermost interface pair to agree with
// one parabola through the two outermost layer means (exact for quadratics).
// iv == -2 replaces the bottom row by a_km = qs.  The kord 9 constraints,
// restated from Lin (2004), the FV3 documentation (Harris et al. 2021) and
// Huynh's second constraint (Suresh & Huynh 1997), with D_u = q_u - q_{u-1}
// the jump of the layer means across interface u:
//   interfaces 1..km-1, with extremum detection: where the neighbouring jumps
//     D_{u-1} and D_{u+1} have one sign (a monotone stretch) the value is
//     clamped into the range of its two layer means; next to a local maximum
//     (D_{u-1} > 0, D_{u+1} <= 0) it is only kept at or above the smaller
//     mean, next to a local minimum only at or below the larger one (and at
//     or above the floor for iv >= 0).  At u = 1 and u = km-1 the missing
//     jump is the one across u itself.  The outermost interfaces are clamped
//     into the range of the two outermost means (not a_km when iv == -2);
//   layers: the two at each end take the CW84 constraint; an interior layer
//     that is a local extremum beside another one (a two-grid-length wave) is
//     flattened; otherwise, when its parabola has an interior extremum
//     (|a6| > |aR - aL|), the right edge is bounded to the range of q,
//     q + 2 D_k and q + 2 D_k - 1.5 D_{k-1} (upper-limit and large-curvature
//     values) and the left edge to the range of q, q - 2 D_{k+1} and
//     q - 2 D_{k+1} + 1.5 D_{k+2}.
//
// kord < 7 (ppm_profile).  Slopes of Colella & Woodward (1984) eq. 1.7 on the
// layer thicknesses, as half increments dm limited by the range of the layer
// and its two neighbours (Lin et al. 1994; dm = 0 in the end layers);
// interfaces 2..km-2 from CW84 eq. 1.6 with the limited slopes; interfaces 1
// and km-1 from the parabola through the three nearest layer means (exact
// for quadratic profiles), clamped into the range of their two means; the
// outermost interfaces make the end layers linear (a_0 = 2 q_0 - a_1, a_km
// likewise, or qs when iv == -2).  Layers 2..km-3 take the kord 4 constraint
// of Lin (2004): each edge deviation at most |2 dm| with the sign of dm; the
// two layers at each end take CW84.
//
// Both families, iv >= 0: where a layer's edges or interior minimum fall below
// the floor (0, or q_min when iv == 1), its deviations from the mean are scaled
// so that the minimum reaches the floor (Zhang & Shu 2010; mean kept).
template <class T>
void cs_interfaces(const T* q, const double* dp, int km, int iv, double qs, T* a) {
  std::vector<T> rhs(km + 1);
  std::vector<double> cp(km + 1), lo(km + 1), di(km + 1), up(km + 1);
  double g = dp[1] / dp[0];
  di[0] = g; up[0] = g + 1.0; lo[0] = 0.0;
  rhs[0] = (T(g * (2.0 * g + 3.0)) * q[0] + q[1]) / T(g + 1.0);
  for (int k = 1; k < km; ++k) {
    double d = dp[k - 1] / dp[k];
    lo[k] = 1.0; di[k] = 2.0 * (1.0 + d); up[k] = d;
    rhs[k] = T(3.0) * (q[k - 1] + T(d) * q[k]);
  }
  if (iv == -2) {
    lo[km] = 0.0; di[km] = 1.0; up[km] = 0.0;
    rhs[km] = T(qs);
  } else {
    double gb = dp[km - 2] / dp[km - 1];
    lo[km] = gb + 1.0; di[km] = gb; up[km] = 0.0;
    rhs[km] = (T(gb * (2.0 * gb + 3.0)) * q[km - 1] + q[km - 2]) / T(gb + 1.0);
  }
  // Thomas algorithm
  cp[0] = up[0] / di[0];
  a[0] = rhs[0] / T(di[0]);
  for (int k = 1; k <= km; ++k) {
    double den = di[k] - lo[k] * cp[k - 1];
    cp[k] = up[k] / den;
    a[k] = (rhs[k] - T(lo[k]) * a[k - 1]) / T(den);
  }
  for (int k = km - 1; k >= 0; --k) a[k] = a[k] - T(cp[k]) * a[k + 1];
}

// kord 9 interface constraint with extremum detection (see above)
template <class T>
void k9_interface_limits(const T* q, int km, int iv, double floor_v, T* a) {
  auto D = [&](int u) { return val(q[u]) - val(q[u - 1]); };  // jump across interface u (1..km-1)
  a[0] = clamp2(a[0], q[0], q[1]);
  for (int u = 1; u < km; ++u) {
    const double dl = D(u > 1 ? u - 1 : u), dr = D(u < km - 1 ? u + 1 : u);
    tally<T>(0, 1, 1);
    if (dl * dr > 0.0) {
      a[u] = clamp2(a[u], q[u - 1], q[u]);
    } else if (dl > 0.0) {
      a[u] = tmax(a[u], tmin(q[u - 1], q[u]));
    } else {
      a[u] = tmin(a[u], tmax(q[u - 1], q[u]));
      if (iv >= 0) a[u] = tmax(a[u], T(floor_v));
    }
  }
  if (iv != -2) a[km] = clamp2(a[km], q[km - 2], q[km - 1]);
}

// Value at the interface between an end layer (mean q0, thickness h0) and the
// next layer (q1, h1) of the parabola whose means over those two layers and
// the one after them (q2, h2) are the layer means: the derivative at that
// interface of the cubic through the cumulative masses.
template <class T>
T quad3_interface(T q0, T q1, T q2, double h0, double h1, double h2) {
  const double w0 = h1 * (h1 + h2) / ((h0 + h1) * (h0 + h1 + h2));
  const double w2 = -h0 * h1 / ((h0 + h1 + h2) * (h1 + h2));
  const double w1 = 1.0 - w0 - w2;
  return T(w0) * q0 + T(w1) * q1 + T(w2) * q2;
}

// PPM interfaces and half-increment slopes (kord < 7, see above)
template <class T>
void ppm_interfaces(const T* q, const double* dp, int km, int iv, double qs, T* a, T* dm) {
  for (int k = 0; k < km; ++k) dm[k] = T(0.0);
  for (int k = 1; k < km - 1; ++k) {
    const double d0 = dp[k - 1], d1 = dp[k], d2 = dp[k + 1];
    const T dq = T(d1 / (d0 + d1 + d2)) * (T((2.0 * d0 + d1) / (d2 + d1)) * (q[k + 1] - q[k]) +
                                            T((d1 + 2.0 * d2) / (d0 + d1)) * (q[k] - q[k - 1]));
    const T mx = tmax(tmax(q[k - 1], q[k]), q[k + 1]) - q[k];
    const T mn = q[k] - tmin(tmin(q[k - 1], q[k]), q[k + 1]);
    dm[k] = tsign(tmin(tmin(T(0.5) * tabs(dq), mx), mn), dq);
  }
  for (int u = 2; u <= km - 2; ++u) {
    const int j = u - 1;
    const double hm = dp[j - 1], h0 = dp[j], h1 = dp[j + 1], h2 = dp[j + 2];
    const double s01 = h0 + h1, sall = hm + h0 + h1 + h2;
    const double c0 = h0 / s01;
    const double c1 = 2.0 * h1 * h0 / s01 * ((hm + h0) / (2.0 * h0 + h1) - (h2 + h1) / (2.0 * h1 + h0)) / sall;
    const double c2 = h0 * (hm + h0) / (2.0 * h0 + h1) / sall;
    const double c3 = h1 * (h1 + h2) / (h0 + 2.0 * h1) / sall;
    const T dq = q[j + 1] - q[j];
    a[u] = q[j] + T(c0 + c1) * dq - T(2.0 * c2) * dm[j + 1] + T(2.0 * c3) * dm[j];
  }
  if (km == 2) {
    a[1] = (q[0] * T(dp[1]) + q[1] * T(dp[0])) / T(dp[0] + dp[1]);
  } else {
    a[1] = clamp2(quad3_interface(q[0], q[1], q[2], dp[0], dp[1], dp[2]), q[0], q[1]);
    a[km - 1] = clamp2(quad3_interface(q[km - 1], q[km - 2], q[km - 3], dp[km - 1], dp[km - 2], dp[km - 3]),
                       q[km - 2], q[km - 1]);
  }
  a[0] = T(2.0) * q[0] - a[1];
  a[km] = (iv == -2) ? T(qs) : T(2.0) * q[km - 1] - a[km - 1];
}

template <class T>
void column_profile_t(const T* q, const double* dp, int km, int iv, int kord, double qs, double q_min,
                      T* aL, T* aR, T* a6) {
  const double floor_v = (iv == 1) ? q_min : 0.0;
  if (km == 1) {
    aL[0] = q[0];
    aR[0] = q[0];
    a6[0] = T(0.0);
    return;
  }
  std::vector<T> a(km + 1), dm(km);
  if (kord >= 7) {
    cs_interfaces(q, dp, km, iv, qs, a.data());
    k9_interface_limits(q, km, iv, floor_v, a.data());
  } else {
    ppm_interfaces(q, dp, km, iv, qs, a.data(), dm.data());
  }
  auto D = [&](int u) { return val(q[u]) - val(q[u - 1]); };
  auto extm = [&](int k) { return k >= 1 && k <= km - 2 && D(k) * D(k + 1) < 0.0; };
  for (int k = 0; k < km; ++k) {
    T bl = a[k] - q[k], br = a[k + 1] - q[k];
    const bool end_layer = k < 2 || k > km - 3;
    if (end_layer) {
      cw84(bl, br);
    } else if (kord >= 7) {
      tally<T>(0, 2, 3);
      if (extm(k) && (extm(k - 1) || extm(k + 1))) {
        bl = T(0.0);
        br = T(0.0);
      } else {
        tally<T>(2, 1, 1);
        if (3.0 * std::fabs(val(bl) + val(br)) > std::fabs(val(br) - val(bl))) {
          const T pr = T(2.0) * (q[k] - q[k - 1]), lr = pr - T(1.5) * (q[k - 1] - q[k - 2]);
          const T pl = T(-2.0) * (q[k + 1] - q[k]), ll = pl + T(1.5) * (q[k + 2] - q[k + 1]);
          br = tmin(tmax(br, tmin(tmin(T(0.0), pr), lr)), tmax(tmax(T(0.0), pr), lr));
          bl = tmin(tmax(bl, tmin(tmin(T(0.0), pl), ll)), tmax(tmax(T(0.0), pl), ll));
        }
      }
    } else {
      const T xt = T(2.0) * dm[k];
      bl = -tsign(tmin(tabs(xt), tabs(bl)), xt);
      br = tsign(tmin(tabs(xt), tabs(br)), xt);
    }
    if (iv >= 0) {
      // Positivity (Zhang & Shu 2010 scaling): when the reconstruction's
      // minimum -- an edge, or the interior minimum q + s6/12 + da^2/(4 s6) of
      // a parabola with s6 < -|da| -- lies below the floor, the deviations are
      // scaled by (q - floor)/(q - min) so that the minimum reaches the floor
      // (by 0 when the mean itself is below it).  Mean-preserving and
      // continuous in q.  The interior test is taken multiplied through by
      // 12 s6: 12 s6 (q - floor) + s6^2 + 3 da^2 > 0.
      const double qv = val(q[k]);
      const double s6 = -3.0 * (val(bl) + val(br)), da = val(br) - val(bl);
      const bool inner = -s6 > std::fabs(da);
      const bool low = qv + val(bl) < floor_v || qv + val(br) < floor_v ||
                       (inner && 12.0 * s6 * (qv - floor_v) + s6 * s6 + 3.0 * da * da > 0.0);
      if (low) {
        T pmin = tmin(q[k] + bl, q[k] + br);
        if (inner) {
          const T s6t = T(-3.0) * (bl + br), dat = br - bl;
          pmin = tmin(pmin, q[k] + s6t / T(12.0) + dat * dat / (T(4.0) * s6t));
        }
        const T lam = qv > floor_v ? (q[k] - T(floor_v)) / (q[k] - pmin) : T(0.0);
        bl = lam * bl;
        br = lam * br;
      }
    }
    aL[k] = q[k] + bl;
    aR[k] = q[k] + br;
    a6[k] = T(-3.0) * (bl + br);
  }
}

// mean of the parabola of layer k over [x1, x2] (fractions of the layer)
template <class T> inline T pmean(const T& l, const T& r, const T& s6, double x1, double x2) {
  return l + T(0.5 * (x1 + x2)) * ((r - l) + s6) - s6 * T((x2 * x2 + x1 * x2 + x1 * x1) / 3.0);
}

// Conservative remap of one column (merge of the two sorted interface lists).
// dp2 (optional): the target thicknesses that divide the overlap masses
// (map1_q2), else pe2 differences.
template <class T>
void remap_column_t(int km, const double* pe1, const T* q1, double qs, int kn, const double* pe2, T* q2,
                    int iv, int kord, double q_min, const double* dp2 = nullptr) {
  std::vector<double> dp(km);
  for (int k = 0; k < km; ++k) dp[k] = pe1[k + 1] - pe1[k];
  std::vector<T> aL(km), aR(km), a6(km);
  column_profile_t<T>(q1, dp.data(), km, iv, kord, qs, q_min, aL.data(), aR.data(), a6.data());
  int k1 = 0;
  for (int k2 = 0; k2 < kn; ++k2) {
    const double top = pe2[k2], bot = pe2[k2 + 1];
    while (k1 < km - 1 && pe1[k1 + 1] <= top) ++k1;
    if (bot <= pe1[k1 + 1]) {  // inside one source layer
      if (top == pe1[k1] && bot == pe1[k1 + 1]) {
        q2[k2] = q1[k1];
      } else {
        double x1 = (top - pe1[k1]) / dp[k1], x2 = (bot - pe1[k1]) / dp[k1];
        q2[k2] = pmean(aL[k1], aR[k1], a6[k1], x1, x2);
      }
      continue;
    }
    T mass;
    if (top == pe1[k1]) {
      mass = q1[k1] * T(dp[k1]);
    } else {
      double x1 = (top - pe1[k1]) / dp[k1];
      mass = T(dp[k1] * (1.0 - x1)) * pmean(aL[k1], aR[k1], a6[k1], x1, 1.0);
    }
    int m = k1 + 1;
    while (m < km && pe1[m + 1] <= bot) {
      mass = mass + q1[m] * T(dp[m]);
      ++m;
    }
    if (m < km) {
      if (bot > pe1[m]) {
        double x2 = (bot - pe1[m]) / dp[m];
        mass = mass + T(dp[m] * x2) * pmean(aL[m], aR[m], a6[m], 0.0, x2);
      }
    } else if (bot > pe1[km]) {  // below the source column: constant extension
      mass = mass + q1[km - 1] * T(bot - pe1[km]);
    }
    q2[k2] = mass / T(dp2 ? dp2[k2] : bot - top);
    k1 = std::min(m, km - 1);
  }
}

}  // namespace

// =================================================================== C ABI ===
extern "C" {

void orc_copy_corners(double* q, int npx, int npy, int dir, const orc_grid* g, const orc_bounds* bd) {
  copy_corners_t<double>(q, npx, npy, dir, g, bd);
}

void orc_fv_tp_2d(double* q, const double* crx, const double* cry, int npx, int npy, int hord, double* fx,
                  double* fy, const double* xfx, const double* yfx, const orc_grid* g, const orc_bounds* bd,
                  const double* ra_x, const double* ra_y, double lim_fac, const double* mfx, const double* mfy,
                  const double* mass, int nord, double damp_c) {
  fv_tp_2d_t<double>(q, crx, cry, npx, npy, hord, fx, fy, xfx, yfx, g, bd, ra_x, ra_y, lim_fac, mfx, mfy, mass, nord,
                     damp_c);
}

void orc_count_fv_tp_2d(const double* q, const double* crx, const double* cry, int npx, int npy, int hord,
                        const double* xfx, const double* yfx, const orc_grid* g, const orc_bounds* bd,
                        const double* ra_x, const double* ra_y, const double* mfx, const double* mfy,
                        unsigned long long* counts) {
  Dom d(bd);
  std::vector<Cnt> qq(d.plane), fx(d.nmx), fy(d.nmy);
  for (size_t n = 0; n < d.plane; ++n) qq[n] = Cnt(q[n]);
  g_ops = OpTally{};
  fv_tp_2d_t<Cnt>(qq.data(), crx, cry, npx, npy, hord, fx.data(), fy.data(), xfx, yfx, g, bd, ra_x, ra_y, 1.0, mfx,
                  mfy, nullptr, 0, 0.0);
  counts[0] = g_ops.add;
  counts[1] = g_ops.mul;
  counts[2] = g_ops.div;
  counts[3] = g_ops.cmp;
}

void orc_count_remap_column(int km, const double* pe1, const double* q1, int kn, const double* pe2, int iv, int kord,
                            unsigned long long* counts) {
  std::vector<Cnt> c1(q1, q1 + km), c2(kn);
  g_ops = OpTally{};
  remap_column_t<Cnt>(km, pe1, c1.data(), 0.0, kn, pe2, c2.data(), iv, kord, 0.0);
  counts[0] = g_ops.add;
  counts[1] = g_ops.mul;
  counts[2] = g_ops.div;
  counts[3] = g_ops.cmp;
}

void orc_fv_tp_2d_tl(const double* q, const double* dq, const double* crx, const double* cry, int npx,
                     int npy, int hord, double* dfx, double* dfy, const double* xfx, const double* yfx,
                     const orc_grid* g, const orc_bounds* bd, const double* ra_x, const double* ra_y,
                     double lim_fac, const double* mfx, const double* mfy, const double* mass, int nord,
                     double damp_c) {
  Dom d(bd);
  std::vector<Dual> qq(d.plane), fx(d.nmx), fy(d.nmy);
  for (size_t n = 0; n < d.plane; ++n) qq[n] = Dual(q[n], dq[n]);
  fv_tp_2d_t<Dual>(qq.data(), crx, cry, npx, npy, hord, fx.data(), fy.data(), xfx, yfx, g, bd, ra_x, ra_y, lim_fac,
                   mfx, mfy, mass, nord, damp_c);
  for (size_t n = 0; n < d.nmx; ++n) dfx[n] = fx[n].d;
  for (size_t n = 0; n < d.nmy; ++n) dfy[n] = fy[n].d;
}

// nested_grid_BC_apply_intT for one 3-D field with no staggering: the halo
// cells on the outer sides of the nested domain get the boundary state
// interpolated in time, (t0·(split − step) + step·t1)·(1/split).  West and
// east take the full height of the data domain (the corner blocks with them);
// south and north take the columns between, i = is..ie on a side that is an
// outer side and isd/ied where the rank has a neighbour.  The strips are laid
// out as allocate_fv_nest_BC_type allocates them with istag = jstag = 0
// (moving_nest/fv_moving_nest.F90:2005-2008): west (isd:0, jsd:jed), east
// (npx:ied, jsd:jed), south (isd:ied, jsd:0), north (isd:ied, npy:jed), each
// with npz levels.
static void nest_bc_apply(double* var, const Dom& d, int npx, int npy, int npz, const orc_nest_bc& bc, double step,
                          double split) {
  const double denom = 1.0 / split;
  auto blend = [&](const double* t0, const double* t1, size_t n) {
    return (t0[n] * (split - step) + step * t1[n]) * denom;
  };
  const int nwest = 1 - d.isd, neast = d.ied - npx + 1, nsouth = 1 - d.jsd, nnorth = d.jed - npy + 1;
  const int i0 = (d.is == 1) ? d.is : d.isd, i1 = (d.ie == npx - 1) ? d.ie : d.ied;
  for (int k = 0; k < npz; ++k) {
    View2<double> V{var + (size_t)k * d.plane, d.isd, d.jsd, d.nid};
    if (d.is == 1)
      for (int j = d.jsd; j <= d.jed; ++j)
        for (int i = d.isd; i <= 0; ++i)
          V(i, j) = blend(bc.west_t0, bc.west_t1,
                          (size_t)(i - d.isd) + (size_t)(j - d.jsd) * nwest + (size_t)k * nwest * d.njd);
    if (d.ie == npx - 1)
      for (int j = d.jsd; j <= d.jed; ++j)
        for (int i = npx; i <= d.ied; ++i)
          V(i, j) = blend(bc.east_t0, bc.east_t1,
                          (size_t)(i - npx) + (size_t)(j - d.jsd) * neast + (size_t)k * neast * d.njd);
    if (d.js == 1)
      for (int j = d.jsd; j <= 0; ++j)
        for (int i = i0; i <= i1; ++i)
          V(i, j) = blend(bc.south_t0, bc.south_t1,
                          (size_t)(i - d.isd) + (size_t)(j - d.jsd) * d.nid + (size_t)k * d.nid * nsouth);
    if (d.je == npy - 1)
      for (int j = npy; j <= d.jed; ++j)
        for (int i = i0; i <= i1; ++i)
          V(i, j) = blend(bc.north_t0, bc.north_t1,
                          (size_t)(i - d.isd) + (size_t)(j - npy) * d.nid + (size_t)k * d.nid * nnorth);
  }
}

void orc_nest_bc_apply(double* var, const orc_bounds* bd, int npx, int npy, int npz, const orc_nest_bc* bc,
                       double step, double split) {
  nest_bc_apply(var, Dom(bd), npx, npy, npz, *bc, step, split);
}

// The substep loop of tracer_2d; on a nested grid with boundary states, they
// are applied to every tracer after the halo refresh of each substep, at the
// time of the substep's start: step = the count of tracer substeps taken since
// the parent's t0 (neststruct%tracer_nest_timestep, passed to
// setup_nested_grid_BCs at moving_nest/fv_moving_nest.F90:1781), split =
// nsplt·k_split; the count advances by one per substep of a nested grid.
static int tracer_2d_run(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy, const orc_grid* g,
                         const orc_bounds* bd, int npx, int npy, int npz, int nq, int hord, int q_split,
                         int nord_tr, double trdm, double lim_fac, orc_halo_fn halo_fn, void* halo_ctx,
                         const orc_nest_bc* q_bc, int* nest_timestep, int k_split) {
  Dom d(bd);
  std::vector<double> xfx(d.nxf * npz), yfx(d.nyf * npz);
  for (int k = 0; k < npz; ++k) area_fluxes(cx + k * d.nxf, cy + k * d.nyf, xfx.data() + k * d.nxf,
                                            yfx.data() + k * d.nyf, g, bd);
  int nsplt = q_split > 0 ? q_split : (int)(1.0 + max_courant(cx, cy, d, npz));
  if (nsplt != 1) {
    double frac = 1.0 / nsplt;
    scale_fluxes(mfx, mfy, cx, cy, d, npz, frac);
    for (auto& v : xfx) v *= frac;
    for (auto& v : yfx) v *= frac;
  }
  std::vector<double> fx(d.nmx), fy(d.nmy);
  for (int it = 0; it < nsplt; ++it) {
    if (halo_fn) halo_fn(q, nq, npz, halo_ctx);
    if (nest_timestep && g->nested) {
      if (q_bc)
        for (int iq = 0; iq < nq; ++iq)
          nest_bc_apply(q + (size_t)iq * npz * d.plane, d, npx, npy, npz, q_bc[iq], (double)*nest_timestep,
                        (double)nsplt * k_split);
      ++*nest_timestep;
    }
#pragma omp parallel for schedule(dynamic) firstprivate(fx, fy)
    for (int k = 0; k < npz; ++k) {
      Level L;
      L.xfx.assign(xfx.begin() + k * d.nxf, xfx.begin() + (k + 1) * d.nxf);
      L.yfx.assign(yfx.begin() + k * d.nyf, yfx.begin() + (k + 1) * d.nyf);
      level_setup(L, dp1 + k * d.plane, mfx + k * d.nmx, mfy + k * d.nmy, g, d);
      for (int iq = 0; iq < nq; ++iq) {
        double* qk = q + ((size_t)iq * npz + k) * d.plane;
        // damping on the first substep only, weighted by the thickness at its start
        fv_tp_2d_t<double>(qk, cx + k * d.nxf, cy + k * d.nyf, npx, npy, hord, fx.data(), fy.data(), L.xfx.data(),
                           L.yfx.data(), g, bd, L.rax.data(), L.ray.data(), lim_fac, mfx + k * d.nmx,
                           mfy + k * d.nmy, dp1 + k * d.plane, nord_tr, it == 0 ? trdm : 0.0);
        flux_update(qk, dp1 + k * d.plane, L, fx.data(), fy.data(), g, d);
      }
      if (it < nsplt - 1) {
        View2<double> DP{dp1 + k * d.plane, d.isd, d.jsd, d.nid};
        View2<const double> D2{L.dp2.data(), d.isd, d.jsd, d.nid};
        for (int j = d.js; j <= d.je; ++j)
          for (int i = d.is; i <= d.ie; ++i) DP(i, j) = D2(i, j);
      }
    }
  }
  return nsplt;
}

int orc_tracer_2d(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy, const orc_grid* g,
                  const orc_bounds* bd, int npx, int npy, int npz, int nq, int hord, int q_split, double dt,
                  int nord_tr, double trdm, double lim_fac, orc_halo_fn halo_fn, void* halo_ctx) {
  (void)dt;
  return tracer_2d_run(q, dp1, mfx, mfy, cx, cy, g, bd, npx, npy, npz, nq, hord, q_split, nord_tr, trdm, lim_fac,
                       halo_fn, halo_ctx, nullptr, nullptr, 1);
}

int orc_tracer_2d_nested(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                         const orc_grid* g, const orc_bounds* bd, int npx, int npy, int npz, int nq, int hord,
                         int q_split, double dt, int nord_tr, double trdm, int k_split, const orc_nest_bc* q_bc,
                         int* nest_timestep, double lim_fac, orc_halo_fn halo_fn, void* halo_ctx) {
  (void)dt;
  int counter = nest_timestep ? *nest_timestep : 0;
  const int nsplt = tracer_2d_run(q, dp1, mfx, mfy, cx, cy, g, bd, npx, npy, npz, nq, hord, q_split, nord_tr, trdm,
                                  lim_fac, halo_fn, halo_ctx, q_bc, &counter, k_split);
  if (nest_timestep) *nest_timestep = counter;
  return nsplt;
}

// tracer_2d_1L: the levels one at a time, each with its own substep count
// from its own Courant maximum (or q_split), its fluxes scaled by its own
// 1/nsplt; the halo callback runs before every substep of every level.
int orc_tracer_2d_1L(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy, const orc_grid* g,
                     const orc_bounds* bd, int npx, int npy, int npz, int nq, int hord, int q_split, double dt,
                     int nord_tr, double trdm, double lim_fac, orc_halo_fn halo_fn, void* halo_ctx,
                     int* nsplt_levels) {
  (void)dt;
  Dom d(bd);
  std::vector<double> fx(d.nmx), fy(d.nmy);
  int nmax = 0;
  for (int k = 0; k < npz; ++k) {
    double *cxk = cx + k * d.nxf, *cyk = cy + k * d.nyf, *mxk = mfx + k * d.nmx, *myk = mfy + k * d.nmy;
    double* dpk = dp1 + k * d.plane;
    Level L;
    L.xfx.assign(d.nxf, 0.0);
    L.yfx.assign(d.nyf, 0.0);
    area_fluxes(cxk, cyk, L.xfx.data(), L.yfx.data(), g, bd);
    const int nsplt = q_split > 0 ? q_split : (int)(1.0 + max_courant(cxk, cyk, d, 1));
    if (nsplt != 1) {
      const double frac = 1.0 / nsplt;
      scale_fluxes(mxk, myk, cxk, cyk, d, 1, frac);
      for (auto& v : L.xfx) v *= frac;
      for (auto& v : L.yfx) v *= frac;
    }
    for (int it = 0; it < nsplt; ++it) {
      if (halo_fn) halo_fn(q, nq, npz, halo_ctx);
      level_setup(L, dpk, mxk, myk, g, d);
      for (int iq = 0; iq < nq; ++iq) {
        double* qk = q + ((size_t)iq * npz + k) * d.plane;
        fv_tp_2d_t<double>(qk, cxk, cyk, npx, npy, hord, fx.data(), fy.data(), L.xfx.data(), L.yfx.data(), g, bd,
                           L.rax.data(), L.ray.data(), lim_fac, mxk, myk, dpk, nord_tr, it == 0 ? trdm : 0.0);
        flux_update(qk, dpk, L, fx.data(), fy.data(), g, d);
      }
      if (it < nsplt - 1) {
        View2<double> DP{dpk, d.isd, d.jsd, d.nid};
        View2<const double> D2{L.dp2.data(), d.isd, d.jsd, d.nid};
        for (int j = d.js; j <= d.je; ++j)
          for (int i = d.is; i <= d.ie; ++i) DP(i, j) = D2(i, j);
      }
    }
    if (nsplt_levels) nsplt_levels[k] = nsplt;
    nmax = std::max(nmax, nsplt);
  }
  return nmax;
}

// Edge halo strips of six tiles from their neighbours' interiors.
void orc_cube_halo_fill(double* q, int n, int ng, int nplanes, const int* topo) {
  const int nid = n + 2 * ng;
  const size_t plane = (size_t)nid * nid;
  auto at = [&](int t, int p, int i, int j) -> double& {  // i, j 1-based tile indices
    return q[((size_t)t * nplanes + p) * plane + (size_t)(i - 1 + ng) + (size_t)(j - 1 + ng) * nid];
  };
#pragma omp parallel for schedule(static)
  for (int p = 0; p < nplanes; ++p)
    for (int t = 0; t < 6; ++t)
      for (int e = 0; e < 4; ++e) {
        const int nt = topo[(t * 4 + e) * 3 + 0], ne = topo[(t * 4 + e) * 3 + 1], rev = topo[(t * 4 + e) * 3 + 2];
        for (int dpt = 1; dpt <= ng; ++dpt)
          for (int s = 0; s < n; ++s) {
            int i, j;  // halo cell on tile t
            switch (e) {
              case 0: i = 1 - dpt; j = s + 1; break;
              case 1: i = n + dpt; j = s + 1; break;
              case 2: i = s + 1; j = 1 - dpt; break;
              default: i = s + 1; j = n + dpt; break;
            }
            int sb = rev ? n - 1 - s : s, ib, jb;  // interior cell on tile nt
            switch (ne) {
              case 0: ib = dpt; jb = sb + 1; break;
              case 1: ib = n + 1 - dpt; jb = sb + 1; break;
              case 2: ib = sb + 1; jb = dpt; break;
              default: ib = sb + 1; jb = n + 1 - dpt; break;
            }
            at(t, p, i, j) = at(nt, p, ib, jb);
          }
      }
}

int orc_tracer_2d_cube(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                       const orc_grid* g6, int n, int npz, int nq, int hord, int q_split, const int* topo,
                       int sync_edges, int nord_tr, double trdm, double lim_fac) {
  const int ng = 3;
  orc_bounds bd{1, n, 1, n, 1 - ng, n + ng, 1 - ng, n + ng, ng};
  Dom d(&bd);
  const int npx = n + 1, npy = n + 1;
  std::vector<double> xfx(6 * d.nxf * npz), yfx(6 * d.nyf * npz);
  double cmax = 0.0;
  for (int t = 0; t < 6; ++t) {
    for (int k = 0; k < npz; ++k)
      area_fluxes(cx + (t * npz + k) * d.nxf, cy + (t * npz + k) * d.nyf, xfx.data() + (t * npz + k) * d.nxf,
                  yfx.data() + (t * npz + k) * d.nyf, &g6[t], &bd);
    cmax = std::max(cmax, max_courant(cx + t * npz * d.nxf, cy + t * npz * d.nyf, d, npz));
  }
  int nsplt = q_split > 0 ? q_split : (int)(1.0 + cmax);
  if (nsplt != 1) {
    double frac = 1.0 / nsplt;
    for (int t = 0; t < 6; ++t)
      scale_fluxes(mfx + t * npz * d.nmx, mfy + t * npz * d.nmy, cx + t * npz * d.nxf, cy + t * npz * d.nyf, d,
                   npz, frac);
    for (auto& v : xfx) v *= frac;
    for (auto& v : yfx) v *= frac;
  }
  // edge outflux of each tile-edge face: eflux[((t*4+e)*n + s)]
  for (int it = 0; it < nsplt; ++it) {
    orc_cube_halo_fill(q, n, ng, npz * nq, topo);
#pragma omp parallel for schedule(dynamic)
    for (int k = 0; k < npz; ++k) {
      Level L[6];
      std::vector<double> fx(6 * d.nmx), fy(6 * d.nmy), ef(6 * 4 * n);
      for (int t = 0; t < 6; ++t) {
        L[t].xfx.assign(xfx.begin() + (t * npz + k) * d.nxf, xfx.begin() + (t * npz + k + 1) * d.nxf);
        L[t].yfx.assign(yfx.begin() + (t * npz + k) * d.nyf, yfx.begin() + (t * npz + k + 1) * d.nyf);
        level_setup(L[t], dp1 + (t * npz + k) * d.plane, mfx + (t * npz + k) * d.nmx, mfy + (t * npz + k) * d.nmy,
                    &g6[t], d);
      }
      for (int iq = 0; iq < nq; ++iq) {
        for (int t = 0; t < 6; ++t) {
          double* qk = q + (((size_t)t * nq + iq) * npz + k) * d.plane;
          fv_tp_2d_t<double>(qk, cx + (t * npz + k) * d.nxf, cy + (t * npz + k) * d.nyf, npx, npy, hord,
                             fx.data() + t * d.nmx, fy.data() + t * d.nmy, L[t].xfx.data(), L[t].yfx.data(),
                             &g6[t], &bd, L[t].rax.data(), L[t].ray.data(), lim_fac, mfx + (t * npz + k) * d.nmx,
                             mfy + (t * npz + k) * d.nmy, dp1 + (t * npz + k) * d.plane, nord_tr,
                             it == 0 ? trdm : 0.0);
        }
        if (sync_edges) {
          // outward flux of every tile-edge face, then adopt the owner's value
          auto FX = [&](int t, int i, int j) -> double& { return fx[t * d.nmx + (i - 1) + (size_t)(j - 1) * (n + 1)]; };
          auto FY = [&](int t, int i, int j) -> double& { return fy[t * d.nmy + (i - 1) + (size_t)(j - 1) * n]; };
          auto out = [&](int t, int e, int s) -> double {
            switch (e) {
              case 0: return -FX(t, 1, s + 1);
              case 1: return FX(t, n + 1, s + 1);
              case 2: return -FY(t, s + 1, 1);
              default: return FY(t, s + 1, n + 1);
            }
          };
          for (int t = 0; t < 6; ++t)
            for (int e = 0; e < 4; ++e)
              for (int s = 0; s < n; ++s) ef[(t * 4 + e) * n + s] = out(t, e, s);
          // the face flux is the one computed by the upwind tile (the tile the
          // flow leaves), so every donor cell's outflow comes from its own
          // monotone reconstruction; a face with zero Courant number belongs
          // to the lower-numbered tile
          for (int t = 0; t < 6; ++t)
            for (int e = 0; e < 4; ++e) {
              const int nt = topo[(t * 4 + e) * 3 + 0], ne = topo[(t * 4 + e) * 3 + 1], rev = topo[(t * 4 + e) * 3 + 2];
              const double* cxt = cx + (t * npz + k) * d.nxf;
              const double* cyt = cy + (t * npz + k) * d.nyf;
              for (int s = 0; s < n; ++s) {
                double cin;  // Courant number into tile t through this face
                switch (e) {
                  case 0: cin = cxt[0 + (size_t)(s + 1 - d.jsd) * (n + 1)]; break;
                  case 1: cin = -cxt[n + (size_t)(s + 1 - d.jsd) * (n + 1)]; break;
                  case 2: cin = cyt[(s + 1 - d.isd) + 0 * (size_t)d.nid]; break;
                  default: cin = -cyt[(s + 1 - d.isd) + (size_t)n * d.nid]; break;
                }
                if (!(cin > 0.0 || (cin == 0.0 && nt < t))) continue;  // tile t is upwind: keeps its flux
                double inflow = ef[(nt * 4 + ne) * n + (rev ? n - 1 - s : s)];  // upwind tile's outflux
                switch (e) {
                  case 0: FX(t, 1, s + 1) = inflow; break;
                  case 1: FX(t, n + 1, s + 1) = -inflow; break;
                  case 2: FY(t, s + 1, 1) = inflow; break;
                  default: FY(t, s + 1, n + 1) = -inflow; break;
                }
              }
            }
        }
        for (int t = 0; t < 6; ++t) {
          double* qk = q + (((size_t)t * nq + iq) * npz + k) * d.plane;
          flux_update(qk, dp1 + (t * npz + k) * d.plane, L[t], fx.data() + t * d.nmx, fy.data() + t * d.nmy,
                      &g6[t], d);
        }
      }
      if (it < nsplt - 1)
        for (int t = 0; t < 6; ++t) {
          View2<double> DP{dp1 + (t * npz + k) * d.plane, d.isd, d.jsd, d.nid};
          View2<const double> D2{L[t].dp2.data(), d.isd, d.jsd, d.nid};
          for (int j = 1; j <= n; ++j)
            for (int i = 1; i <= n; ++i) DP(i, j) = D2(i, j);
        }
    }
  }
  return nsplt;
}

void orc_column_profile(const double* q, const double* delp, int km, int iv, int kord, double qs, double q_min,
                        double* a4) {
  std::vector<double> aL(km), aR(km), a6(km);
  column_profile_t<double>(q, delp, km, iv, kord, qs, q_min, aL.data(), aR.data(), a6.data());
  for (int k = 0; k < km; ++k) {
    a4[4 * k + 0] = q[k];
    a4[4 * k + 1] = aL[k];
    a4[4 * k + 2] = aR[k];
    a4[4 * k + 3] = a6[k];
  }
}

void orc_remap_column(int km, const double* pe1, const double* q1, double qs, int kn, const double* pe2, double* q2,
                      int iv, int kord, double q_min) {
  remap_column_t<double>(km, pe1, q1, qs, kn, pe2, q2, iv, kord, q_min);
}

static void map_row(int km, const double* pe1, const double* q1, const double* qs, int kn, const double* pe2,
                    double* q2, int i1, int i2, int j, int ibeg, int iend, int jbeg, int jend, int iv, int kord,
                    double q_min) {
  const int ni = i2 - i1 + 1;
  const size_t nib = (size_t)(iend - ibeg + 1), plane = nib * (size_t)(jend - jbeg + 1);
  std::vector<double> p1(km + 1), p2(kn + 1), c1(km), c2(kn);
  for (int i = i1; i <= i2; ++i) {
    for (int k = 0; k <= km; ++k) p1[k] = pe1[(i - i1) + (size_t)k * ni];
    for (int k = 0; k <= kn; ++k) p2[k] = pe2[(i - i1) + (size_t)k * ni];
    const size_t off = (size_t)(i - ibeg) + (size_t)(j - jbeg) * nib;
    for (int k = 0; k < km; ++k) c1[k] = q1[off + k * plane];
    remap_column_t<double>(km, p1.data(), c1.data(), qs ? qs[i - i1] : 0.0, kn, p2.data(), c2.data(), iv, kord,
                           q_min);
    for (int k = 0; k < kn; ++k) q2[off + k * plane] = c2[k];
  }
}

void orc_map_scalar(int km, const double* pe1, const double* q1, const double* qs, int kn, const double* pe2,
                    double* q2, int i1, int i2, int j, int ibeg, int iend, int jbeg, int jend, int iv, int kord,
                    double q_min) {
  map_row(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j, ibeg, iend, jbeg, jend, iv, kord, q_min);
}

void orc_map1_ppm(int km, const double* pe1, const double* q1, const double* qs, int kn, const double* pe2,
                  double* q2, int i1, int i2, int j, int ibeg, int iend, int jbeg, int jend, int iv, int kord) {
  map_row(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j, ibeg, iend, jbeg, jend, iv, kord, 0.0);
}

// map1_q2 (fv_mapz.F90): the remap of columns with the target thicknesses
// dp2 (kn, ncol) given for the division of the overlap masses.
void orc_remap_columns_dp2(int ncol, int km, const double* pe1, const double* q1, const double* qs, int kn,
                           const double* pe2, const double* dp2, double* q2, int iv, int kord, double q_min) {
#pragma omp parallel
  {
    std::vector<double> p1(km + 1), p2(kn + 1), c1(km), c2(kn), d2(kn);
#pragma omp for schedule(static)
    for (int c = 0; c < ncol; ++c) {
      for (int k = 0; k <= km; ++k) p1[k] = pe1[c + (size_t)k * ncol];
      for (int k = 0; k <= kn; ++k) p2[k] = pe2[c + (size_t)k * ncol];
      for (int k = 0; k < km; ++k) c1[k] = q1[c + (size_t)k * ncol];
      for (int k = 0; k < kn; ++k) d2[k] = dp2[c + (size_t)k * ncol];
      remap_column_t<double>(km, p1.data(), c1.data(), qs ? qs[c] : 0.0, kn, p2.data(), c2.data(), iv, kord, q_min,
                             d2.data());
      for (int k = 0; k < kn; ++k) q2[c + (size_t)k * ncol] = c2[k];
    }
  }
}

void orc_remap_columns(int ncol, int km, const double* pe1, const double* q1, const double* qs, int kn,
                       const double* pe2, double* q2, int iv, int kord, double q_min) {
#pragma omp parallel
  {
    std::vector<double> p1(km + 1), p2(kn + 1), c1(km), c2(kn);
#pragma omp for schedule(static)
    for (int c = 0; c < ncol; ++c) {
      for (int k = 0; k <= km; ++k) p1[k] = pe1[c + (size_t)k * ncol];
      for (int k = 0; k <= kn; ++k) p2[k] = pe2[c + (size_t)k * ncol];
      for (int k = 0; k < km; ++k) c1[k] = q1[c + (size_t)k * ncol];
      remap_column_t<double>(km, p1.data(), c1.data(), qs ? qs[c] : 0.0, kn, p2.data(), c2.data(), iv, kord, q_min);
      for (int k = 0; k < kn; ++k) q2[c + (size_t)k * ncol] = c2[k];
    }
  }
}

void orc_remap_columns_tl(int ncol, int km, const double* pe1, const double* q1, const double* dq1, const double* qs,
                          int kn, const double* pe2, double* q2, double* dq2, int iv, int kord, double q_min) {
  std::vector<double> p1(km + 1), p2(kn + 1);
  std::vector<Dual> c1(km), c2(kn);
  for (int c = 0; c < ncol; ++c) {
    for (int k = 0; k <= km; ++k) p1[k] = pe1[c + (size_t)k * ncol];
    for (int k = 0; k <= kn; ++k) p2[k] = pe2[c + (size_t)k * ncol];
    for (int k = 0; k < km; ++k) c1[k] = Dual(q1[c + (size_t)k * ncol], dq1[c + (size_t)k * ncol]);
    remap_column_t<Dual>(km, p1.data(), c1.data(), qs ? qs[c] : 0.0, kn, p2.data(), c2.data(), iv, kord, q_min);
    for (int k = 0; k < kn; ++k) {
      q2[c + (size_t)k * ncol] = c2[k].v;
      dq2[c + (size_t)k * ncol] = c2[k].d;
    }
  }
}

// fillz (fv_fill.F90), restated: per column and tracer, a negative top layer
// is pushed into the layer below; an interior negative borrows first from the
// layer above, then from the layer below, as much as they hold; a negative
// bottom layer borrows from above; if negatives remain, the column's positive
// layer masses are scaled by (total mass)/(positive mass) and the negatives
// zeroed (no change when the total is not positive).  q (im, km, nq),
// dp (im, km), i fastest.
void orc_fillz(int im, int km, int nq, double* q, const double* dp) {
  for (int iq = 0; iq < nq; ++iq)
    for (int i = 0; i < im; ++i) {
      auto Q = [&](int k) -> double& { return q[i + (size_t)im * (k + (size_t)km * iq)]; };
      auto D = [&](int k) { return dp[i + (size_t)im * k]; };
      if (km < 2) continue;
      if (Q(0) < 0.0) {
        Q(1) += Q(0) * D(0) / D(1);
        Q(0) = 0.0;
      }
      bool fix = false;
      for (int k = 1; k < km - 1; ++k) {
        if (Q(k) >= 0.0) continue;
        fix = true;
        if (Q(k - 1) > 0.0) {
          const double dq = std::min(Q(k - 1) * D(k - 1), -Q(k) * D(k));
          Q(k - 1) -= dq / D(k - 1);
          Q(k) += dq / D(k);
        }
        if (Q(k) < 0.0 && Q(k + 1) > 0.0) {
          const double dq = std::min(Q(k + 1) * D(k + 1), -Q(k) * D(k));
          Q(k + 1) -= dq / D(k + 1);
          Q(k) += dq / D(k);
        }
      }
      const int kb = km - 1;
      if (Q(kb) < 0.0 && Q(kb - 1) > 0.0) {
        fix = true;
        const double dq = std::min(Q(kb - 1) * D(kb - 1), -Q(kb) * D(kb));
        Q(kb - 1) -= dq / D(kb - 1);
        Q(kb) += dq / D(kb);
      }
      if (!fix) continue;
      double tot = 0.0, pos = 0.0;
      for (int k = 0; k < km; ++k) {
        const double m = Q(k) * D(k);
        tot += m;
        pos += std::max(m, 0.0);
      }
      if (tot > 0.0 && pos > 0.0 && tot < pos) {
        const double f = tot / pos;
        for (int k = 0; k < km; ++k) Q(k) = std::max(Q(k), 0.0) * f;
      }
    }
}

// Pressure variables of the columns after the remap: interface pressure pe,
// its logarithm peln, pk = pe^akap and the layer mean pkz of p^akap over
// ln p, (pk(k+1) - pk(k)) / (akap (peln(k+1) - peln(k))).  delp (im, km);
// pe, peln, pk (im, km+1); pkz (im, km).
void orc_pressure_vars(int im, int km, double ptop, double akap, const double* delp, double* pe, double* peln,
                       double* pk, double* pkz) {
  for (int i = 0; i < im; ++i) {
    double p = ptop;
    for (int k = 0; k <= km; ++k) {
      if (k > 0) p += delp[i + (size_t)im * (k - 1)];
      pe[i + (size_t)im * k] = p;
      peln[i + (size_t)im * k] = std::log(p);
      pk[i + (size_t)im * k] = std::exp(akap * peln[i + (size_t)im * k]);
    }
    for (int k = 0; k < km; ++k)
      pkz[i + (size_t)im * k] = (pk[i + (size_t)im * (k + 1)] - pk[i + (size_t)im * k]) /
                                (akap * (peln[i + (size_t)im * (k + 1)] - peln[i + (size_t)im * k]));
  }
}

double orc_mass_sum(const double* q, const double* dp, const double* area, long n, long narea) {
  double s = 0.0, comp = 0.0;  // Neumaier
  for (long i = 0; i < n; ++i) {
    double x = q[i] * dp[i] * area[i % narea];
    double t = s + x;
    if (std::fabs(s) >= std::fabs(x)) comp += (s - t) + x;
    else comp += (x - t) + s;
    s = t;
  }
  return s + comp;
}

}  // extern "C"
