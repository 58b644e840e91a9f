// fv3g_profile.cuh -- sub-grid reconstruction of the layers of one column
// (cs_profile for kord 9, ppm_profile for kord 4; fv_mapz.F90 of
// GFDL_atmos_cubed_sphere, absent submodule .gitmodules:1-4), shared by the
// warp-per-column and thread-per-column remap kernels.
//
// Layer values are reached through functors q(k) and h(k) (mean and thickness
// of layer k, any k in 0..km-1), so each kernel keeps its own storage.  Every
// limiter is written with selects, so lanes of a warp that take different
// cases do not diverge.  Sign tests compare the two operands with zero rather
// than forming their product, which keeps FP32 columns free of underflow in
// the product (the sign of a difference of two floats is exact).
//
// kord 9.  Interfaces a_u (u = 0..km) come from the C1 tridiagonal system
// (the kernels solve it).  With D_u = q_u - q_{u-1} the jump across
// interface u: where the neighbouring jumps D_{u-1}, D_{u+1} have one sign
// the interface is clamped into the range of its two means; next to a local
// maximum only from below, next to a local minimum only from above (and at
// the floor for iv >= 0); at u = 1 and km-1 the missing jump is the one
// across u; the outermost interfaces are clamped into the range of the two
// outermost means (not a_km when iv == -2).  Layers: CW84 on the two at each
// end; an interior extremum beside another extremum (two-grid-length wave)
// is flattened; otherwise, when the parabola has an interior extremum, the
// edges are bounded by Huynh's second constraint (Suresh & Huynh 1997): the
// right edge to the range of q, q + 2 D_k, q + 2 D_k - 1.5 D_{k-1}, the left
// edge to the range of q, q - 2 D_{k+1}, q - 2 D_{k+1} + 1.5 D_{k+2}.
//
// kord 4.  Half-increment slopes dm from Colella & Woodward (1984) eq. 1.7
// limited by the range of the layer and its neighbours (0 in the end layers);
// interfaces 2..km-2 from CW84 eq. 1.6; interfaces 1 and km-1 from the
// parabola through the three nearest means, clamped into their two means;
// a_0 = 2 q_0 - a_1 and a_km = 2 q_{km-1} - a_{km-1} (qs when iv == -2).
// Layers 2..km-3: Lin (2004) kord 4 constraint (edge deviations at most
// |2 dm| with the sign of dm); the two layers at each end: CW84.
//
// Both: for iv >= 0, where a layer's edges or interior minimum fall below the
// floor, its deviations are scaled so that the minimum reaches the floor
// (Zhang & Shu 2010; the mean is kept and the result is continuous in q).
#pragma once

#include "fv3g_internal.cuh"

namespace fv3g {

template <typename T>
struct Profile {  // sub-grid parabola of one source layer
  T q, l, r, s6;
};

// magnitude of a with the sign of b, b == 0 (either sign) counting as positive
template <typename T> __device__ __forceinline__ T sign_of(T a, T b) {
  const T m = tabs(a);
  return b < T(0) ? -m : m;
}
// x and y of opposite strict signs (x * y < 0 without forming the product)
template <typename T> __device__ __forceinline__ bool opposite(T x, T y) {
  return (x > T(0) && y < T(0)) || (x < T(0) && y > T(0));
}
template <typename T> __device__ __forceinline__ bool same_sign(T x, T y) {
  return (x > T(0) && y > T(0)) || (x < T(0) && y < T(0));
}

// CW84 eq. 1.10 in perturbation form with selects in place of branches
template <typename T> __device__ __forceinline__ void cw84_sel(T& bl, T& br) {
  const bool flat = !opposite(bl, br);
  const T d = br - bl;
  const T t = T(3) * d * (bl + br);
  const T d2 = d * d;
  const bool lo = -t > d2, hi = !lo && t > d2;
  const T nbl = lo ? T(-2) * br : bl, nbr = hi ? T(-2) * bl : br;
  bl = flat ? T(0) : nbl;
  br = flat ? T(0) : nbr;
}

// kord 9: the limited value of raw interface a at u (0..km), given the
// means of layers u-2, u-1, u, u+1 (read only where they exist: the top
// interface reads layers 0, 1 as qb, qp1, the bottom one km-2, km-1 as qm2, qa)
template <typename T>
__device__ __forceinline__ T k9_interface(T a, int u, int km, int iv, T floor_v, T qm2, T qa, T qb, T qp1) {
  if (u <= 0) return clamp2(a, qb, qp1);
  if (u >= km) return iv == -2 ? a : clamp2(a, qm2, qa);
  const T dc = qb - qa;
  const T dl = u > 1 ? qa - qm2 : dc;
  const T dr = u < km - 1 ? qp1 - qb : dc;
  const T lo = tmin(qa, qb), hi = tmax(qa, qb);
  const bool mono = same_sign(dl, dr);
  const bool near_max = !mono && dl > T(0);
  const T below = tmin(a, hi);
  return mono ? tmin(tmax(a, lo), hi) : (near_max ? tmax(a, lo) : (iv >= 0 ? tmax(below, floor_v) : below));
}

// the same through a layer functor q(k): the end interfaces take their
// layers from the column ends
template <typename T, class QF>
__device__ __forceinline__ T k9_interface_f(T a, int u, int km, int iv, T floor_v, QF q) {
  if (u <= 0) return k9_interface(a, 0, km, iv, floor_v, T(0), T(0), q(0), q(1));
  if (u >= km) return k9_interface(a, km, km, iv, floor_v, q(km - 2), q(km - 1), T(0), T(0));
  return k9_interface(a, u, km, iv, floor_v, u > 1 ? q(u - 2) : T(0), q(u - 1), q(u), u < km - 1 ? q(u + 1) : T(0));
}

// kord 4: half-increment slope of layer k in 1..km-2 from the means and
// thicknesses of layers k-1, k, k+1
template <typename T>
__device__ __forceinline__ T ppm_slope(T qm, T q0, T qp, T d0, T d1, T d2) {
  const T dq = d1 / (d0 + d1 + d2) * ((T(2) * d0 + d1) / (d2 + d1) * (qp - q0) + (d1 + T(2) * d2) / (d0 + d1) * (q0 - qm));
  const T mx = tmax(tmax(qm, q0), qp) - q0;
  const T mn = q0 - tmin(tmin(qm, q0), qp);
  return sign_of(tmin(tmin(T(0.5) * tabs(dq), mx), mn), dq);
}
template <typename T, class QF, class HF>
__device__ __forceinline__ T ppm_slope_f(int k, int km, QF q, HF h) {
  if (k < 1 || k > km - 2) return T(0);
  return ppm_slope(q(k - 1), q(k), q(k + 1), h(k - 1), h(k), h(k + 1));
}

// interface between an end layer (q0, h0) and the next (q1, h1) from the
// parabola through those means and the one after them (q2, h2)
template <typename T>
__device__ __forceinline__ T quad3_interface(T q0, T q1, T q2, T h0, T h1, T h2) {
  const T w0 = h1 * (h1 + h2) / ((h0 + h1) * (h0 + h1 + h2));
  const T w2 = -h0 * h1 / ((h0 + h1 + h2) * (h1 + h2));
  const T w1 = T(1) - w0 - w2;
  return w0 * q0 + w1 * q1 + w2 * q2;
}

// kord 4: CW84 eq. 1.6 at interface u in 2..km-2 (between layers j = u-1 and
// u: means q0, q1) from the thicknesses of layers u-2..u+1 and the slopes
// dml, dmr of layers u-1, u
template <typename T>
__device__ __forceinline__ T ppm_interface_inner(T q0, T q1, T dml, T dmr, T hm, T h0, T h1, T h2) {
  const T s01 = h0 + h1, sall = hm + h0 + h1 + h2;
  const T c0 = h0 / s01;
  const T c1 = T(2) * h1 * h0 / s01 * ((hm + h0) / (T(2) * h0 + h1) - (h2 + h1) / (T(2) * h1 + h0)) / sall;
  const T c2 = h0 * (hm + h0) / (T(2) * h0 + h1) / sall;
  const T c3 = h1 * (h1 + h2) / (h0 + T(2) * h1) / sall;
  return q0 + (c0 + c1) * (q1 - q0) - (T(2) * c2) * dmr + (T(2) * c3) * dml;
}

// kord 4: interface u (0..km); dml, dmr: the slopes of layers u-1 and u
template <typename T, class QF, class HF>
__device__ __forceinline__ T ppm_interface(int u, int km, int iv, T qs, T dml, T dmr, QF q, HF h) {
  if (km == 2) {
    const T a1 = (q(0) * h(1) + q(1) * h(0)) / (h(0) + h(1));
    return u <= 0 ? T(2) * q(0) - a1 : (u == 1 ? a1 : (iv == -2 ? qs : T(2) * q(1) - a1));
  }
  if (u <= 1) {
    const T a1 = clamp2(quad3_interface(q(0), q(1), q(2), h(0), h(1), h(2)), q(0), q(1));
    return u == 1 ? a1 : T(2) * q(0) - a1;
  }
  if (u >= km - 1) {
    const T b1 = clamp2(quad3_interface(q(km - 1), q(km - 2), q(km - 3), h(km - 1), h(km - 2), h(km - 3)),
                        q(km - 2), q(km - 1));
    return u == km - 1 ? b1 : (iv == -2 ? qs : T(2) * q(km - 1) - b1);
  }
  return ppm_interface_inner(q(u - 1), q(u), dml, dmr, h(u - 2), h(u - 1), h(u), h(u + 1));
}

// a / b for the positivity scaling: FP32 columns take the fast reciprocal
// form (2 ulp; the scaling is continuous, so this moves results by rounding
// only), FP64 and tangent-linear columns the exact division
template <typename T> __device__ __forceinline__ T pos_div(T a, T b) { return a / b; }
template <> __device__ __forceinline__ float pos_div<float>(float a, float b) { return __fdividef(a, b); }

// Positivity for iv >= 0 (Zhang & Shu 2010 scaling, continuous in q): when an
// edge or the interior minimum q + s6/12 + da^2/(4 s6) (s6 < -|da|) lies
// below the floor, the deviations are scaled by (q - floor)/(q - min) (0 when
// q is below the floor).  The interior test is multiplied through by 12 s6:
// 12 s6 (q - floor) + s6^2 + 3 da^2 > 0.  Layers that need it are rare, so the
// divisions sit in a branch.  FP32 columns scale by a factor smaller by
// 2^-21, which keeps the fast division's result at or above the floor.
template <typename T>
__device__ __forceinline__ void positivity(T qk, T floor_v, T& bl, T& br) {
  const T s6 = T(-3) * (bl + br), da = br - bl;
  const bool inner = -s6 > tabs(da);
  const bool low = (qk + bl < floor_v) || (qk + br < floor_v) ||
                   (inner && T(12) * s6 * (qk - floor_v) + s6 * s6 + T(3) * da * da > T(0));
  if (low) {
    T pmin = tmin(qk + bl, qk + br);
    if (inner) pmin = tmin(pmin, qk + pos_div(s6, T(12)) + pos_div(da * da, T(4) * s6));
    T lam = qk > floor_v ? pos_div(qk - floor_v, qk - pmin) : T(0);
    if (Single<T>::value) lam = lam * T(1.0 - 1.0 / (1 << 21));
    bl = lam * bl;
    br = lam * br;
  }
}

// Constraint of an interior layer k (2 <= k <= km-3; see the header) on its
// edge deviations bl = aL - q, br = aR - q (kord 9: edges after k9_interface;
// kord 4: the PPM interfaces and the layer's slope dmk), with the means of
// layers k-2..k+2.
template <typename T, int KORD>
__device__ __forceinline__ void interior_constraint(T qm2, T qm1, T qk, T qp1, T qp2, T dmk, T& bl, T& br) {
  if (KORD == 9) {
    const T Dm = qm1 - qm2, D0 = qk - qm1, D1 = qp1 - qk, D2 = qp2 - qp1;
    const bool flat = opposite(D0, D1) && (opposite(Dm, D0) || opposite(D1, D2));
    const bool nonmono = T(3) * tabs(bl + br) > tabs(br - bl);
    const T pr = T(2) * D0, lr = pr - T(1.5) * Dm;
    const T pl = T(-2) * D1, ll = pl + T(1.5) * D2;
    const T brc = tmin(tmax(br, tmin(tmin(T(0), pr), lr)), tmax(tmax(T(0), pr), lr));
    const T blc = tmin(tmax(bl, tmin(tmin(T(0), pl), ll)), tmax(tmax(T(0), pl), ll));
    bl = flat ? T(0) : (nonmono ? blc : bl);
    br = flat ? T(0) : (nonmono ? brc : br);
  } else {
    const T xt = T(2) * dmk;
    const T ax = tabs(xt);
    bl = -sign_of(tmin(ax, tabs(bl)), xt);
    br = sign_of(tmin(ax, tabs(br)), xt);
  }
}

// Parabola of layer k (see the header) from its edges aL, aR and the means of
// layers k-2..k+2 (read only for interior layers): the two layers at each
// end take CW84, the others interior_constraint; then the floor.
template <typename T, int KORD>
__device__ __forceinline__ Profile<T> layer_profile(int k, int km, T qm2, T qm1, T qk, T qp1, T qp2, T aL, T aR,
                                                    T dmk, int iv, T floor_v) {
  T bl = aL - qk, br = aR - qk;
  if (k < 2 || k > km - 3) cw84_sel(bl, br);
  else interior_constraint<T, KORD>(qm2, qm1, qk, qp1, qp2, dmk, bl, br);
  if (iv >= 0) positivity(qk, floor_v, bl, br);
  return Profile<T>{qk, qk + bl, qk + br, T(-3) * (bl + br)};
}

// the same through a layer functor q(k)
template <typename T, int KORD, class QF>
__device__ __forceinline__ Profile<T> layer_profile_f(int k, int km, T qk, T aL, T aR, T dmk, int iv, T floor_v,
                                                      QF q) {
  const bool inner = k >= 2 && k <= km - 3;
  return layer_profile<T, KORD>(k, km, inner ? q(k - 2) : qk, inner ? q(k - 1) : qk, qk, inner ? q(k + 1) : qk,
                                inner ? q(k + 2) : qk, aL, aR, dmk, iv, floor_v);
}

}  // namespace fv3g
