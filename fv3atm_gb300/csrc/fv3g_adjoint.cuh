// fv3g_adjoint.cuh -- the linearised transport step of the six-tile state
// (tracer_2d substeps of fv_tracer2d.F90 with fv_tp_2d / xppm / yppm /
// copy_corners of tp_core.F90, then the map1_ppm remap of fv_mapz.F90), in
// tangent-linear and hand-written reverse (adjoint) form, FP64.
//
// The trajectory of a substep is recomputed from a checkpoint of its input
// field (halo strips filled): the two corner-filled copies, the inner-sweep
// fluxes and the inner-updated lines q_i and q_j, and for each of the four
// PPM sweeps (inner x on the dir-1 copy, inner y on the dir-2 copy, outer x
// on q_i, outer y on q_j) the weights of every face flux on its six cells,
// flux(f) = sum_s W[s](f) x(f-3+s), with the 2-dx filter (hord 1, 5) and
// the limiter branches (hord 8) frozen at the trajectory.  The tangent-linear
// substep applies those stencils forward; the adjoint gathers through their
// transposes cell by cell (no atomics: a cell sums the faces whose stencils
// hold it), then moves the adjoints of the corner blocks to the halo cells
// they were rotated from and those of the halo strips to the neighbouring
// tiles' cells they were copied from.
#pragma once

#include "fv3g_dual.cuh"
#include "fv3g_internal.cuh"

namespace fv3g {

// Planes of the state: q-shaped arrays hold nt*nq*npz planes [tile][tracer]
// [level]; per-level fields nt*npz planes [tile][level]; metrics nt planes.
struct LinArgs {
  PlaneGeom pg;
  long long P;  // elements per plane
  int is, ie, js, je;      // compute domain (tile indices)
  int isd, ied, jsd, jed;  // data domain
  int npx, npy;            // tile cells + 1 per direction
  int ew, ee, es, en;      // cube-face edge faces of the x lines (ew, ee) and y lines (es, en), or NO_EDGE
  int corners;             // copy_corners blocks filled: bit 0 sw, 1 se, 2 nw, 3 ne (0 on nested tiles)
  int n, nt, nq, npz;      // six-tile state: tile size (halo transpose), tiles, tracers, levels
  int hord;
  double lim_fac;
  Topo topo;
  // frozen inputs of the substep (per-level planes, scaled by 1/nsplt)
  const double *cx, *cy, *xfx, *yfx, *mfx, *mfy;  // mfx / mfy: the weights of the face fluxes (times 0.5)
  const double *ra_x, *ra_y;  // optional; else area + xfx(i) - xfx(i+1), area + yfx(j) - yfx(j+1)
  const double *dp1, *dp2;  // layer thickness at the substep's start and end
  const double *area, *rarea, *dxa, *dya;
};

// Trajectory of one substep and its face weights (all planes at once).
struct LinTraj {
  double *qc1, *qc2;  // input with the corner blocks filled for x (1) and y (2) sweeps
  double *qi, *qj;    // inner-updated lines: rows js..je (q_i), columns is..ie (q_j)
  double *fx2, *fy2;  // inner-sweep fluxes (values)
  double *wxi, *wyi, *wxo, *wyo;  // face weights, 6 planes-sets each: w[s * nplanes * P + plane * P + p]
};

// Work planes of the tangent-linear / adjoint substep (q-shaped each).
struct LinWork {
  double *a1, *a2;    // corner-filled tangents / their adjoints (dir 1, dir 2)
  double *ai, *aj;    // tangents / adjoints of q_i, q_j
  double *gx, *gy;    // adjoint: outer-sweep flux adjoints 0.5 mfx FX_ad, 0.5 mfy FY_ad
  double *fx2, *fy2;  // tangents / adjoints of the inner-sweep fluxes
};

// the arguments of the six-tile state's substeps (n cells per tile edge)
LinArgs lin_state_args(const PlaneGeom& pg, long long P, int n, int nt, int nq, int npz, int hord, double lim_fac,
                       const Topo& topo);

// trajectory of the substep whose halo-filled input is q
int lin_trajectory(const LinArgs& a, const double* q, const LinTraj& tr, cudaStream_t s);
// tangent-linear substep: dq (halo strips filled) -> dq_out (interior cells)
int lin_substep_tl(const LinArgs& a, const LinTraj& tr, const LinWork& w, const double* dq, double* dq_out,
                   cudaStream_t s);
// adjoint substep: q_ad_out (interior cells of the substep's output) ->
// q_ad_in (interior cells of its input; halo cells zero)
int lin_substep_ad(const LinArgs& a, const LinTraj& tr, const LinWork& w, const double* q_ad_out, double* q_ad_in,
                   cudaStream_t s);

// fv_tp_2d's adjoint from its flux adjoints (one plane; fluxes 0.5 (outer +
// inner) times a.mfx / a.mfy): q_ad (data domain) += J^T (fx_ad, fy_ad).
// d6x / d6y (may be null): del-2 damping flux weights, the damping flux
// through a face being d6 times the difference of the two cells beside it
// (x: q(i-1) - q(i); y: q(j-1) - q(j)).
int lin_fluxes_ad(const LinArgs& a, const LinTraj& tr, const LinWork& w, const double* fx_ad, const double* fy_ad,
                  const double* d6x, const double* d6y, double* q_ad, cudaStream_t s);

// Adjoint of the kord-4 remap of every interior column of the state: q_ad
// (the source field's adjoint, q-shaped) = J^T q2_ad at the trajectory q
// (Lagrangian levels of thickness dp) remapped onto ak + bk ps; q2_ad is
// read only.  iv: map1_ppm's iv (-1..1); q_min: the floor of iv 1.
int lin_remap_ad(const double* q, const double* dp, const double* ak, const double* bk, const double* q2_ad,
                 double* q_ad, PlaneGeom pg, long long P, int n, int nt, int nq, int km, int kn, int iv,
                 double q_min, int kord, cudaStream_t s);

// The hand-written column adjoint of the drop-in map1_ppm (kord 4): one row
// of columns in [level][column] layout, pe1/pe2 the interface pressures;
// q1_ad += J^T q2_ad.
int lin_remap_ad_rows(const double* q1, const double* pe1, const double* pe2, const double* qs, const double* q2_ad,
                      double* q1_ad, int ncol, int km, int kn, int iv, int kord, cudaStream_t s);

// (value, tangent) planes from value and tangent arrays (d may be null: zero
// tangent), and the tangents back out
int lin_pack_dual(Dual<double>* out, const double* v, const double* d, long long n, cudaStream_t s);
int lin_unpack_tangent(const Dual<double>* in, double* d, long long n, cudaStream_t s);

}  // namespace fv3g
