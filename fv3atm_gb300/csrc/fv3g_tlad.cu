// fv3g_tlad.cu -- tangent-linear and adjoint entries of the transport path:
// fv3g_fv_tp_2d_tl / fv3g_fv_tp_2d_ad (fv_tp_2d of tp_core.F90) and
// fv3g_map1_ppm_tl / fv3g_map1_ppm_ad (map1_ppm of fv_mapz.F90), with the
// Courant numbers, mass fluxes and pressures frozen and every limiter branch
// frozen at the trajectory.
//
// The tangent-linear models are the forward kernels instantiated on
// Dual<double> (value, tangent) planes.  The adjoints are hand-written
// reverse sweeps (fv3g_adjoint.cu):
//   * fv_tp_2d: the face weights of the four PPM sweeps on the trajectory,
//     then the transposed stencils gathered cell by cell, the inner updates
//     transposed, and the copy_corners fills transposed (del-2 damping, nord
//     0, transposed as its two-cell face differences);
//   * map1_ppm, kord 4: the column reversed (integration over the overlaps,
//     the layer parabolas, the PPM interfaces and slopes).  kord 9, whose
//     interfaces solve a tridiagonal system per column, runs the km unit
//     directions as km fields of one tangent-linear launch.
// Adjoint convention (as generated adjoint code): input adjoints are
// incremented, output adjoints are consumed and set to zero.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "fv3g_adjoint.cuh"
#include "fv3g_hostio.cuh"
#include "fv3g_remap.cuh"

namespace {

using D2 = Dual<double>;

__global__ void k_pack_dual(D2* out, const double* v, const double* d, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = D2(v[i], d ? d[i] : 0.0);
}

__global__ void k_unpack_dual(const D2* in, double* v, double* d, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (v) v[i] = in[i].v;
    if (d) d[i] = in[i].d;
  }
}

unsigned grid_1d(long long n) { return (unsigned)std::min<long long>((n + 255) / 256, 4096); }

int check_tp_args(const fv3g_bounds* bd, int npx, int npy, int hord, const fv3g_grid* grid, double lim_fac,
                  const double* mfx, const double* mass, double damp_c) {
  CHECK(check_bounds(bd, npx, npy));
  if (!grid || !grid->dxa || !grid->dya || !grid->area) return set_error(FV3G_E_ARG, "grid needs dxa, dya, area");
  if (hord != 1 && hord != 5 && hord != 8)
    return set_error(FV3G_E_UNSUPPORTED, "hord %d not implemented (1, 5 and 8 are)", hord);
  if (hord == 1 && !(lim_fac > 0.0)) return set_error(FV3G_E_ARG, "hord 1 needs lim_fac > 0 (got %g)", lim_fac);
  return 0;
}

// Damping of the tangent-linear / adjoint fv_tp_2d (as upstream: damp_c > 1e-4,
// with mass fluxes only if mass is given): del-2 only.
int check_tp_damping(bool damping, int nord, const fv3g_grid* grid) {
  if (!damping) return 0;
  if (nord != 0)
    return set_error(FV3G_E_UNSUPPORTED, "the tangent-linear / adjoint fv_tp_2d damps with nord 0 only (got %d)",
                     nord);
  if (!grid->del6_u || !grid->del6_v) return set_error(FV3G_E_ARG, "tracer damping needs grid del6_u and del6_v");
  if (!(grid->da_min > 0.0)) return set_error(FV3G_E_ARG, "tracer damping needs grid da_min > 0");
  return 0;
}

// The frozen damping inputs (del6_u, del6_v, mass) as value planes with zero
// tangent, and the damping arguments of the tangent-linear launch.
int damping_args(AdvArgs<D2>& ad, D2* d6u, D2* d6v, D2* dms, double* stage, const PlaneGeom& pg,
                 const fv3g_bounds* bd, const fv3g_grid* grid, const double* mfx, const double* mass, double damp_c,
                 cudaStream_t s) {
  const long long P = pg.plane();
  const int isd = bd->isd, ied = bd->ied, jsd = bd->jsd, jed = bd->jed;
  struct Item {
    D2* dst;
    const double* src;
    int ihi, jhi;
  } items[] = {{d6u, grid->del6_u, ied, jed + 1},
               {d6v, grid->del6_v, ied + 1, jed},
               {dms, mfx ? mass : nullptr, ied, jed}};
  for (const Item& it : items) {
    if (!it.src) continue;
    FV3G_CUDA(cudaMemsetAsync(stage, 0, sizeof(double) * P, s));
    CHECK(h2d_planes(stage, pg, it.src, isd, it.ihi, jsd, it.jhi, 1, s));
    k_pack_dual<<<grid_1d(P), 256, 0, s>>>(it.dst, stage, nullptr, P);
    FV3G_CUDA(cudaGetLastError());
  }
  ad.del6_u = d6u;
  ad.del6_v = d6v;
  ad.damp = D2(damp_coefficient(damp_c, grid->da_min, 0));
  ad.nord = 0;
  ad.damp_mass = mfx != nullptr;
  ad.dp1 = mfx ? dms : nullptr;
  return 0;
}

// The frozen inputs of fv_tp_2d as value planes with zero tangent, and the
// argument block of the flux-mode kernel on them.
struct FrozenTp {
  D2 *cx, *cy, *xf, *yf, *rx, *ry, *mx, *my, *dxa, *dya, *area;
};

int upload_frozen(FrozenTp& f, double* stage, const PlaneGeom& pg, const fv3g_bounds* bd, const double* crx,
                  const double* cry, const double* xfx, const double* yfx, const double* ra_x, const double* ra_y,
                  const double* mfx, const double* mfy, const fv3g_grid* grid, cudaStream_t s) {
  const long long P = pg.plane();
  const int is = bd->is, ie = bd->ie, js = bd->js, je = bd->je, isd = bd->isd, ied = bd->ied, jsd = bd->jsd,
            jed = bd->jed;
  struct Item {
    D2* dst;
    const double* src;
    int ilo, ihi, jlo, jhi;
  } items[] = {{f.cx, crx, is, ie + 1, jsd, jed},        {f.cy, cry, isd, ied, js, je + 1},
               {f.xf, xfx, is, ie + 1, jsd, jed},        {f.yf, yfx, isd, ied, js, je + 1},
               {f.rx, ra_x, is, ie, jsd, jed},           {f.ry, ra_y, isd, ied, js, je},
               // without mass fluxes the area fluxes weight the result, as upstream
               {f.mx, mfx ? mfx : xfx, is, ie + 1, mfx ? js : jsd, mfx ? je : jed},
               {f.my, mfy ? mfy : yfx, mfy ? is : isd, mfy ? ie : ied, js, je + 1},
               {f.dxa, grid->dxa, isd, ied, jsd, jed},   {f.dya, grid->dya, isd, ied, jsd, jed},
               {f.area, grid->area, isd, ied, jsd, jed}};
  for (const Item& it : items) {
    FV3G_CUDA(cudaMemsetAsync(stage, 0, sizeof(double) * P, s));
    CHECK(h2d_planes(stage, pg, it.src, it.ilo, it.ihi, it.jlo, it.jhi, 1, s));
    k_pack_dual<<<grid_1d(P), 256, 0, s>>>(it.dst, stage, nullptr, P);
    FV3G_CUDA(cudaGetLastError());
  }
  return 0;
}

AdvArgs<D2> tp_args(const FrozenTp& f, const PlaneGeom& pg, const fv3g_bounds* bd, int npx, int npy, int ntracer) {
  AdvArgs<D2> a{};
  a.cx = f.cx; a.cy = f.cy; a.xfx = f.xf; a.yfx = f.yf;
  a.mfx = f.mx; a.mfy = f.my;
  a.area = f.area; a.rarea = f.area; a.dxa = f.dxa; a.dya = f.dya;
  a.ra_x = f.rx; a.ra_y = f.ry;
  a.pg = pg;
  a.is = bd->is; a.ie = bd->ie; a.js = bd->js; a.je = bd->je;
  a.npx = npx; a.npy = npy;
  a.nq = ntracer; a.npz = 1;
  a.sQq = pg.plane(); a.sQk = pg.plane();
  a.cube = 0;
  a.sFlux = pg.plane();
  return a;
}

// One row of map1_ppm columns on the device, [level][column] layout, as
// value/tangent pairs; nfield copies of the trajectory, field f carrying the
// tangent tan(f, k, c).
struct RowRemap {
  int km, kn, ncol, nfield;
  D2 *q1, *q2, *scratch;
  double *pe1, *pe2, *qs;
  unsigned char* sched;
};

int row_remap_setup(RowRemap& R, int km, int kn, int ncol, int nfield, const double* pe1, const double* pe2,
                    const double* qs, cudaStream_t* s) {
  R.km = km; R.kn = kn; R.ncol = ncol; R.nfield = nfield;
  const size_t scr = remap_scratch_bytes(ncol, sizeof(D2));
  CHECK(g_ctx.begin(padded((size_t)nfield * km * ncol, 16) + padded((size_t)nfield * kn * ncol, 16) +
                    padded((size_t)(km + 1) * ncol, 8) + padded((size_t)(kn + 1) * ncol, 8) + padded(ncol, 8) +
                    scr + 1024));
  *s = g_ctx.stream;
  R.q1 = g_ctx.take<D2>((size_t)nfield * km * ncol);
  R.q2 = g_ctx.take<D2>((size_t)nfield * kn * ncol);
  R.pe1 = g_ctx.take<double>((size_t)(km + 1) * ncol);
  R.pe2 = g_ctx.take<double>((size_t)(kn + 1) * ncol);
  R.qs = g_ctx.take<double>(ncol);
  R.scratch = g_ctx.take<D2>((size_t)ncol * (KMAX + 1) * 6);
  R.sched = g_ctx.take<unsigned char>((size_t)ncol * (KMAX + 1));
  FV3G_CUDA(cudaMemcpyAsync(R.pe1, pe1, sizeof(double) * (km + 1) * ncol, cudaMemcpyHostToDevice, *s));
  FV3G_CUDA(cudaMemcpyAsync(R.pe2, pe2, sizeof(double) * (kn + 1) * ncol, cudaMemcpyHostToDevice, *s));
  if (qs) FV3G_CUDA(cudaMemcpyAsync(R.qs, qs, sizeof(double) * ncol, cudaMemcpyHostToDevice, *s));
  return 0;
}

int row_remap_run(const RowRemap& R, const double* qs, int iv, int kord, cudaStream_t s) {
  RemapArgs<D2> r{};
  r.q_in = R.q1;
  r.q_out = R.q2;
  r.sQk = R.ncol;
  r.sQq = (long long)R.km * R.ncol;
  r.sQt = 0;
  r.sQqo = (long long)R.kn * R.ncol;
  r.nfield = R.nfield;
  r.pe1 = R.pe1;
  r.pe2 = R.pe2;
  r.qs = qs ? R.qs : nullptr;
  r.pg.isd = 0; r.pg.jsd = 0; r.pg.pitch = R.ncol; r.pg.rows = 1;
  r.i1 = 0; r.j1 = 0; r.ni = R.ncol; r.nj = 1;
  r.ncol = R.ncol;
  r.km = R.km; r.kn = R.kn; r.iv = iv; r.q_min = 0.0;
  r.scratch = R.scratch;
  r.sched = R.sched;
  return launch_remap_tl(r, kord, s);
}

int check_map_args(int km, int kn, int i1, int i2, int j, int ibeg, int iend, int jbeg, int jend) {
  if (km < 1 || kn < 1 || km > KMAX || kn > KMAX) return set_error(FV3G_E_ARG, "remap supports 1..%d layers", KMAX);
  if (i1 < ibeg || i2 > iend || i2 < i1 || j < jbeg || j > jend) return set_error(FV3G_E_ARG, "row out of bounds");
  return 0;
}

}  // namespace

extern "C" {

int fv3g_map1_ppm_tl(int km, const double* pe1, const double* q1, const double* q1_tl, const double* qs, int kn,
                     const double* pe2, double* q2, double* q2_tl, int i1, int i2, int j, int ibeg, int iend,
                     int jbeg, int jend, int iv, int kord) {
  CHECK(check_map_args(km, kn, i1, i2, j, ibeg, iend, jbeg, jend));
  if (!pe1 || !q1 || !q1_tl || !pe2 || !q2_tl) return set_error(FV3G_E_ARG, "null array argument");
  if (iv == -2 && qs == nullptr) return set_error(FV3G_E_ARG, "iv -2 needs the surface values qs");
  const int ncol = i2 - i1 + 1;
  const size_t nib = (size_t)(iend - ibeg + 1), plane = nib * (size_t)(jend - jbeg + 1);
  const size_t row = (size_t)(j - jbeg) * nib;
  std::vector<D2> h1((size_t)km * ncol), h2((size_t)kn * ncol);
  for (int k = 0; k < km; ++k)
    for (int c = 0; c < ncol; ++c) {
      const size_t o = (size_t)(i1 + c - ibeg) + row + k * plane;
      h1[(size_t)k * ncol + c] = D2(q1[o], q1_tl[o]);
    }
  RowRemap R;
  cudaStream_t s;
  CHECK(row_remap_setup(R, km, kn, ncol, 1, pe1, pe2, qs, &s));
  FV3G_CUDA(cudaMemcpyAsync(R.q1, h1.data(), sizeof(D2) * h1.size(), cudaMemcpyHostToDevice, s));
  CHECK(row_remap_run(R, qs, iv, kord, s));
  FV3G_CUDA(cudaMemcpyAsync(h2.data(), R.q2, sizeof(D2) * h2.size(), cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  for (int k = 0; k < kn; ++k)
    for (int c = 0; c < ncol; ++c) {
      const size_t o = (size_t)(i1 + c - ibeg) + row + k * plane;
      if (q2) q2[o] = h2[(size_t)k * ncol + c].v;
      q2_tl[o] = h2[(size_t)k * ncol + c].d;
    }
  return 0;
}

int fv3g_map1_ppm_ad(int km, const double* pe1, const double* q1, double* q1_ad, const double* qs, int kn,
                     const double* pe2, double* q2_ad, int i1, int i2, int j, int ibeg, int iend, int jbeg, int jend,
                     int iv, int kord) {
  CHECK(check_map_args(km, kn, i1, i2, j, ibeg, iend, jbeg, jend));
  if (!pe1 || !q1 || !q1_ad || !pe2 || !q2_ad) return set_error(FV3G_E_ARG, "null array argument");
  if (iv == -2 && qs == nullptr) return set_error(FV3G_E_ARG, "iv -2 needs the surface values qs");
  const int ncol = i2 - i1 + 1;
  const size_t nib = (size_t)(iend - ibeg + 1), plane = nib * (size_t)(jend - jbeg + 1);
  const size_t row = (size_t)(j - jbeg) * nib;
  if (kord == 4 && km >= 3) {  // the hand-written reverse of the column remap
    std::vector<double> h1((size_t)km * ncol), h2((size_t)kn * ncol), ha((size_t)km * ncol, 0.0);
    std::vector<double> hq(qs ? (size_t)ncol : 0);
    for (int k = 0; k < km; ++k)
      for (int c = 0; c < ncol; ++c) h1[(size_t)k * ncol + c] = q1[(size_t)(i1 + c - ibeg) + row + k * plane];
    for (int k = 0; k < kn; ++k)
      for (int c = 0; c < ncol; ++c) h2[(size_t)k * ncol + c] = q2_ad[(size_t)(i1 + c - ibeg) + row + k * plane];
    CHECK(g_ctx.begin(padded((size_t)km * ncol, 8) * 2 + padded((size_t)kn * ncol, 8) +
                      padded((size_t)(km + 1) * ncol, 8) + padded((size_t)(kn + 1) * ncol, 8) + padded(ncol, 8)));
    cudaStream_t s = g_ctx.stream;
    double *d1 = g_ctx.take<double>((size_t)km * ncol), *da = g_ctx.take<double>((size_t)km * ncol);
    double *d2 = g_ctx.take<double>((size_t)kn * ncol), *p1 = g_ctx.take<double>((size_t)(km + 1) * ncol);
    double *p2 = g_ctx.take<double>((size_t)(kn + 1) * ncol), *dq = g_ctx.take<double>(ncol);
    FV3G_CUDA(cudaMemcpyAsync(d1, h1.data(), sizeof(double) * h1.size(), cudaMemcpyHostToDevice, s));
    FV3G_CUDA(cudaMemcpyAsync(d2, h2.data(), sizeof(double) * h2.size(), cudaMemcpyHostToDevice, s));
    FV3G_CUDA(cudaMemcpyAsync(p1, pe1, sizeof(double) * (km + 1) * ncol, cudaMemcpyHostToDevice, s));
    FV3G_CUDA(cudaMemcpyAsync(p2, pe2, sizeof(double) * (kn + 1) * ncol, cudaMemcpyHostToDevice, s));
    if (qs) FV3G_CUDA(cudaMemcpyAsync(dq, qs, sizeof(double) * ncol, cudaMemcpyHostToDevice, s));
    FV3G_CUDA(cudaMemsetAsync(da, 0, sizeof(double) * km * ncol, s));
    CHECK(lin_remap_ad_rows(d1, p1, p2, qs ? dq : nullptr, d2, da, ncol, km, kn, iv, kord, s));
    FV3G_CUDA(cudaMemcpyAsync(ha.data(), da, sizeof(double) * ha.size(), cudaMemcpyDeviceToHost, s));
    FV3G_CUDA(cudaStreamSynchronize(s));
    for (int k = 0; k < km; ++k)
      for (int c = 0; c < ncol; ++c) q1_ad[(size_t)(i1 + c - ibeg) + row + k * plane] += ha[(size_t)k * ncol + c];
    for (int t = 0; t < kn; ++t)
      for (int c = 0; c < ncol; ++c) q2_ad[(size_t)(i1 + c - ibeg) + row + t * plane] = 0.0;
    return 0;
  }
  // kord 9 (whose interfaces solve a tridiagonal system per column): field f
  // carries the unit tangent of source layer f through the tangent-linear remap
  std::vector<D2> h1((size_t)km * km * ncol);
  for (int f = 0; f < km; ++f)
    for (int k = 0; k < km; ++k)
      for (int c = 0; c < ncol; ++c)
        h1[((size_t)f * km + k) * ncol + c] = D2(q1[(size_t)(i1 + c - ibeg) + row + k * plane], k == f ? 1.0 : 0.0);
  RowRemap R;
  cudaStream_t s;
  CHECK(row_remap_setup(R, km, kn, ncol, km, pe1, pe2, qs, &s));
  FV3G_CUDA(cudaMemcpyAsync(R.q1, h1.data(), sizeof(D2) * h1.size(), cudaMemcpyHostToDevice, s));
  CHECK(row_remap_run(R, qs, iv, kord, s));
  std::vector<D2> jac((size_t)km * kn * ncol);  // [f][t][c] = d q2(t) / d q1(f)
  FV3G_CUDA(cudaMemcpyAsync(jac.data(), R.q2, sizeof(D2) * jac.size(), cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  for (int f = 0; f < km; ++f)
    for (int c = 0; c < ncol; ++c) {
      double acc = 0.0;
      for (int t = 0; t < kn; ++t)
        acc += jac[((size_t)f * kn + t) * ncol + c].d * q2_ad[(size_t)(i1 + c - ibeg) + row + t * plane];
      q1_ad[(size_t)(i1 + c - ibeg) + row + f * plane] += acc;
    }
  for (int t = 0; t < kn; ++t)
    for (int c = 0; c < ncol; ++c) q2_ad[(size_t)(i1 + c - ibeg) + row + t * plane] = 0.0;
  return 0;
}

int fv3g_fv_tp_2d_tl(const double* q, const double* q_tl, const double* crx, const double* cry, int npx, int npy,
                     int hord, double* fx, double* fx_tl, double* fy, double* fy_tl, const double* xfx,
                     const double* yfx, const fv3g_grid* grid, const fv3g_bounds* bd, const double* ra_x,
                     const double* ra_y, double lim_fac, const double* mfx, const double* mfy, const double* mass,
                     int nord, double damp_c) {
  CHECK(check_tp_args(bd, npx, npy, hord, grid, lim_fac, mfx, mass, damp_c));
  const bool damping = damp_c > 1e-4 && (mfx == nullptr || mass != nullptr);
  CHECK(check_tp_damping(damping, nord, grid));
  if (!q || !q_tl || !crx || !cry || !xfx || !yfx || !ra_x || !ra_y || !fx_tl || !fy_tl)
    return set_error(FV3G_E_ARG, "null array argument");
  const PlaneGeom pg = plane_for(bd);
  const size_t P = (size_t)pg.plane();
  CHECK(g_ctx.begin(3 * padded(P, 8) + 17 * padded(P, 16)));
  cudaStream_t s = g_ctx.stream;
  double *stage = g_ctx.take<double>(P), *qv = g_ctx.take<double>(P), *qd = g_ctx.take<double>(P);
  FrozenTp f;
  D2** slots[] = {&f.cx, &f.cy, &f.xf, &f.yf, &f.rx, &f.ry, &f.mx, &f.my, &f.dxa, &f.dya, &f.area};
  for (D2** sl : slots) *sl = g_ctx.take<D2>(P);
  D2 *dq = g_ctx.take<D2>(P), *dfx = g_ctx.take<D2>(P), *dfy = g_ctx.take<D2>(P);
  D2 *d6u = g_ctx.take<D2>(P), *d6v = g_ctx.take<D2>(P), *dms = g_ctx.take<D2>(P);
  FV3G_CUDA(cudaMemsetAsync(g_ctx.arena, 0, g_ctx.used, s));
  CHECK(upload_frozen(f, stage, pg, bd, crx, cry, xfx, yfx, ra_x, ra_y, mfx, mfy, grid, s));
  CHECK(h2d_planes(qv, pg, q, bd->isd, bd->ied, bd->jsd, bd->jed, 1, s));
  CHECK(h2d_planes(qd, pg, q_tl, bd->isd, bd->ied, bd->jsd, bd->jed, 1, s));
  k_pack_dual<<<grid_1d(P), 256, 0, s>>>(dq, qv, qd, P);
  FV3G_CUDA(cudaGetLastError());
  AdvArgs<D2> a = tp_args(f, pg, bd, npx, npy, 1);
  a.q_in = dq;
  a.corners = corner_mask(grid);
  a.nested = grid->nested;
  a.lim_fac = lim_fac;
  a.fx_out = dfx;
  a.fy_out = dfy;
  CHECK(launch_substep_tl(a, hord, s));
  if (damping) {
    AdvArgs<D2> ad = a;
    CHECK(damping_args(ad, d6u, d6v, dms, stage, pg, bd, grid, mfx, mass, damp_c, s));
    CHECK(launch_damp_tl(ad, s));
  }
  double* out_v = qv;
  double* out_d = qd;
  const int is = bd->is, ie = bd->ie, js = bd->js, je = bd->je;
  k_unpack_dual<<<grid_1d(P), 256, 0, s>>>(dfx, out_v, out_d, P);
  FV3G_CUDA(cudaGetLastError());
  if (fx) CHECK(d2h_planes(fx, out_v, pg, is, ie + 1, js, je, 1, s));
  CHECK(d2h_planes(fx_tl, out_d, pg, is, ie + 1, js, je, 1, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  k_unpack_dual<<<grid_1d(P), 256, 0, s>>>(dfy, out_v, out_d, P);
  FV3G_CUDA(cudaGetLastError());
  if (fy) CHECK(d2h_planes(fy, out_v, pg, is, ie, js, je + 1, 1, s));
  CHECK(d2h_planes(fy_tl, out_d, pg, is, ie, js, je + 1, 1, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  return 0;
}

int fv3g_fv_tp_2d_ad(const double* q, double* q_ad, const double* crx, const double* cry, int npx, int npy, int hord,
                     double* fx_ad, double* fy_ad, const double* xfx, const double* yfx, const fv3g_grid* grid,
                     const fv3g_bounds* bd, const double* ra_x, const double* ra_y, double lim_fac,
                     const double* mfx, const double* mfy, const double* mass, int nord, double damp_c) {
  CHECK(check_tp_args(bd, npx, npy, hord, grid, lim_fac, mfx, mass, damp_c));
  const bool damping = damp_c > 1e-4 && (mfx == nullptr || mass != nullptr);
  CHECK(check_tp_damping(damping, nord, grid));
  if (!q || !q_ad || !crx || !cry || !xfx || !yfx || !ra_x || !ra_y || !fx_ad || !fy_ad)
    return set_error(FV3G_E_ARG, "null array argument");
  const PlaneGeom pg = plane_for(bd);
  const size_t P = (size_t)pg.plane();
  const int is = bd->is, ie = bd->ie, js = bd->js, je = bd->je, isd = bd->isd, ied = bd->ied, jsd = bd->jsd,
            jed = bd->jed;
  CHECK(g_ctx.begin(60 * padded(P, 8)));
  cudaStream_t s = g_ctx.stream;
  // frozen planes and the trajectory of the call
  double *qv = g_ctx.take<double>(P), *cx = g_ctx.take<double>(P), *cy = g_ctx.take<double>(P);
  double *xf = g_ctx.take<double>(P), *yf = g_ctx.take<double>(P), *rx = g_ctx.take<double>(P);
  double *ry = g_ctx.take<double>(P), *wx = g_ctx.take<double>(P), *wy = g_ctx.take<double>(P);
  double *dxa = g_ctx.take<double>(P), *dya = g_ctx.take<double>(P), *area = g_ctx.take<double>(P);
  double *fxa = g_ctx.take<double>(P), *fya = g_ctx.take<double>(P), *qa = g_ctx.take<double>(P);
  double *d6x = g_ctx.take<double>(P), *d6y = g_ctx.take<double>(P);
  LinTraj tr{};
  LinWork w{};
  double** one[] = {&tr.qc1, &tr.qc2, &tr.qi, &tr.qj, &tr.fx2, &tr.fy2, &w.a1, &w.a2,
                    &w.ai, &w.aj, &w.gx, &w.gy, &w.fx2, &w.fy2};
  for (double** b : one) *b = g_ctx.take<double>(P);
  for (double** b : {&tr.wxi, &tr.wyi, &tr.wxo, &tr.wyo}) *b = g_ctx.take<double>(6 * P);
  FV3G_CUDA(cudaMemsetAsync(g_ctx.arena, 0, g_ctx.used, s));
  struct Item {
    double* dst;
    const double* src;
    int ilo, ihi, jlo, jhi;
  } items[] = {{qv, q, isd, ied, jsd, jed},
               {cx, crx, is, ie + 1, jsd, jed},
               {cy, cry, isd, ied, js, je + 1},
               {xf, xfx, is, ie + 1, jsd, jed},
               {yf, yfx, isd, ied, js, je + 1},
               {rx, ra_x, is, ie, jsd, jed},
               {ry, ra_y, isd, ied, js, je},
               // without mass fluxes the area fluxes weight the result, as upstream
               {wx, mfx ? mfx : xfx, is, ie + 1, mfx ? js : jsd, mfx ? je : jed},
               {wy, mfy ? mfy : yfx, mfy ? is : isd, mfy ? ie : ied, js, je + 1},
               {dxa, grid->dxa, isd, ied, jsd, jed},
               {dya, grid->dya, isd, ied, jsd, jed},
               {area, grid->area, isd, ied, jsd, jed},
               {fxa, fx_ad, is, ie + 1, js, je},
               {fya, fy_ad, is, ie, js, je + 1}};
  for (const Item& it : items) CHECK(h2d_planes(it.dst, pg, it.src, it.ilo, it.ihi, it.jlo, it.jhi, 1, s));
  if (damping) {
    // del-2 damping flux weights: d6 (difference across the face), times the
    // face mean of mass with mass fluxes, else times the damping coefficient
    const double damp = damp_coefficient(damp_c, grid->da_min, 0);
    const int nid = ied - isd + 1, njd = jed - jsd + 1;
    std::vector<double> hx((size_t)(ie - is + 2) * (je - js + 1)), hy((size_t)(ie - is + 1) * (je - js + 2));
    auto M = [&](int i, int j) { return mass[(size_t)(j - jsd) * nid + (i - isd)]; };
    for (int j = js; j <= je; ++j)
      for (int i = is; i <= ie + 1; ++i) {
        const double d6 = grid->del6_v[(size_t)(j - jsd) * (nid + 1) + (i - isd)];
        hx[(size_t)(j - js) * (ie - is + 2) + (i - is)] = d6 * (mfx ? 0.5 * damp * (M(i - 1, j) + M(i, j)) : damp);
      }
    for (int j = js; j <= je + 1; ++j)
      for (int i = is; i <= ie; ++i) {
        const double d6 = grid->del6_u[(size_t)(j - jsd) * nid + (i - isd)];
        hy[(size_t)(j - js) * (ie - is + 1) + (i - is)] = d6 * (mfx ? 0.5 * damp * (M(i, j - 1) + M(i, j)) : damp);
      }
    (void)njd;
    CHECK(h2d_planes(d6x, pg, hx.data(), is, ie + 1, js, je, 1, s));
    CHECK(h2d_planes(d6y, pg, hy.data(), is, ie, js, je + 1, 1, s));
  }
  LinArgs a{};
  a.pg = pg;
  a.P = (long long)P;
  a.is = is; a.ie = ie; a.js = js; a.je = je;
  a.isd = isd; a.ied = ied; a.jsd = jsd; a.jed = jed;
  a.npx = npx; a.npy = npy;
  a.ew = (!grid->nested && is == 1) ? 1 : NO_EDGE;
  a.ee = (!grid->nested && ie + 1 == npx) ? npx : NO_EDGE;
  a.es = (!grid->nested && js == 1) ? 1 : NO_EDGE;
  a.en = (!grid->nested && je + 1 == npy) ? npy : NO_EDGE;
  a.corners = grid->nested ? 0 : corner_mask(grid);
  a.nt = 1; a.nq = 1; a.npz = 1;
  a.hord = hord;
  a.lim_fac = lim_fac;
  a.cx = cx; a.cy = cy; a.xfx = xf; a.yfx = yf;
  a.mfx = wx; a.mfy = wy;
  a.ra_x = rx; a.ra_y = ry;
  a.area = area; a.dxa = dxa; a.dya = dya;
  CHECK(lin_trajectory(a, qv, tr, s));
  CHECK(lin_fluxes_ad(a, tr, w, fxa, fya, damping ? d6x : nullptr, damping ? d6y : nullptr, qa, s));
  // q_ad += J^T (fx_ad, fy_ad) over the caller's data domain; the flux adjoints are consumed
  const int ni = ied - isd + 1, nj = jed - jsd + 1;
  std::vector<double> h((size_t)ni * nj);
  CHECK(d2h_planes(h.data(), qa, pg, isd, ied, jsd, jed, 1, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  for (size_t e = 0; e < h.size(); ++e) q_ad[e] += h[e];
  std::fill(fx_ad, fx_ad + (size_t)(ie - is + 2) * (je - js + 1), 0.0);
  std::fill(fy_ad, fy_ad + (size_t)(ie - is + 1) * (je - js + 2), 0.0);
  return 0;
}

}  // extern "C"
