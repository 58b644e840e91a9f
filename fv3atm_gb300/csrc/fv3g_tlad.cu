// fv3g_tlad.cu -- tangent-linear and adjoint entries of the transport path:
// fv3g_fv_tp_2d_tl / fv3g_fv_tp_2d_ad (fv_tp_2d of tp_core.F90) and
// fv3g_map1_ppm_tl / fv3g_map1_ppm_ad (map1_ppm of fv_mapz.F90), with the
// Courant numbers, mass fluxes and pressures frozen and every limiter branch
// frozen at the trajectory (hord 5 and the unlimited parts have none).
//
// The tangent-linear model is the forward kernel instantiated on Dual<double>
// (value, tangent) planes.  The adjoint is assembled from tangent-linear runs
// in which the inputs are coloured so that every Jacobian entry is recovered
// exactly, then contracted with the output adjoints:
//   * fv_tp_2d: the fluxes depend on the x-sweep input (q with the dir-1
//     corner fill) through boxes of 6x1 (fx) and 7x6 (fy) cells, and on the
//     y-sweep input (dir-2 fill) through 6x7 (fx) and 1x6 (fy) boxes.  With
//     the corner fills taken out of the kernel (they are applied to the
//     trajectory and transposed afterwards), colouring the x input with
//     periods (7, 6) and the y input with (6, 7) gives each cell of a box its
//     own colour: 42 colours per input, run as 42 tracer planes of one launch.
//   * map1_ppm: a column's output depends on every source layer (the
//     interface values solve a tridiagonal system), so the km unit directions
//     run as km fields of one launch.
// Adjoint convention (as generated adjoint code): input adjoints are
// incremented, output adjoints are consumed and set to zero.
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

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

// ncolor planes of the trajectory; with tangent_on, tangent 1 on the cells of
// the plane's colour ((i - ilo) mod px) + px ((j - jlo) mod py), else 0.
__global__ void k_color_planes(D2* out, const double* traj, PlaneGeom pg, int ilo, int ihi, int jlo, int jhi, int px,
                               int py, int ncolor, int tangent_on) {
  const long long P = pg.plane();
  for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < P * ncolor;
       id += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(id / P);
    const long long p = id - (long long)c * P;
    const int i = pg.isd + (int)(p % pg.pitch), j = pg.jsd + (int)(p / pg.pitch);
    double d = 0.0;
    if (tangent_on && i >= ilo && i <= ihi && j >= jlo && j <= jhi)
      d = ((i - ilo) % px) + px * ((j - jlo) % py) == c ? 1.0 : 0.0;
    out[id] = D2(traj[p], d);
  }
}

struct FaceBox {  // faces (fi, fj) in [i+a0, i+a1] x [j+b0, j+b1] hold cell (i, j) in their stencil box
  int a0, a1, b0, b1;
};

// g(i, j) = sum over the faces whose box holds (i, j) of d flux / d q(i, j)
// (the tangent of the cell's colour plane) times the flux adjoint.
__global__ void k_gather_adjoint(double* g, const D2* fx, const D2* fy, const double* fxa, const double* fya,
                                 PlaneGeom pg, int ilo, int ihi, int jlo, int jhi, int px, int py, FaceBox bx,
                                 FaceBox by, int is, int ie, int js, int je) {
  const long long P = pg.plane();
  const int ni = ihi - ilo + 1, nj = jhi - jlo + 1;
  for (long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x; id < (long long)ni * nj;
       id += (long long)gridDim.x * blockDim.x) {
    const int i = ilo + (int)(id % ni), j = jlo + (int)(id / ni);
    const int c = ((i - ilo) % px) + px * ((j - jlo) % py);
    const D2* fxc = fx + (long long)c * P;
    const D2* fyc = fy + (long long)c * P;
    double s = 0.0;
    for (int fj = max(j + bx.b0, js); fj <= min(j + bx.b1, je); ++fj)
      for (int fi = max(i + bx.a0, is); fi <= min(i + bx.a1, ie + 1); ++fi) {
        const long long p = pg.at(fi, fj);
        s += fxc[p].d * fxa[p];
      }
    for (int fj = max(j + by.b0, js); fj <= min(j + by.b1, je + 1); ++fj)
      for (int fi = max(i + by.a0, is); fi <= min(i + by.a1, ie); ++fi) {
        const long long p = pg.at(fi, fj);
        s += fyc[p].d * fya[p];
      }
    g[pg.at(i, j)] += s;
  }
}

// Transpose of the copy_corners fill of direction dir: the adjoint of every
// cube-corner halo cell moves to the strip cell it was copied from.
__global__ void k_corners_adjoint(double* g, PlaneGeom pg, int npx, int npy, int corners, int dir) {
  const int id = threadIdx.x;
  if (id >= 36) return;
  const int c = id / 9, a = (id % 9) / 3 + 1, b = id % 3 + 1;
  if (!(corners & (1 << c))) return;
  const int su = (c & 1) ? 1 : -1, sv = (c & 2) ? 1 : -1;
  const int cx2 = su < 0 ? 1 : 2 * npx - 1, cy2 = sv < 0 ? 1 : 2 * npy - 1;
  const int U = su * (2 * a - 1), V = sv * (2 * b - 1);
  const bool plus = (dir == 1) ? (su == -sv) : (su == sv);
  const int U2 = plus ? -V : V, V2 = plus ? U : -U;
  const int i = (U + cx2) / 2, j = (V + cy2) / 2, is = (U2 + cx2) / 2, js = (V2 + cy2) / 2;
  if (i < pg.isd || j < pg.jsd || is < pg.isd || js < pg.jsd || i >= pg.isd + pg.pitch || is >= pg.isd + pg.pitch ||
      j >= pg.jsd + pg.rows || js >= pg.jsd + pg.rows)
    return;
  // corner cells and their sources are disjoint, and each source has one corner cell
  g[pg.at(is, js)] += g[pg.at(i, j)];
  g[pg.at(i, j)] = 0.0;
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
  // field f: the trajectory with the unit tangent of source layer f
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
  constexpr int NC = 42;  // colours per input: 7 x 6
  const PlaneGeom pg = plane_for(bd);
  const size_t P = (size_t)pg.plane();
  CHECK(g_ctx.begin(7 * padded(P, 8) + 14 * padded(P, 16) + 4 * padded(P * NC, 16)));
  cudaStream_t s = g_ctx.stream;
  double *stage = g_ctx.take<double>(P), *qx = g_ctx.take<double>(P), *qy = g_ctx.take<double>(P);
  double *fxa = g_ctx.take<double>(P), *fya = g_ctx.take<double>(P), *gx = g_ctx.take<double>(P);
  double* gy = g_ctx.take<double>(P);
  FrozenTp f;
  D2** slots[] = {&f.cx, &f.cy, &f.xf, &f.yf, &f.rx, &f.ry, &f.mx, &f.my, &f.dxa, &f.dya, &f.area};
  for (D2** sl : slots) *sl = g_ctx.take<D2>(P);
  D2 *in_x = g_ctx.take<D2>(P * NC), *in_y = g_ctx.take<D2>(P * NC), *fl = g_ctx.take<D2>(P * NC * 2);
  D2 *d6u = g_ctx.take<D2>(P), *d6v = g_ctx.take<D2>(P), *dms = g_ctx.take<D2>(P);
  FV3G_CUDA(cudaMemsetAsync(g_ctx.arena, 0, g_ctx.used, s));
  CHECK(upload_frozen(f, stage, pg, bd, crx, cry, xfx, yfx, ra_x, ra_y, mfx, mfy, grid, s));
  const int is = bd->is, ie = bd->ie, js = bd->js, je = bd->je, isd = bd->isd, ied = bd->ied, jsd = bd->jsd,
            jed = bd->jed;
  CHECK(h2d_planes(qx, pg, q, isd, ied, jsd, jed, 1, s));
  CHECK(h2d_planes(qy, pg, q, isd, ied, jsd, jed, 1, s));
  CHECK(h2d_planes(fxa, pg, fx_ad, is, ie + 1, js, je, 1, s));
  CHECK(h2d_planes(fya, pg, fy_ad, is, ie, js, je + 1, 1, s));
  // trajectories of the two sweep directions: the copy_corners fills
  const int corners = grid->nested ? 0 : corner_mask(grid);
  if (corners) {
    k_corners<<<1, 64, 0, s>>>(qx, pg, npx, npy, corners, 1, 1);
    k_corners<<<1, 64, 0, s>>>(qy, pg, npx, npy, corners, 2, 1);
    FV3G_CUDA(cudaGetLastError());
  }
  AdvArgs<D2> a = tp_args(f, pg, bd, npx, npy, NC);
  a.q_in = in_y;
  a.q_in_x = in_x;
  a.corners = 0;  // fills are in the trajectories; their transposes follow
  a.nested = grid->nested;
  a.lim_fac = lim_fac;
  a.fx_out = fl;
  a.fy_out = fl + P * NC;
  // the del-2 damping reads the y-sweep input's strip and interior cells (the two cells beside each face),
  // inside the boxes the gather below reads for that input
  AdvArgs<D2> ad = a;
  if (damping) CHECK(damping_args(ad, d6u, d6v, dms, stage, pg, bd, grid, mfx, mass, damp_c, s));
  for (int pass = 0; pass < 2; ++pass) {  // 0: x-sweep input, 1: y-sweep input
    const int px = pass == 0 ? 7 : 6, py = pass == 0 ? 6 : 7;
    const long long n = (long long)P * NC;
    k_color_planes<<<grid_1d(n), 256, 0, s>>>(in_x, qx, pg, isd, ied, jsd, jed, px, py, NC, pass == 0);
    k_color_planes<<<grid_1d(n), 256, 0, s>>>(in_y, qy, pg, isd, ied, jsd, jed, px, py, NC, pass == 1);
    FV3G_CUDA(cudaGetLastError());
    FV3G_CUDA(cudaMemsetAsync(fl, 0, sizeof(D2) * P * NC * 2, s));
    CHECK(launch_substep_tl(a, hord, s));
    if (damping) CHECK(launch_damp_tl(ad, s));
    // face boxes holding a cell: x input fx [i-2, i+3] x {j}, fy [i-3, i+3] x [j-2, j+3];
    // y input fx [i-2, i+3] x [j-3, j+3], fy {i} x [j-2, j+3]
    const FaceBox bxf = pass == 0 ? FaceBox{-2, 3, 0, 0} : FaceBox{-2, 3, -3, 3};
    const FaceBox byf = pass == 0 ? FaceBox{-3, 3, -2, 3} : FaceBox{0, 0, -2, 3};
    k_gather_adjoint<<<grid_1d((long long)(ied - isd + 1) * (jed - jsd + 1)), 256, 0, s>>>(
        pass == 0 ? gx : gy, fl, fl + P * NC, fxa, fya, pg, isd, ied, jsd, jed, px, py, bxf, byf, is, ie, js, je);
    FV3G_CUDA(cudaGetLastError());
  }
  if (corners) {
    k_corners_adjoint<<<1, 64, 0, s>>>(gx, pg, npx, npy, corners, 1);
    k_corners_adjoint<<<1, 64, 0, s>>>(gy, pg, npx, npy, corners, 2);
    FV3G_CUDA(cudaGetLastError());
  }
  // q_ad += gx + gy on the host (the data domain of the caller's array)
  const int ni = ied - isd + 1, nj = jed - jsd + 1;
  std::vector<double> hx((size_t)ni * nj), hy((size_t)ni * nj);
  CHECK(d2h_planes(hx.data(), gx, pg, isd, ied, jsd, jed, 1, s));
  CHECK(d2h_planes(hy.data(), gy, pg, isd, ied, jsd, jed, 1, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  for (size_t e = 0; e < hx.size(); ++e) q_ad[e] += hx[e] + hy[e];
  std::fill(fx_ad, fx_ad + (size_t)(ie - is + 2) * (je - js + 1), 0.0);
  std::fill(fy_ad, fy_ad + (size_t)(ie - is + 1) * (je - js + 2), 0.0);
  return 0;
}

}  // extern "C"
