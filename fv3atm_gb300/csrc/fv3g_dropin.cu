// fv3g_dropin.cu -- exact-shape (host-array) entries: fv3g_fv_tp_2d,
// fv3g_tracer_2d, fv3g_tracer_2d_1L, fv3g_tracer_2d_nested, fv3g_map_scalar,
// fv3g_map1_ppm, fv3g_map_scalar_3d.
//
// Each entry keeps the upstream Fortran argument list (fv_tp_2d / tracer_2d
// of tp_core.F90 / fv_tracer2d.F90, map_scalar / map1_ppm of fv_mapz.F90 in
// GFDL_atmos_cubed_sphere) with the array bounds passed explicitly, copies the
// caller's column-major host arrays into a device plane layout with one
// cudaMemcpy2D/3D per array, runs the batched kernels on that one domain and
// copies the results back.  Work buffers and the stream are per calling host
// thread, so the row-wise remap entries may be called from OpenMP threads.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "fv3g_internal.cuh"
#include "fv3g_remap.cuh"

using namespace fv3g;

#include "fv3g_hostio.cuh"

namespace {

int check_scheme(int hord, double lim_fac) {
  if (hord != 1 && hord != 5 && hord != 8)
    return set_error(FV3G_E_UNSUPPORTED, "hord %d not implemented (1, 5 and 8 are)", hord);
  if (hord == 1 && !(lim_fac > 0.0)) return set_error(FV3G_E_ARG, "hord 1 needs lim_fac > 0 (got %g)", lim_fac);
  return 0;
}

int check_damping(const fv3g_grid* grid, int nord, bool need_rarea) {
  if (nord < 0 || nord > 2)
    return set_error(FV3G_E_UNSUPPORTED, "tracer damping supports nord 0..2 with a 3-cell halo (got %d)", nord);
  if (!grid->del6_u || !grid->del6_v) return set_error(FV3G_E_ARG, "tracer damping needs grid del6_u and del6_v");
  if (!(grid->da_min > 0.0)) return set_error(FV3G_E_ARG, "tracer damping needs grid da_min > 0");
  if (need_rarea && !grid->rarea) return set_error(FV3G_E_ARG, "tracer damping needs grid rarea");
  return 0;
}

// One outer side of a nested domain: the boundary states of every (tracer,
// level) plane at t0 and t1, ni x nj cells from (i0, j0), i fastest.
struct NestSide {
  const double* t0;
  const double* t1;
  int i0, j0, ni, nj;
};
struct NestSides {
  NestSide side[4];
  int n;
};

// nested_grid_BC_apply_intT on every plane: q = (t0·(split − step) + step·t1)
// · (1/split) at the outer-side halo cells, rounded after every operation as
// the unfused expression is (w0 = split − step and denom = 1/split come from
// the host).  blockIdx.y picks the side.
__global__ void k_nest_bc(double* q, PlaneGeom pg, long long plane, NestSides ns, long long nplanes, double step,
                          double w0, double denom) {
  const NestSide sd = ns.side[blockIdx.y];
  const long long cells = (long long)sd.ni * sd.nj, total = cells * nplanes;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long p = t / cells;
    const int c = (int)(t - p * cells);
    const int i = sd.i0 + c % sd.ni, j = sd.j0 + c / sd.ni;
    q[p * plane + pg.at(i, j)] = __dmul_rn(__dadd_rn(__dmul_rn(sd.t0[t], w0), __dmul_rn(step, sd.t1[t])), denom);
  }
}

// The outer sides of a rank's domain that a nested grid's boundary states
// cover, as nested_grid_BC_apply_intT picks them: west/east over the data
// domain's full height when is == 1 / ie == npx-1; south/north over i = is..ie
// on an outer side (isd/ied toward a neighbour rank) when js == 1 / je == npy-1.
// off[] is where each side's cells start inside its host strip and pitch[] the
// strip's row length: west (isd:0, jsd:jed), east (npx:ied, jsd:jed), south
// (isd:ied, jsd:0), north (isd:ied, npy:jed).
struct NestLayout {
  NestSides ns{};
  int which[4];  // 0 west, 1 east, 2 south, 3 north
  size_t off[4], pitch[4], slice[4];
  size_t cells = 0;  // per plane, all sides
};

NestLayout nest_layout(const fv3g_bounds* bd, int npx, int npy) {
  NestLayout L;
  const int nid = bd->ied - bd->isd + 1, njd = bd->jed - bd->jsd + 1;
  const int i0 = (bd->is == 1) ? bd->is : bd->isd, i1 = (bd->ie == npx - 1) ? bd->ie : bd->ied;
  auto add = [&](int w, int ilo, int jlo, int ni, int nj, size_t off, size_t pitch, size_t slice) {
    NestSide& sd = L.ns.side[L.ns.n];
    sd.i0 = ilo; sd.j0 = jlo; sd.ni = ni; sd.nj = nj;
    L.which[L.ns.n] = w;
    L.off[L.ns.n] = off; L.pitch[L.ns.n] = pitch; L.slice[L.ns.n] = slice;
    L.cells += (size_t)ni * nj;
    ++L.ns.n;
  };
  const int nw = 1 - bd->isd, ne = bd->ied - npx + 1, nsr = 1 - bd->jsd, nnr = bd->jed - npy + 1;
  if (bd->is == 1) add(0, bd->isd, bd->jsd, nw, njd, 0, nw, (size_t)nw * njd);
  if (bd->ie == npx - 1) add(1, npx, bd->jsd, ne, njd, 0, ne, (size_t)ne * njd);
  if (bd->js == 1) add(2, i0, bd->jsd, i1 - i0 + 1, nsr, (size_t)(i0 - bd->isd), nid, (size_t)nid * nsr);
  if (bd->je == npy - 1) add(3, i0, npy, i1 - i0 + 1, nnr, (size_t)(i0 - bd->isd), nid, (size_t)nid * nnr);
  return L;
}

void nest_strips(const fv3g_nest_bc& bc, int w, const double** t0, const double** t1) {
  switch (w) {
    case 0: *t0 = bc.west_t0; *t1 = bc.west_t1; break;
    case 1: *t0 = bc.east_t0; *t1 = bc.east_t1; break;
    case 2: *t0 = bc.south_t0; *t1 = bc.south_t1; break;
    default: *t0 = bc.north_t0; *t1 = bc.north_t1; break;
  }
}

}  // namespace

extern "C" {

int fv3g_fv_tp_2d(double* q, const double* crx, const double* cry, int npx, int npy, int hord, double* fx, double* fy,
                  const double* xfx, const double* yfx, const fv3g_grid* grid, const fv3g_bounds* bd,
                  const double* ra_x, const double* ra_y, double lim_fac, const double* mfx, const double* mfy,
                  const double* mass, int nord, double damp_c) {
  CHECK(check_bounds(bd, npx, npy));
  if (!q || !crx || !cry || !fx || !fy || !xfx || !yfx || !grid || !ra_x || !ra_y)
    return set_error(FV3G_E_ARG, "null array argument");
  if (!grid->dxa || !grid->dya || !grid->area) return set_error(FV3G_E_ARG, "grid needs dxa, dya, area");
  CHECK(check_scheme(hord, lim_fac));
  // upstream damps when damp_c > 1e-4: mass-weighted with mass fluxes (and only
  // if mass is present), unweighted without them
  const bool damping = damp_c > 1e-4 && (mfx == nullptr || mass != nullptr);
  if (damping) CHECK(check_damping(grid, nord, true));
  const PlaneGeom pg = plane_for(bd);
  const size_t P = (size_t)pg.plane();
  CHECK(g_ctx.begin((14 + (damping ? 4 : 0)) * padded(P, 8)));
  cudaStream_t s = g_ctx.stream;
  double *dq = g_ctx.take<double>(P), *dcx = g_ctx.take<double>(P), *dcy = g_ctx.take<double>(P);
  double *dxf = g_ctx.take<double>(P), *dyf = g_ctx.take<double>(P), *drx = g_ctx.take<double>(P);
  double *dry = g_ctx.take<double>(P), *dmx = g_ctx.take<double>(P), *dmy = g_ctx.take<double>(P);
  double *ddxa = g_ctx.take<double>(P), *ddya = g_ctx.take<double>(P), *dar = g_ctx.take<double>(P);
  double *dfx = g_ctx.take<double>(P), *dfy = g_ctx.take<double>(P);
  double *d6u = nullptr, *d6v = nullptr, *dms = nullptr, *drar = nullptr;
  if (damping) {
    d6u = g_ctx.take<double>(P);
    d6v = g_ctx.take<double>(P);
    dms = g_ctx.take<double>(P);
    drar = g_ctx.take<double>(P);
  }
  FV3G_CUDA(cudaMemsetAsync(g_ctx.arena, 0, g_ctx.used, s));
  const int is = bd->is, ie = bd->ie, js = bd->js, je = bd->je, isd = bd->isd, ied = bd->ied, jsd = bd->jsd,
            jed = bd->jed;
  CHECK(h2d_planes(dq, pg, q, isd, ied, jsd, jed, 1, s));
  CHECK(h2d_planes(dcx, pg, crx, is, ie + 1, jsd, jed, 1, s));
  CHECK(h2d_planes(dcy, pg, cry, isd, ied, js, je + 1, 1, s));
  CHECK(h2d_planes(dxf, pg, xfx, is, ie + 1, jsd, jed, 1, s));
  CHECK(h2d_planes(dyf, pg, yfx, isd, ied, js, je + 1, 1, s));
  CHECK(h2d_planes(drx, pg, ra_x, is, ie, jsd, jed, 1, s));
  CHECK(h2d_planes(dry, pg, ra_y, isd, ied, js, je, 1, s));
  if (mfx) CHECK(h2d_planes(dmx, pg, mfx, is, ie + 1, js, je, 1, s));
  if (mfy) CHECK(h2d_planes(dmy, pg, mfy, is, ie, js, je + 1, 1, s));
  CHECK(h2d_planes(ddxa, pg, grid->dxa, isd, ied, jsd, jed, 1, s));
  CHECK(h2d_planes(ddya, pg, grid->dya, isd, ied, jsd, jed, 1, s));
  CHECK(h2d_planes(dar, pg, grid->area, isd, ied, jsd, jed, 1, s));
  if (damping) {
    CHECK(h2d_planes(d6u, pg, grid->del6_u, isd, ied, jsd, jed + 1, 1, s));
    CHECK(h2d_planes(d6v, pg, grid->del6_v, isd, ied + 1, jsd, jed, 1, s));
    CHECK(h2d_planes(drar, pg, grid->rarea, isd, ied, jsd, jed, 1, s));
    if (mfx) CHECK(h2d_planes(dms, pg, mass, isd, ied, jsd, jed, 1, s));
  }
  AdvArgs<double> a{};
  a.q_in = dq;
  a.q_out = nullptr;
  a.cx = dcx; a.cy = dcy; a.xfx = dxf; a.yfx = dyf;
  // without mass fluxes the area fluxes weight the result, as upstream
  a.mfx = mfx ? dmx : dxf;
  a.mfy = mfy ? dmy : dyf;
  a.dp1 = nullptr; a.dp2 = nullptr;
  a.area = dar; a.rarea = dar; a.dxa = ddxa; a.dya = ddya;
  a.ra_x = drx; a.ra_y = dry;
  a.pg = pg;
  a.is = is; a.ie = ie; a.js = js; a.je = je;
  a.npx = npx; a.npy = npy;
  a.nq = 1; a.npz = 1;
  a.corners = corner_mask(grid);
  a.nested = grid->nested;
  a.cube = 0;
  a.fx_out = dfx; a.fy_out = dfy; a.sFlux = (long long)P;
  a.lim_fac = lim_fac;
  CHECK(launch_substep<double>(a, hord, true, 1, s));
  if (damping) {  // deln_flux on the same q, added to the fluxes
    AdvArgs<double> ad = a;
    ad.del6_u = d6u;
    ad.del6_v = d6v;
    ad.rarea = drar;
    ad.damp = damp_coefficient(damp_c, grid->da_min, nord);
    ad.nord = nord;
    ad.damp_mass = mfx != nullptr;
    ad.dp1 = mfx ? dms : nullptr;
    CHECK(launch_damp<double>(ad, true, s));
  }
  if (!grid->nested && a.corners) {
    k_corners<<<1, 64, 0, s>>>(dq, pg, npx, npy, a.corners, 1, 1);
    FV3G_CUDA(cudaGetLastError());
  }
  CHECK(d2h_planes(fx, dfx, pg, is, ie + 1, js, je, 1, s));
  CHECK(d2h_planes(fy, dfy, pg, is, ie, js, je + 1, 1, s));
  CHECK(d2h_planes(q, dq, pg, isd, ied, jsd, jed, 1, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  return 0;
}

// tracer_2d (one substep count for all levels) or, per_level, tracer_2d_1L
// (each level with its own count from its own Courant maximum, its fluxes
// scaled by its own 1/nsplt, halos refreshed before each of its substeps).
static int tracer_2d_impl(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                          const fv3g_grid* grid, const fv3g_bounds* bd, int npx, int npy, int npz, int nq, int hord,
                          int q_split, int nord_tr, double trdm, double lim_fac, fv3g_halo_fn halo_fn,
                          void* halo_ctx, int* nsplt_out, bool per_level, const fv3g_nest_bc* q_bc = nullptr,
                          int* nest_timestep = nullptr, int k_split = 1) {
  CHECK(check_bounds(bd, npx, npy));
  if (!q || !dp1 || !mfx || !mfy || !cx || !cy || !grid) return set_error(FV3G_E_ARG, "null array argument");
  if (!grid->dx || !grid->dy || !grid->dxa || !grid->dya || !grid->area || !grid->rarea || !grid->sin_sg)
    return set_error(FV3G_E_ARG, "incomplete grid");
  if (npz < 1 || nq < 1) return set_error(FV3G_E_ARG, "npz and nq must be positive");
  CHECK(check_scheme(hord, lim_fac));
  // damping of the first substep, weighted by its starting thickness
  const bool damping = trdm > 1e-4;
  if (damping) CHECK(check_damping(grid, nord_tr, false));
  // boundary states of a nested grid, applied before every substep
  const bool nest = nest_timestep != nullptr && grid->nested;
  NestLayout nl;
  if (nest) {
    if (!q_bc) return set_error(FV3G_E_ARG, "a nested grid needs q_bc boundary states");
    if (k_split < 1) return set_error(FV3G_E_ARG, "k_split must be positive (got %d)", k_split);
    nl = nest_layout(bd, npx, npy);
    for (int iq = 0; iq < nq; ++iq)
      for (int m = 0; m < nl.ns.n; ++m) {
        const double *t0, *t1;
        nest_strips(q_bc[iq], nl.which[m], &t0, &t1);
        if (!t0 || !t1) return set_error(FV3G_E_ARG, "q_bc(%d) lacks the strips of an outer side", iq + 1);
      }
  }
  const PlaneGeom pg = plane_for(bd);
  const size_t P = (size_t)pg.plane();
  const size_t nqp = (size_t)nq * npz;
  CHECK(g_ctx.begin(padded(P * nqp, 8) * 2 + padded(P * npz, 8) * 9 + padded(P, 8) * 14 + 256 +
                    (nest ? 2 * padded(nl.cells * nqp, 8) + 8 * 256 : 0)));
  cudaStream_t s = g_ctx.stream;
  double* qa = g_ctx.take<double>(P * nqp);
  double* qb = g_ctx.take<double>(P * nqp);
  double* dpb[3] = {g_ctx.take<double>(P * npz), g_ctx.take<double>(P * npz), g_ctx.take<double>(P * npz)};
  double *dcx = g_ctx.take<double>(P * npz), *dcy = g_ctx.take<double>(P * npz);
  double *dmx = g_ctx.take<double>(P * npz), *dmy = g_ctx.take<double>(P * npz);
  double *dxf = g_ctx.take<double>(P * npz), *dyf = g_ctx.take<double>(P * npz);
  double *ddx = g_ctx.take<double>(P), *ddy = g_ctx.take<double>(P), *ddxa = g_ctx.take<double>(P);
  double *ddya = g_ctx.take<double>(P), *dar = g_ctx.take<double>(P), *drar = g_ctx.take<double>(P);
  double* dsin = g_ctx.take<double>(4 * P);
  double *d6u = g_ctx.take<double>(P), *d6v = g_ctx.take<double>(P);
  unsigned long long* dmax = g_ctx.take<unsigned long long>(1);
  FV3G_CUDA(cudaMemsetAsync(g_ctx.arena, 0, g_ctx.used, s));
  const int is = bd->is, ie = bd->ie, js = bd->js, je = bd->je, isd = bd->isd, ied = bd->ied, jsd = bd->jsd,
            jed = bd->jed;
  CHECK(h2d_planes(qa, pg, q, isd, ied, jsd, jed, (long long)nqp, s));
  CHECK(h2d_planes(dpb[0], pg, dp1, isd, ied, jsd, jed, npz, s));
  CHECK(h2d_planes(dcx, pg, cx, is, ie + 1, jsd, jed, npz, s));
  CHECK(h2d_planes(dcy, pg, cy, isd, ied, js, je + 1, npz, s));
  CHECK(h2d_planes(dmx, pg, mfx, is, ie + 1, js, je, npz, s));
  CHECK(h2d_planes(dmy, pg, mfy, is, ie, js, je + 1, npz, s));
  CHECK(h2d_planes(ddx, pg, grid->dx, isd, ied, jsd, jed + 1, 1, s));
  CHECK(h2d_planes(ddy, pg, grid->dy, isd, ied + 1, jsd, jed, 1, s));
  CHECK(h2d_planes(ddxa, pg, grid->dxa, isd, ied, jsd, jed, 1, s));
  CHECK(h2d_planes(ddya, pg, grid->dya, isd, ied, jsd, jed, 1, s));
  CHECK(h2d_planes(dar, pg, grid->area, isd, ied, jsd, jed, 1, s));
  CHECK(h2d_planes(drar, pg, grid->rarea, isd, ied, jsd, jed, 1, s));
  CHECK(h2d_planes(dsin, pg, grid->sin_sg, isd, ied, jsd, jed, 4, s));  // slots 1..4 of sin_sg(:,:,9)
  if (damping) {
    CHECK(h2d_planes(d6u, pg, grid->del6_u, isd, ied, jsd, jed + 1, 1, s));
    CHECK(h2d_planes(d6v, pg, grid->del6_v, isd, ied + 1, jsd, jed, 1, s));
  }
  if (nest) {  // each side's t0 and t1 for every (tracer, level) plane, packed
    for (int m = 0; m < nl.ns.n; ++m) {
      NestSide& sd = nl.ns.side[m];
      const size_t cells = (size_t)sd.ni * sd.nj;
      double* dev[2] = {g_ctx.take<double>(cells * nqp), g_ctx.take<double>(cells * nqp)};
      for (int iq = 0; iq < nq; ++iq) {
        const double* src[2];
        nest_strips(q_bc[iq], nl.which[m], &src[0], &src[1]);
        for (int t = 0; t < 2; ++t)
          CHECK(copy_planes(dev[t] + (size_t)iq * npz * cells, (size_t)sd.ni * 8, cells * 8, src[t] + nl.off[m],
                            nl.pitch[m] * 8, nl.slice[m] * 8, (size_t)sd.ni * 8, sd.nj, npz,
                            cudaMemcpyHostToDevice, s));
      }
      sd.t0 = dev[0];
      sd.t1 = dev[1];
    }
  }

  if (per_level) {
    const int nif = ie - is + 2, njd = jed - jsd + 1, nid = ied - isd + 1, njf = je - js + 2;
    const size_t hplane = (size_t)nid * njd;
    std::vector<int> ns(npz);
    int nmax = 1;
    for (int k = 0; k < npz; ++k) {  // the level's Courant maximum over the compute domain
      double cmax = 0.0;
      for (int j = js; j <= je; ++j)
        for (int i = is; i <= ie; ++i) {
          cmax = std::max(cmax, std::fabs(cx[(size_t)(i - is) + (size_t)(j - jsd) * nif + (size_t)k * nif * njd]));
          cmax = std::max(cmax, std::fabs(cy[(size_t)(i - isd) + (size_t)(j - js) * nid + (size_t)k * nid * njf]));
        }
      if (!std::isfinite(cmax)) return set_error(FV3G_E_NONFINITE, "non-finite Courant number (level %d)", k + 1);
      ns[k] = q_split > 0 ? q_split : (int)(1.0 + cmax);
      if (ns[k] > 64)
        return set_error(FV3G_E_COURANT, "Courant number too large (level %d: nsplt=%d > 64)", k + 1, ns[k]);
      nmax = std::max(nmax, ns[k]);
    }
    if (nsplt_out) *nsplt_out = nmax;
    const long long PL = (long long)P;
    for (int k = 0; k < npz; ++k) {
      const long long ko = (long long)k * PL;
      const double frac = (ns[k] == 1) ? 1.0 : 1.0 / ns[k];
      CHECK(launch_area_flux<double>(dcx + ko, dcy + ko, dxf + ko, dyf + ko, dmx + ko, dmy + ko, ddxa, ddya, ddx,
                                     ddy, dsin, 0, PL, 0, PL, pg, is, ie, js, je, 1, 1, frac, s));
      int dpi = 0, dp_start = 0;
      for (int it = 0; it < ns[k]; ++it) {
        if (halo_fn) {  // the caller refreshes halos; only this level's planes change meanwhile
          for (int iq = 0; iq < nq; ++iq)
            CHECK(d2h_planes(q + ((size_t)iq * npz + k) * hplane, qa + ((long long)iq * npz + k) * PL, pg, isd, ied,
                             jsd, jed, 1, s));
          FV3G_CUDA(cudaStreamSynchronize(s));
          halo_fn(q, nq, npz, halo_ctx);
          for (int iq = 0; iq < nq; ++iq)
            CHECK(h2d_planes(qa + ((long long)iq * npz + k) * PL, pg, q + ((size_t)iq * npz + k) * hplane, isd, ied,
                             jsd, jed, 1, s));
        }
        const int dpo = (dpi == 1) ? 2 : 1;
        AdvArgs<double> a{};
        a.q_in = qa + ko; a.q_out = qb + ko;
        a.sQk = PL; a.sQq = PL * npz; a.sQt = 0;
        a.cx = dcx + ko; a.cy = dcy + ko; a.xfx = dxf + ko; a.yfx = dyf + ko; a.mfx = dmx + ko; a.mfy = dmy + ko;
        a.dp1 = dpb[dpi] + ko; a.dp2 = dpb[dpo] + ko;
        a.sFk = PL; a.sFt = 0;
        a.area = dar; a.rarea = drar; a.dxa = ddxa; a.dya = ddya; a.sMt = 0;
        a.pg = pg;
        a.is = is; a.ie = ie; a.js = js; a.je = je;
        a.npx = npx; a.npy = npy;
        a.nq = nq; a.npz = 1;
        a.corners = corner_mask(grid);
        a.nested = grid->nested;
        a.cube = 0;
        a.lim_fac = lim_fac;
        CHECK(launch_substep<double>(a, hord, false, std::min(nq, 4), s));
        if (damping && it == 0) {
          a.del6_u = d6u;
          a.del6_v = d6v;
          a.damp = damp_coefficient(trdm, grid->da_min, nord_tr);
          a.nord = nord_tr;
          a.damp_mass = 1;
          CHECK(launch_damp<double>(a, false, s));
        }
        // the level's updated compute domain, every tracer, back into the halo-carrying buffer
        const size_t pitch = (size_t)pg.pitch * 8, slice = (size_t)PL * npz * 8;
        CHECK(copy_planes(qa + ko + pg.at(is, js), pitch, slice, qb + ko + pg.at(is, js), pitch, slice,
                          (size_t)(ie - is + 1) * 8, je - js + 1, nq, cudaMemcpyDeviceToDevice, s));
        dp_start = dpi;
        dpi = dpo;
      }
      // this level's dp1: the thickness at the start of its last substep (compute domain)
      const int ni = ie - is + 1, nj = je - js + 1;
      CHECK(copy_planes(dp1 + k * hplane + (is - isd) + (size_t)(js - jsd) * nid, (size_t)nid * 8, hplane * 8,
                        dpb[dp_start] + ko + pg.at(is, js), (size_t)pg.pitch * 8, (size_t)PL * 8, (size_t)ni * 8, nj,
                        1, cudaMemcpyDeviceToHost, s));
    }
    if (!grid->nested && corner_mask(grid)) {
      const long long np = (long long)nqp;
      k_corners<<<(unsigned)((np * 36 + 255) / 256), 256, 0, s>>>(qa, pg, npx, npy, corner_mask(grid), 1, np);
      FV3G_CUDA(cudaGetLastError());
    }
    CHECK(d2h_planes(q, qa, pg, isd, ied, jsd, jed, (long long)nqp, s));
    CHECK(d2h_planes(cx, dcx, pg, is, ie + 1, jsd, jed, npz, s));
    CHECK(d2h_planes(cy, dcy, pg, isd, ied, js, je + 1, npz, s));
    CHECK(d2h_planes(mfx, dmx, pg, is, ie + 1, js, je, npz, s));
    CHECK(d2h_planes(mfy, dmy, pg, is, ie, js, je + 1, npz, s));
    FV3G_CUDA(cudaStreamSynchronize(s));
    return 0;
  }

  int nsplt = q_split;
  if (q_split <= 0) {
    k_max_abs2<<<64, 256, 0, s>>>(dcx, dcy, pg, is, ie, js, je, npz, dmax);
    FV3G_CUDA(cudaGetLastError());
    unsigned long long bits = 0;
    FV3G_CUDA(cudaMemcpyAsync(&bits, dmax, 8, cudaMemcpyDeviceToHost, s));
    FV3G_CUDA(cudaStreamSynchronize(s));
    double cmax;
    memcpy(&cmax, &bits, 8);
    if (!std::isfinite(cmax)) return set_error(FV3G_E_NONFINITE, "non-finite Courant number");
    nsplt = (int)(1.0 + cmax);
  }
  if (nsplt > 64) return set_error(FV3G_E_COURANT, "Courant number too large (nsplt=%d > 64)", nsplt);
  if (nsplt_out) *nsplt_out = nsplt;
  const double frac = (nsplt == 1) ? 1.0 : 1.0 / nsplt;
  CHECK(launch_area_flux<double>(dcx, dcy, dxf, dyf, dmx, dmy, ddxa, ddya, ddx, ddy, dsin, 0, (long long)P, 0,
                                 (long long)P, pg, is, ie, js, je, 1, npz, frac, s));
  int dpi = 0;
  int dp_start = 0;
  for (int it = 0; it < nsplt; ++it) {
    if (halo_fn) {
      // refresh halos through the caller (FMS mpp_update_domains upstream)
      CHECK(d2h_planes(q, qa, pg, isd, ied, jsd, jed, (long long)nqp, s));
      FV3G_CUDA(cudaStreamSynchronize(s));
      halo_fn(q, nq, npz, halo_ctx);
      CHECK(h2d_planes(qa, pg, q, isd, ied, jsd, jed, (long long)nqp, s));
    }
    if (nest) {
      const double step = (double)*nest_timestep, split = (double)nsplt * k_split;
      if (nl.ns.n > 0) {
        size_t most = 0;
        for (int m = 0; m < nl.ns.n; ++m) most = std::max(most, (size_t)nl.ns.side[m].ni * nl.ns.side[m].nj);
        const unsigned bx = (unsigned)std::min<size_t>((most * nqp + 255) / 256, 1024);
        k_nest_bc<<<dim3(bx, nl.ns.n), 256, 0, s>>>(qa, pg, (long long)P, nl.ns, (long long)nqp, step,
                                                     split - step, 1.0 / split);
        FV3G_CUDA(cudaGetLastError());
      }
      ++*nest_timestep;
    }
    const int dpo = (dpi == 1) ? 2 : 1;
    AdvArgs<double> a{};
    a.q_in = qa; a.q_out = qb;
    a.sQk = (long long)P; a.sQq = (long long)P * npz; a.sQt = 0;
    a.cx = dcx; a.cy = dcy; a.xfx = dxf; a.yfx = dyf; a.mfx = dmx; a.mfy = dmy;
    a.dp1 = dpb[dpi]; a.dp2 = dpb[dpo];
    a.sFk = (long long)P; a.sFt = 0;
    a.area = dar; a.rarea = drar; a.dxa = ddxa; a.dya = ddya; a.sMt = 0;
    a.pg = pg;
    a.is = is; a.ie = ie; a.js = js; a.je = je;
    a.npx = npx; a.npy = npy;
    a.nq = nq; a.npz = npz;
    a.corners = corner_mask(grid);
    a.nested = grid->nested;
    a.cube = 0;
    a.lim_fac = lim_fac;
    CHECK(launch_substep<double>(a, hord, false, std::min(nq, 4), s));
    if (damping && it == 0) {
      a.del6_u = d6u;
      a.del6_v = d6v;
      a.damp = damp_coefficient(trdm, grid->da_min, nord_tr);
      a.nord = nord_tr;
      a.damp_mass = 1;
      CHECK(launch_damp<double>(a, false, s));
    }
    // the updated compute domain goes back into the halo-carrying buffer
    CHECK(d2d_planes(qa, qb, pg, is, ie, js, je, (long long)nqp, s));
    dp_start = dpi;
    dpi = dpo;
  }
  if (!grid->nested && corner_mask(grid)) {
    const long long np = (long long)nqp;
    k_corners<<<(unsigned)((np * 36 + 255) / 256), 256, 0, s>>>(qa, pg, npx, npy, corner_mask(grid), 1, np);
    FV3G_CUDA(cudaGetLastError());
  }
  // upstream leaves dp1 at the thickness of the start of the last substep
  CHECK(d2h_planes(q, qa, pg, isd, ied, jsd, jed, (long long)nqp, s));
  {
    // dp1 compute domain of every level (halo of dp1 is left untouched)
    const int ni = ie - is + 1, nj = je - js + 1, nid = ied - isd + 1, njd = jed - jsd + 1;
    CHECK(copy_planes(dp1 + (is - isd) + (size_t)(js - jsd) * nid, (size_t)nid * 8, (size_t)nid * njd * 8,
                      dpb[dp_start] + pg.at(is, js), (size_t)pg.pitch * 8, (size_t)pg.plane() * 8, (size_t)ni * 8,
                      nj, npz, cudaMemcpyDeviceToHost, s));
  }
  CHECK(d2h_planes(cx, dcx, pg, is, ie + 1, jsd, jed, npz, s));
  CHECK(d2h_planes(cy, dcy, pg, isd, ied, js, je + 1, npz, s));
  CHECK(d2h_planes(mfx, dmx, pg, is, ie + 1, js, je, npz, s));
  CHECK(d2h_planes(mfy, dmy, pg, is, ie, js, je + 1, npz, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  return 0;
}

int fv3g_tracer_2d(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy, const fv3g_grid* grid,
                   const fv3g_bounds* bd, int npx, int npy, int npz, int nq, int hord, int q_split, double dt,
                   int nord_tr, double trdm, double lim_fac, fv3g_halo_fn halo_fn, void* halo_ctx, int* nsplt_out) {
  (void)dt;
  return tracer_2d_impl(q, dp1, mfx, mfy, cx, cy, grid, bd, npx, npy, npz, nq, hord, q_split, nord_tr, trdm,
                        lim_fac, halo_fn, halo_ctx, nsplt_out, false);
}

int fv3g_tracer_2d_nested(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                          const fv3g_grid* grid, const fv3g_bounds* bd, int npx, int npy, int npz, int nq, int hord,
                          int q_split, double dt, int nord_tr, double trdm, int k_split, const fv3g_nest_bc* q_bc,
                          int* nest_timestep, double lim_fac, fv3g_halo_fn halo_fn, void* halo_ctx,
                          int* nsplt_out) {
  (void)dt;
  if (!nest_timestep) return set_error(FV3G_E_ARG, "nest_timestep must not be NULL");
  if (!grid) return set_error(FV3G_E_ARG, "null array argument");
  // the counter advances only when the call succeeds
  int counter = *nest_timestep;
  CHECK(tracer_2d_impl(q, dp1, mfx, mfy, cx, cy, grid, bd, npx, npy, npz, nq, hord, q_split, nord_tr, trdm,
                       lim_fac, halo_fn, halo_ctx, nsplt_out, false, q_bc, &counter, k_split));
  *nest_timestep = counter;
  return 0;
}

int fv3g_tracer_2d_1L(double* q, double* dp1, double* mfx, double* mfy, double* cx, double* cy,
                      const fv3g_grid* grid, const fv3g_bounds* bd, int npx, int npy, int npz, int nq, int hord,
                      int q_split, double dt, int nord_tr, double trdm, double lim_fac, fv3g_halo_fn halo_fn,
                      void* halo_ctx, int* nsplt_out) {
  (void)dt;
  return tracer_2d_impl(q, dp1, mfx, mfy, cx, cy, grid, bd, npx, npy, npz, nq, hord, q_split, nord_tr, trdm,
                        lim_fac, halo_fn, halo_ctx, nsplt_out, true);
}

// dp2 (optional, map1_q2): (i1:i2, kn) target thicknesses dividing the overlap
// masses, and q2 then the 2-D (i1:i2, kn) row
static int map_common(int km, const double* pe1, const double* q1, const double* qs, int kn, const double* pe2,
                      double* q2, int i1, int i2, int j1, int j2, int ibeg, int iend, int jbeg, int jend, int nq,
                      int iv, int kord, double q_min, const double* dp2 = nullptr) {
  if (!pe1 || !q1 || !pe2 || !q2) return set_error(FV3G_E_ARG, "null array argument");
  if (km < 1 || km > KMAX || kn < 1 || kn > KMAX)
    return set_error(FV3G_E_ARG, "remap supports 1..%d layers (km=%d, kn=%d)", KMAX, km, kn);
  if (i1 < ibeg || i2 > iend || i2 < i1 || j1 < jbeg || j2 > jend || j2 < j1)
    return set_error(FV3G_E_ARG, "row/column range outside the array bounds");
  if (kord != 4 && kord != 9) return set_error(FV3G_E_UNSUPPORTED, "kord %d not implemented (4 and 9 are)", kord);
  if (iv < -2 || iv > 1) return set_error(FV3G_E_ARG, "iv %d outside -2..1", iv);
  if (iv == -2 && qs == nullptr) return set_error(FV3G_E_ARG, "iv -2 needs the surface values qs");
  const int ni = i2 - i1 + 1, nj = j2 - j1 + 1;
  const long long ncol = (long long)ni * nj;
  // device copy of the selected columns, planes of ni x nj per (field, level)
  PlaneGeom pg;
  pg.isd = i1;
  pg.jsd = j1;
  pg.pitch = ni;
  pg.rows = nj;
  const size_t P = (size_t)ni * nj;
  CHECK(g_ctx.begin(padded(P * km * nq, 8) + padded(P * kn * nq, 8) + padded(P * (km + 1), 8) +
                    padded(P * (kn + 1), 8) + padded(P, 8) + padded(P * kn, 8) + 1024));
  cudaStream_t s = g_ctx.stream;
  double* d1 = g_ctx.take<double>(P * km * nq);
  double* d2 = g_ctx.take<double>(P * kn * nq);
  double* dpe1 = g_ctx.take<double>(P * (km + 1));
  double* dpe2 = g_ctx.take<double>(P * (kn + 1));
  double* dqs = g_ctx.take<double>(P);
  double* ddp2 = g_ctx.take<double>(P * kn);
  if (dp2) FV3G_CUDA(cudaMemcpyAsync(ddp2, dp2, sizeof(double) * P * kn, cudaMemcpyHostToDevice, s));
  const int nib = iend - ibeg + 1, njb = jend - jbeg + 1;
  // q1(ibeg:iend, jbeg:jend, km*nq): the (i1:i2, j1:j2) block of every plane
  {
    CHECK(copy_planes(d1, (size_t)ni * 8, (size_t)ni * nj * 8, q1 + (i1 - ibeg) + (size_t)(j1 - jbeg) * nib,
                      (size_t)nib * 8, (size_t)nib * njb * 8, (size_t)ni * 8, nj, (long long)km * nq,
                      cudaMemcpyHostToDevice, s));
  }
  FV3G_CUDA(cudaMemcpyAsync(dpe1, pe1, sizeof(double) * P * (km + 1), cudaMemcpyHostToDevice, s));
  FV3G_CUDA(cudaMemcpyAsync(dpe2, pe2, sizeof(double) * P * (kn + 1), cudaMemcpyHostToDevice, s));
  if (qs) FV3G_CUDA(cudaMemcpyAsync(dqs, qs, sizeof(double) * P, cudaMemcpyHostToDevice, s));
  RemapArgs<double> r{};
  r.q_in = d1;
  r.q_out = d2;
  r.sQk = (long long)P;
  r.sQq = (long long)P * km;
  r.sQt = 0;
  r.sQqo = (long long)P * kn;
  r.nfield = nq;
  r.dp = nullptr;
  r.dp_out = nullptr;
  r.pe1 = dpe1;
  r.pe2 = dpe2;
  r.qs = qs ? dqs : nullptr;
  r.dp2 = dp2 ? ddp2 : nullptr;
  r.pg = pg;
  r.i1 = i1; r.j1 = j1; r.ni = ni; r.nj = nj;
  r.ncol = ncol;
  r.km = km; r.kn = kn; r.iv = iv; r.q_min = q_min;
  CHECK(launch_remap<double>(r, kord, s));
  if (dp2) {  // the 2-D (i1:i2, kn) row of map1_q2
    FV3G_CUDA(cudaMemcpyAsync(q2, d2, sizeof(double) * P * kn, cudaMemcpyDeviceToHost, s));
  } else {
    CHECK(copy_planes(q2 + (i1 - ibeg) + (size_t)(j1 - jbeg) * nib, (size_t)nib * 8, (size_t)nib * njb * 8, d2,
                      (size_t)ni * 8, (size_t)ni * nj * 8, (size_t)ni * 8, nj, (long long)kn * nq,
                      cudaMemcpyDeviceToHost, s));
  }
  FV3G_CUDA(cudaStreamSynchronize(s));
  return 0;
}

int fv3g_map_scalar(int km, const double* pe1, const double* q1, const double* qs, int kn, const double* pe2,
                    double* q2, int i1, int i2, int j, int ibeg, int iend, int jbeg, int jend, int iv, int kord,
                    double q_min) {
  return map_common(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j, j, ibeg, iend, jbeg, jend, 1, iv, kord, q_min);
}

int fv3g_map1_ppm(int km, const double* pe1, const double* q1, const double* qs, int kn, const double* pe2,
                  double* q2, int i1, int i2, int j, int ibeg, int iend, int jbeg, int jend, int iv, int kord) {
  return map_common(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j, j, ibeg, iend, jbeg, jend, 1, iv, kord, 0.0);
}

int fv3g_map1_q2(int km, const double* pe1, const double* q1, int kn, const double* pe2, double* q2,
                 const double* dp2, int i1, int i2, int iv, int kord, int j, int ibeg, int iend, int jbeg, int jend,
                 double q_min) {
  if (!dp2) return set_error(FV3G_E_ARG, "null array argument");
  if (iv == -2) return set_error(FV3G_E_ARG, "map1_q2 takes iv -1..1 (no surface values)");
  return map_common(km, pe1, q1, nullptr, kn, pe2, q2, i1, i2, j, j, ibeg, iend, jbeg, jend, 1, iv, kord, q_min,
                    dp2);
}

int fv3g_map_scalar_3d(int km, const double* pe1, const double* q1, const double* qs, int kn, const double* pe2,
                       double* q2, int i1, int i2, int j1, int j2, int ibeg, int iend, int jbeg, int jend, int nq,
                       int iv, int kord, double q_min) {
  if (nq < 1) return set_error(FV3G_E_ARG, "nq must be positive");
  return map_common(km, pe1, q1, qs, kn, pe2, q2, i1, i2, j1, j2, ibeg, iend, jbeg, jend, nq, iv, kord, q_min);
}

}  // extern "C"
