// fv3g_advect.cu -- the kernels around the advection substep of tracer_2d
// (tracer_2d / copy_corners of GFDL_atmos_cubed_sphere, fv_tracer2d.F90 and
// tp_core.F90; absent submodule, .gitmodules:1-4): halo strips of the six
// tiles, the tile-edge flux reconciliation, the area fluxes and Courant
// maximum of the prologue, and the dispatch of the substep kernels
// (fv3g_substep.cuh) by hord.
#include <cstdio>
#include <algorithm>
#include <mutex>
#include <type_traits>

#include "fv3g_stencil.cuh"

namespace fv3g {

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

// Halo strips (NG cells deep along the four tile edges) of every plane of
// the six tiles, copied from the neighbouring tiles through the cube-edge
// mapping (the strip of edge e of tile t is the NG-deep interior strip along
// edge nedge of tile nbr, position reversed when rev).  The corner blocks are
// left to the sweeps: their copy_corners rotation depends on the sweep
// direction.  One CTA per (plane, edge, tile): the source strip is read in
// its own storage order into shared memory and the halo strip written in
// its own, so rows are coalesced and column strips move NG cells per row.
template <typename T>
__global__ void __launch_bounds__(256) k_cube_halo(T* q, long long sQt, long long splane, int nplanes, int nlev,
                                                   long long sQq, PlaneGeom pg, int n, Topo topo) {
  extern __shared__ __align__(16) unsigned char halo_raw[];
  T* strip = reinterpret_cast<T*>(halo_raw);  // [depth][position along the source edge]
  const int e = blockIdx.y, t = blockIdx.z;
  const int nt = topo.nbr[t][e], ne = topo.nedge[t][e], rev = topo.rev[t][e];
  const int cells = NG * n;
  for (int pl = blockIdx.x; pl < nplanes; pl += gridDim.x) {
    // planes of a tile: nlev levels of each tracer, tracers sQq apart
    const long long off = (long long)(pl / nlev) * sQq + (long long)(pl % nlev) * splane;
    const T* src = q + nt * sQt + off;
    T* dst = q + t * sQt + off;
    for (int c = threadIdx.x; c < cells; c += blockDim.x) {
      int d, sp, i, j;
      if (ne == ES || ne == EN) {  // source rows: positions along i are contiguous
        d = c / n + 1;
        sp = c - (d - 1) * n;
        i = sp + 1;
        j = ne == ES ? d : n + 1 - d;
      } else {  // source columns: the NG depths of a row are contiguous
        sp = c / NG;
        d = c - sp * NG + 1;
        i = ne == EW ? d : n + 1 - d;
        j = sp + 1;
      }
      strip[(d - 1) * n + sp] = src[pg.at(i, j)];
    }
    __syncthreads();
    for (int c = threadIdx.x; c < cells; c += blockDim.x) {
      int d, sv, i, j;
      if (e == ES || e == EN) {
        d = c / n + 1;
        sv = c - (d - 1) * n;
        i = sv + 1;
        j = e == ES ? 1 - d : n + d;
      } else {
        sv = c / NG;
        d = c - sv * NG + 1;
        i = e == EW ? 1 - d : n + d;
        j = sv + 1;
      }
      dst[pg.at(i, j)] = strip[(d - 1) * n + (rev ? n - 1 - sv : sv)];
    }
    __syncthreads();
  }
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
// A compute face's inputs: finite, and the Courant number of one substep
// (c * frac) at most 1 in magnitude (the swept region stays in the upwind cell).
template <typename T>
__device__ __forceinline__ void face_check(T c, T m, T frac, int* err) {
  if (!isfinite(c) || !isfinite(m)) raise_error(err, FV3G_E_NONFINITE);
  else if (fabs(c * frac) > T(1)) raise_error(err, FV3G_E_COURANT);
}

template <typename T>
__global__ void k_area_flux(T* cx, T* cy, T* xfx, T* yfx, T* mfx, T* mfy, const T* dxa, const T* dya,
                            const T* dx, const T* dy, const T* sin_sg, long long sFt, long long sFk,
                            long long sMt, long long sSin, PlaneGeom pg, int is, int ie, int js, int je, T frac,
                            AreaFluxSrc<T> src) {
  // unscaled inputs: src when given (the scaled copies are written), else cx.. themselves (in place)
  const T* cxi = src.cx ? src.cx : cx;
  const T* cyi = src.cy ? src.cy : cy;
  const T* mxi = src.mfx ? src.mfx : mfx;
  const T* myi = src.mfy ? src.mfy : mfy;
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
      const T c = cxi[fo + p];
      T v;
      if (c > T(0)) v = c * dxa[mo + pg.at(i - 1, j)] * dy[mo + p] * s_e[pg.at(i - 1, j)];
      else v = c * dxa[mo + p] * dy[mo + p] * s_w[p];
      xfx[fo + p] = v * frac;
      cx[fo + p] = c * frac;
      if (j >= js && j <= je) {
        const T m = mxi[fo + p];
        mfx[fo + p] = m * frac;
        if (src.err != nullptr) face_check(c, m, frac, src.err);
      }
    }
    // y faces: j in js..je+1, cols isd..ied
    if (j >= js && j <= je + 1 && i <= ie + NG) {
      const T c = cyi[fo + p];
      T v;
      if (c > T(0)) v = c * dya[mo + pg.at(i, j - 1)] * dx[mo + p] * s_n[pg.at(i, j - 1)];
      else v = c * dya[mo + p] * dx[mo + p] * s_s[p];
      yfx[fo + p] = v * frac;
      cy[fo + p] = c * frac;
      if (i >= is && i <= ie) {
        const T m = myi[fo + p];
        mfy[fo + p] = m * frac;
        if (src.err != nullptr) face_check(c, m, frac, src.err);
      }
    }
  }
}

template <typename T>
__global__ void k_max_courant(const T* cx, const T* cy, long long sFt, long long sFk, PlaneGeom pg, int is, int ie,
                              int js, int je, unsigned long long* out) {
  // max(|cx|, |cy|) over the compute cells (tracer_2d's cmax), exact in FP64; a non-finite value wins
  // (NaN compares false, so it is carried explicitly)
  const int t = blockIdx.z, k = blockIdx.y;
  const int ni = ie - is + 1, nj = je - js + 1;
  double m = 0.0;
  bool bad = false;
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ni * nj; e += gridDim.x * blockDim.x) {
    const int i = is + e % ni, j = js + e / ni;
    const long long p = t * sFt + k * sFk + pg.at(i, j);
    const double a = fabs((double)cx[p]), b = fabs((double)cy[p]);
    bad = bad || !isfinite(a) || !isfinite(b);
    m = fmax(m, fmax(a, b));
  }
  if (bad) m = __longlong_as_double(0x7ff0000000000000LL);  // +inf
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  // non-negative doubles order as their bit patterns
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// ------------------------------------------------------------ launchers ---
// Contiguous range [lo, lo+cnt) of CTA tiles along one axis whose windows see
// no cube-face edge (edges sit only near the two ends of the axis).
static void edge_free_range(int is, int ie, int np, int nested, int nb, int& lo, int& cnt) {
  lo = nb;
  int hi = -1;
  for (int b = 0; b < nb; ++b) {
    const int i0 = is + b * TW;
    if (window_edge_lo(is, i0, nested) == NO_EDGE && window_edge_hi(ie, np, i0, nested) == NO_EDGE) {
      lo = std::min(lo, b);
      hi = b;
    }
  }
  cnt = hi >= lo ? hi - lo + 1 : 0;
}

BlockMap block_map(int is, int ie, int js, int je, int npx, int npy, int nested) {
  BlockMap m;
  m.nbx = (ie - is + TW) / TW;
  m.nby = (je - js + TW) / TW;
  edge_free_range(is, ie, npx, nested, m.nbx, m.bx0, m.nbxi);
  edge_free_range(js, je, npy, nested, m.nby, m.by0, m.nbyi);
  if (m.nbxi == 0 || m.nbyi == 0) {  // no interior: the ring is every tile
    m.bx0 = 0;
    m.nbxi = 0;
    m.by0 = m.nby;
    m.nbyi = 0;
  }
  return m;
}

// Raise the dynamic shared-memory limit of every advection kernel once per
// process (before any stream capture).
int prepare_kernels() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    prepare_substep_hord<1>(err);
    prepare_substep_hord<5>(err);
    prepare_substep_hord<8>(err);
  });
  return err == cudaSuccess ? 0 : cuda_error(err, "cudaFuncSetAttribute(advection kernels)");
}

template <typename T>
int launch_substep(const AdvArgs<T>& a, int hord, bool flux_mode, int warps, cudaStream_t s) {
  {
    int prc = prepare_kernels();
    if (prc) return prc;
  }
  if (hord == 1 && !(a.lim_fac > 0.0)) return set_error(FV3G_E_ARG, "hord 1 needs lim_fac > 0 (got %g)", a.lim_fac);
  if constexpr (std::is_same<T, float>::value) {
    if (a.pairs && hord == 8 && !flux_mode) return launch_substep_pair(a, warps, s);
  }
  switch (hord) {
    case 8: return launch_substep_hord<T, 8>(a, flux_mode, warps, s);
    case 5: return launch_substep_hord<T, 5>(a, flux_mode, warps, s);
    case 1: return launch_substep_hord<T, 1>(a, flux_mode, warps, s);
    default: return set_error(FV3G_E_UNSUPPORTED, "hord %d not implemented (1, 5 and 8 are)", hord);
  }
}

template <typename T>
int launch_cube_halo(T* q, long long sQt, long long splane, int nplanes, PlaneGeom pg, int n, const Topo& topo,
                     cudaStream_t s, int nlev, long long sQq) {
  const size_t smem = (size_t)NG * n * sizeof(T);
  if (smem > 48 * 1024) return set_error(FV3G_E_ARG, "tile size %d too large for the halo kernel", n);
  dim3 grid((unsigned)std::min(nplanes, 65535), 4, 6);
  k_cube_halo<T><<<grid, 256, smem, s>>>(q, sQt, splane, nplanes, nlev > 0 ? nlev : nplanes, sQq, pg, n, topo);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

// Tangent-linear fluxes (fv_tp_2d flux mode on value/tangent pairs), one warp.
int launch_substep_tl(const AdvArgs<Dual<double>>& a, int hord, cudaStream_t s) {
  {
    int prc = prepare_kernels();
    if (prc) return prc;
  }
  if (hord == 1 && !(a.lim_fac > 0.0)) return set_error(FV3G_E_ARG, "hord 1 needs lim_fac > 0 (got %g)", a.lim_fac);
  switch (hord) {
    case 8: return launch_substep_tl_hord<8>(a, s);
    case 5: return launch_substep_tl_hord<5>(a, s);
    case 1: return launch_substep_tl_hord<1>(a, s);
    default: return set_error(FV3G_E_UNSUPPORTED, "hord %d not implemented (1, 5 and 8 are)", hord);
  }
}

// Halo ring (the NG-deep strips and the corner blocks) of every plane copied
// from src to dst: the prescribed halo of single tiles, held over the
// substeps of a step.  nplanes planes per tile, ntiles tiles sQt apart.
template <typename T>
__global__ void k_copy_halo_ring(T* dst, const T* src, long long splane, int nplanes, long long sQt, int ntiles,
                                 PlaneGeom pg, int n) {
  const int nd = n + 2 * NG, ring = nd * nd - n * n;
  const long long tot = (long long)nplanes * ntiles;
  for (long long tp = blockIdx.y; tp < tot; tp += gridDim.y)
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < ring; c += gridDim.x * blockDim.x) {
      int i, j;
      if (c < NG * nd) {  // rows below the tile
        j = 1 - NG + c / nd;
        i = 1 - NG + c % nd;
      } else if (c < 2 * NG * nd) {  // rows above
        const int r = c - NG * nd;
        j = n + 1 + r / nd;
        i = 1 - NG + r % nd;
      } else {  // the two side strips of the tile's rows
        const int r = c - 2 * NG * nd;
        j = 1 + r / (2 * NG);
        const int k = r % (2 * NG);
        i = k < NG ? 1 - NG + k : n + 1 + (k - NG);
      }
      const long long p = (tp / nplanes) * sQt + (tp % nplanes) * splane + pg.at(i, j);
      dst[p] = src[p];
    }
}

template <typename T>
int launch_copy_halo_ring(T* dst, const T* src, long long splane, int nplanes, long long sQt, int ntiles,
                          PlaneGeom pg, int n, cudaStream_t s) {
  const int nd = n + 2 * NG, ring = nd * nd - n * n;
  const long long tot = (long long)nplanes * ntiles;
  dim3 grid((unsigned)std::min((ring + 255) / 256, 16), (unsigned)std::min<long long>(tot, 65535));
  k_copy_halo_ring<T><<<grid, 256, 0, s>>>(dst, src, splane, nplanes, sQt, ntiles, pg, n);
  FV3G_CUDA(cudaGetLastError());
  return 0;
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
                     PlaneGeom pg, int is, int ie, int js, int je, int ntiles, int npz, T frac, cudaStream_t s,
                     AreaFluxSrc<T> src) {
  const int ncell = (ie - is + 2 + 2 * NG) * (je - js + 2 + 2 * NG);
  dim3 grid((ncell + 255) / 256, npz, ntiles);
  k_area_flux<T><<<grid, 256, 0, s>>>(cx, cy, xfx, yfx, mfx, mfy, dxa, dya, dx, dy, sin_sg, sFt, sFk, sMt, sSin,
                                      pg, is, ie, js, je, frac, src);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

template <typename T>
int launch_max_courant(const T* cx, const T* cy, long long sFt, long long sFk, PlaneGeom pg, int is, int ie, int js,
                       int je, int ntiles, int npz, unsigned long long* d_out, cudaStream_t s) {
  const int ncell = (ie - is + 1) * (je - js + 1);
  dim3 grid(std::min((ncell + 255) / 256, 64), npz, ntiles);
  k_max_courant<T><<<grid, 256, 0, s>>>(cx, cy, sFt, sFk, pg, is, ie, js, je, d_out);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

#define FV3G_INST(T)                                                                                          \
  template int launch_substep<T>(const AdvArgs<T>&, int, bool, int, cudaStream_t);                          \
  template int launch_edge_fix<T>(const AdvArgs<T>&, int, cudaStream_t);                                     \
  template int launch_cube_halo<T>(T*, long long, long long, int, PlaneGeom, int, const Topo&, cudaStream_t, int,  \
                                   long long);                                                                 \
  template int launch_copy_halo_ring<T>(T*, const T*, long long, int, long long, int, PlaneGeom, int, cudaStream_t);             \
  template int launch_area_flux<T>(T*, T*, T*, T*, T*, T*, const T*, const T*, const T*, const T*, const T*, \
                                   long long, long long, long long, long long, PlaneGeom, int, int, int, int, int, \
                                   int, T, cudaStream_t, AreaFluxSrc<T>);                                    \
  template int launch_max_courant<T>(const T*, const T*, long long, long long, PlaneGeom, int, int, int, int, int, \
                                     int, unsigned long long*, cudaStream_t);
FV3G_INST(float)
FV3G_INST(double)
#undef FV3G_INST

}  // namespace fv3g
