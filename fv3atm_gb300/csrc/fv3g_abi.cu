// fv3g_abi.cu -- the extern "C" boundary declared in include/fv3g.h.
//
// Exact-shape entries take the caller's HOST arrays in Fortran order with
// explicit bounds (drop-in for tracer_2d / fv_tp_2d / map_scalar / map1_ppm
// of GFDL_atmos_cubed_sphere, called in fv3atm from atmosphere_dynamics,
// atmos_model.F90:879), copy them into the device plane layout, run the same
// kernels as the batched path, and copy the results back.  Batched entries
// keep all six tiles and all tracers resident in HBM inside an opaque state.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "fv3g_adjoint.cuh"
#include "fv3g_internal.cuh"
#include "fv3g_mass.cuh"
#include "fv3g_remap.cuh"

namespace fv3g {

// --------------------------------------------------------------- errors ---
static thread_local char g_last_error[512] = "";

int set_error(int code, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return code;
}

int cuda_error(cudaError_t e, const char* what) {
  set_error(FV3G_E_CUDA, "%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
  return e == cudaErrorMemoryAllocation ? FV3G_E_NOMEM : FV3G_E_CUDA;
}

#define CHECK(expr)            \
  do {                         \
    int rc__ = (expr);         \
    if (rc__ != 0) return rc__; \
  } while (0)

// ----------------------------------------------------- small kernels -------
// Scatter/convert stacked host-order planes (ni x nj each, contiguous) into
// device planes with an (i, j) offset; FP64 source, T destination.
template <typename T>
__global__ void k_to_planes(const double* src, T* dst, int ni, int nj, long long nplanes, int pitch,
                            long long dplane, int ioff, int joff, long long sstride) {
  const long long tot = (long long)ni * nj * nplanes;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % ni);
    const long long r = e / ni;
    const int j = (int)(r % nj);
    const long long p = r / nj;
    dst[p * dplane + (long long)(j + joff) * pitch + (i + ioff)] = (T)src[p * sstride + (long long)j * ni + i];
  }
}

template <typename T>
__global__ void k_from_planes(const T* src, double* dst, int ni, int nj, long long nplanes, int pitch,
                              long long splane, int ioff, int joff, long long dstride) {
  const long long tot = (long long)ni * nj * nplanes;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % ni);
    const long long r = e / ni;
    const int j = (int)(r % nj);
    const long long p = r / nj;
    dst[p * dstride + (long long)j * ni + i] = (double)src[p * splane + (long long)(j + joff) * pitch + (i + ioff)];
  }
}

template <typename T>
__global__ void k_scale(T* x, long long n, T f) {
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
    x[e] *= f;
}

template <typename T>
__global__ void k_copy_corners(T* q, PlaneGeom pg, int npx, int npy, int corners, int dir, long long nplanes,
                               long long plane) {
  // 4 corners x 9 cells per plane, rotation of the strip beside the corner
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= nplanes * 36) return;
  const long long p = id / 36;
  const int c = (int)(id % 36) / 9, a = (int)(id % 9) / 3 + 1, b = (int)(id % 3) + 1;
  if (!(corners & (1 << c))) return;
  const int su = (c & 1) ? 1 : -1, sv = (c & 2) ? 1 : -1;
  const int cx2 = su < 0 ? 1 : 2 * npx - 1, cy2 = sv < 0 ? 1 : 2 * npy - 1;
  const int U = su * (2 * a - 1), V = sv * (2 * b - 1);
  const bool plus = (dir == 1) ? (su == -sv) : (su == sv);
  const int U2 = plus ? -V : V, V2 = plus ? U : -U;
  const int i = (U + cx2) / 2, j = (V + cy2) / 2, is = (U2 + cx2) / 2, js = (V2 + cy2) / 2;
  q[p * plane + pg.at(i, j)] = q[p * plane + pg.at(is, js)];
}

static unsigned grid_for(long long n, int block = 256) {
  long long g = (n + block - 1) / block;
  return (unsigned)std::max<long long>(1, std::min<long long>(g, 152LL * 16));
}

}  // namespace fv3g

using namespace fv3g;

// ================================================================ state ====
struct fv3g_state {
  fv3g_state_desc d{};
  bool fp64 = true;
  int n = 0, nd = 0, npz = 0, nq = 0;
  int nt = 6;  // tiles: the cube's 6, or single faces whose halo ring the caller prescribes (1, or a batch)
  bool cube = true;  // the tiles are the six faces of the cube (halos from the neighbours)
  PlaneGeom pg{};
  long long plane = 0;
  size_t esz = 8;
  void* q[3] = {nullptr, nullptr, nullptr};  // home, work B, work C
  void* dp[3] = {nullptr, nullptr, nullptr};  // home (call start), work B, work C
  void* cx = nullptr; void* cy = nullptr; void* mfx = nullptr; void* mfy = nullptr;  // inputs (unscaled)
  void* cxs = nullptr; void* cys = nullptr; void* mfxs = nullptr; void* mfys = nullptr;  // scaled copies
  void* xfx = nullptr; void* yfx = nullptr;
  void* dp_eul = nullptr;
  void* area = nullptr; void* rarea = nullptr; void* dxa = nullptr; void* dya = nullptr;
  void* dx = nullptr; void* dy = nullptr; void* sin4 = nullptr;
  void* del6u = nullptr; void* del6v = nullptr;  // tracer-damping metrics
  std::vector<char> del6_set;                    // per tile: its damping metrics were set
  int warps_ring = 0;                            // edge-ring CTA width (0: warps_per_cta), set by autotune
  int pairs = 0;                                 // FP32 hord 8: tracers two per warp (k_substep_pair)
  int remap_form = 0;                            // 0: warp-per-column remap; 1: thread-per-column FP32 where it applies
  double da_min = 0.0;
  void* eflux = nullptr;
  double* ak = nullptr; double* bk = nullptr;
  double* partials = nullptr; double* mass_out = nullptr;
  double* mass0 = nullptr;  // mass fixer: each tracer's mass at the step's start, then scratch (6 nq)
  int* emax = nullptr;      // mass fixer: each tracer's largest biased exponent at the step's start
  unsigned long long* cmax = nullptr;  // bits of the Courant maximum (q_split 0)
  int last_nsplt = 0;                  // substeps of the last tracer_2d
  int* err = nullptr;
  double* stage = nullptr; size_t stage_bytes = 0;  // FP64 staging for uploads
  cudaStream_t stream = nullptr;
  cudaStream_t up = nullptr, down = nullptr;  // fv3g_step_host: upload and download streams
  std::vector<cudaEvent_t> pev;               // fv3g_step_host: its events
  cudaEvent_t xev = nullptr;                  // orders copies on a caller's stream with the state's stream
  int q_cur = 0;      // buffer holding the latest tracer field
  int dp_start = 0;   // buffer holding dp at the start of the last substep
  int dp_end = 0;     // buffer holding dp at the end of the last substep
  bool remapped = false;  // q[0] holds a remapped field (thickness dp_eul)
  bool levels_set = false;
  cudaGraphExec_t gexec = nullptr;
  int g_qsplit = -1;
  // optional per-kernel timing: an event is recorded before the step and after
  // every kernel of it (also inside the captured graph)
  bool timing = false;
  std::vector<cudaEvent_t> ev;
  std::vector<int> ev_kind;  // kernel kind ending at event i (i >= 1)
  std::vector<int> ev_nk;    // kernels launched since event i-1
  int nev = 0;
  Topo topo{};
  std::vector<void*> allocs;
};

namespace {

enum { K_PROLOGUE = 0, K_SUBSTEP = 1, K_EDGEFIX = 2, K_REMAP = 3, K_HALO = 4, K_NKINDS = 5 };

// Record a timing event (when enabled) marking the end of the work of `kind`
// since the previous mark: nkern kernel launches.
int mark(fv3g_state* st, int kind, cudaStream_t s, int nkern = 1) {
  if (!st->timing) return 0;
  if (st->nev >= (int)st->ev.size()) {
    cudaEvent_t e;
    FV3G_CUDA(cudaEventCreate(&e));
    st->ev.push_back(e);
    st->ev_kind.push_back(kind);
    st->ev_nk.push_back(nkern);
  }
  st->ev_kind[st->nev] = kind;
  st->ev_nk[st->nev] = nkern;
  // inside stream capture the record must become an event node of the graph
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  FV3G_CUDA(cudaStreamIsCapturing(s, &cap));
  if (cap == cudaStreamCaptureStatusActive)
    FV3G_CUDA(cudaEventRecordWithFlags(st->ev[st->nev], s, cudaEventRecordExternal));
  else
    FV3G_CUDA(cudaEventRecord(st->ev[st->nev], s));
  ++st->nev;
  return 0;
}

int dalloc(fv3g_state* st, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) return cuda_error(e, "cudaMalloc");
  st->allocs.push_back(*p);
  e = cudaMemsetAsync(*p, 0, bytes, st->stream);
  if (e != cudaSuccess) return cuda_error(e, "cudaMemsetAsync");
  return 0;
}

// Six-tile topology of the face convention used by the grid generator
// (fv3atm_gb300/grid.py): faces (centre, i axis, j axis).
void build_topo(Topo& tp) {
  const int F[6][3][3] = {{{1, 0, 0}, {0, 1, 0}, {0, 0, 1}},  {{0, 1, 0}, {-1, 0, 0}, {0, 0, 1}},
                          {{-1, 0, 0}, {0, -1, 0}, {0, 0, 1}}, {{0, -1, 0}, {1, 0, 0}, {0, 0, 1}},
                          {{0, 0, 1}, {0, 1, 0}, {-1, 0, 0}},  {{0, 0, -1}, {0, 1, 0}, {1, 0, 0}}};
  const int ends[4][2][2] = {{{-1, -1}, {-1, 1}}, {{1, -1}, {1, 1}}, {{-1, -1}, {1, -1}}, {{-1, 1}, {1, 1}}};
  auto pt = [&](int f, int sx, int sy, int* o) {
    for (int c = 0; c < 3; ++c) o[c] = F[f][0][c] + sx * F[f][1][c] + sy * F[f][2][c];
  };
  for (int t = 0; t < 6; ++t)
    for (int e = 0; e < 4; ++e) {
      int p0[3], p1[3];
      pt(t, ends[e][0][0], ends[e][0][1], p0);
      pt(t, ends[e][1][0], ends[e][1][1], p1);
      for (int u = 0; u < 6; ++u) {
        if (u == t) continue;
        for (int f = 0; f < 4; ++f) {
          int q0[3], q1[3];
          pt(u, ends[f][0][0], ends[f][0][1], q0);
          pt(u, ends[f][1][0], ends[f][1][1], q1);
          const bool same = !memcmp(q0, p0, sizeof p0) && !memcmp(q1, p1, sizeof p1);
          const bool flip = !memcmp(q0, p1, sizeof p0) && !memcmp(q1, p0, sizeof p1);
          if (same || flip) {
            tp.nbr[t][e] = (signed char)u;
            tp.nedge[t][e] = (signed char)f;
            tp.rev[t][e] = flip ? 1 : 0;
          }
        }
      }
    }
}

// Paired advection (two tracers per warp) exists for FP32 states with hord 8.
bool pairs_allowed(const fv3g_state* st) { return !st->fp64 && st->d.hord == 8; }

template <typename T>
AdvArgs<T> adv_args(fv3g_state* st, int src, int dst, int dp_in, int dp_out) {
  AdvArgs<T> a{};
  a.q_in = (const T*)st->q[src];
  a.q_out = (T*)st->q[dst];
  a.sQk = st->plane;
  a.sQq = st->plane * st->npz;
  a.sQt = a.sQq * st->nq;
  a.cx = (const T*)st->cxs;
  a.cy = (const T*)st->cys;
  a.xfx = (const T*)st->xfx;
  a.yfx = (const T*)st->yfx;
  a.mfx = (const T*)st->mfxs;
  a.mfy = (const T*)st->mfys;
  a.dp1 = (const T*)st->dp[dp_in];
  a.dp2 = (T*)st->dp[dp_out];
  a.sFk = st->plane;
  a.sFt = st->plane * st->npz;
  a.area = (const T*)st->area;
  a.rarea = (const T*)st->rarea;
  a.dxa = (const T*)st->dxa;
  a.dya = (const T*)st->dya;
  a.sMt = st->plane;
  a.pg = st->pg;
  a.is = 1; a.ie = st->n; a.js = 1; a.je = st->n;
  a.npx = st->n + 1; a.npy = st->n + 1;
  a.nq = st->nq;
  a.npz = st->npz;
  a.corners = 15;
  a.nested = 0;
  a.cube = st->cube ? 1 : 0;
  a.topo = st->topo;
  a.eflux = (T*)st->eflux;
  a.lim_fac = st->d.lim_fac > 0.0 ? st->d.lim_fac : 1.0;
  a.warps_ring = st->warps_ring;
  a.err = st->err;
  a.pairs = pairs_allowed(st) ? st->pairs : 0;
  a.ntiles = st->nt;
  return a;
}

// Shape of a field in the host (Fortran) layout: (nplanes, nj, ni) and the
// (i, j) offset of its first element in the device plane.
struct FieldShape {
  long long nplanes;
  int ni, nj, ioff, joff;
  void* dev;
};

int field_shape(fv3g_state* st, int field, FieldShape& fs, bool for_upload) {
  const int n = st->n, nd = st->nd;
  const long long t = st->nt;
  switch (field) {
    case FV3G_FIELD_Q:
      fs = {t * st->nq * st->npz, nd, nd, 0, 0, for_upload ? st->q[0] : st->q[st->q_cur]};
      return 0;
    case FV3G_FIELD_Q_REMAPPED:
      fs = {t * st->nq * st->npz, nd, nd, 0, 0, st->q[0]};
      return 0;
    case FV3G_FIELD_DELP: fs = {t * st->npz, nd, nd, 0, 0, st->dp[0]}; return 0;
    case FV3G_FIELD_DELP_OUT: fs = {t * st->npz, nd, nd, 0, 0, st->dp[st->dp_end]}; return 0;
    case FV3G_FIELD_CX: fs = {t * st->npz, n + 1, nd, NG, 0, st->cx}; return 0;
    case FV3G_FIELD_CY: fs = {t * st->npz, nd, n + 1, 0, NG, st->cy}; return 0;
    case FV3G_FIELD_MFX: fs = {t * st->npz, n + 1, n, NG, NG, st->mfx}; return 0;
    case FV3G_FIELD_MFY: fs = {t * st->npz, n, n + 1, NG, NG, st->mfy}; return 0;
    default: return set_error(FV3G_E_ARG, "unknown field %d", field);
  }
}

// Copy a field between its device planes and a contiguous (nplanes, nj, ni)
// buffer of the state's element type; to_buf selects the direction.
int plane_copy(fv3g_state* st, const FieldShape& fs, void* buf, bool to_buf, cudaMemcpyKind kind, cudaStream_t s,
               int max_ctas = 0) {
  const size_t es = st->esz;
  char* dev = (char*)fs.dev + ((size_t)fs.joff * st->pg.pitch + fs.ioff) * es;
  const size_t dp = (size_t)st->pg.pitch * es, ds = (size_t)st->plane * es;
  const size_t bp = (size_t)fs.ni * es, bs = (size_t)fs.ni * fs.nj * es;
  if (to_buf) return copy_planes(buf, bp, bs, dev, dp, ds, (size_t)fs.ni * es, fs.nj, fs.nplanes, kind, s, max_ctas);
  return copy_planes(dev, dp, ds, buf, bp, bs, (size_t)fs.ni * es, fs.nj, fs.nplanes, kind, s, max_ctas);
}

int ensure_stage(fv3g_state* st, size_t bytes) {
  if (st->stage_bytes >= bytes) return 0;
  if (st->stage) cudaFree(st->stage);
  st->stage = nullptr;
  st->stage_bytes = 0;
  FV3G_CUDA(cudaMalloc((void**)&st->stage, bytes));
  st->stage_bytes = bytes;
  return 0;
}

template <typename T>
int upload_t(fv3g_state* st, const FieldShape& fs, const double* host, cudaStream_t s) {
  const size_t bytes = (size_t)fs.nplanes * fs.ni * fs.nj * sizeof(double);
  CHECK(ensure_stage(st, bytes));
  FV3G_CUDA(cudaMemcpyAsync(st->stage, host, bytes, cudaMemcpyHostToDevice, s));
  k_to_planes<T><<<grid_for((long long)fs.nplanes * fs.ni * fs.nj), 256, 0, s>>>(
      st->stage, (T*)fs.dev, fs.ni, fs.nj, fs.nplanes, st->pg.pitch, st->plane, fs.ioff, fs.joff,
      (long long)fs.ni * fs.nj);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

template <typename T>
int download_t(fv3g_state* st, const FieldShape& fs, double* host, cudaStream_t s) {
  const size_t bytes = (size_t)fs.nplanes * fs.ni * fs.nj * sizeof(double);
  CHECK(ensure_stage(st, bytes));
  k_from_planes<T><<<grid_for((long long)fs.nplanes * fs.ni * fs.nj), 256, 0, s>>>(
      (const T*)fs.dev, st->stage, fs.ni, fs.nj, fs.nplanes, st->pg.pitch, st->plane, fs.ioff, fs.joff,
      (long long)fs.ni * fs.nj);
  FV3G_CUDA(cudaGetLastError());
  FV3G_CUDA(cudaMemcpyAsync(host, st->stage, bytes, cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  return 0;
}

// Prologue of tracer_2d: scaled work copies of cx, cy, mfx, mfy and the area
// fluxes, shared by every tracer; levels [k0, k0+nk) (nk < 0: every level).
template <typename T>
int prologue_t(fv3g_state* st, int nsplt, cudaStream_t s, int k0 = 0, int nk = -1) {
  if (nk < 0) nk = st->npz;
  const long long lo = (long long)k0 * st->plane;  // first level's offset in every per-level field
  if (st->d.trdm > 1e-4 && (std::count(st->del6_set.begin(), st->del6_set.end(), 1) != st->nt || !(st->da_min > 0.0)))
    return set_error(FV3G_E_ARG, "tracer damping (trdm > 1e-4) needs every tile's grid with del6_u, del6_v, da_min");
  // scaled copies of cx, cy, mfx, mfy (read from the inputs, written scaled) and the area fluxes
  const T frac = (nsplt == 1) ? T(1) : T(1.0 / nsplt);
  AreaFluxSrc<T> src;
  src.cx = (const T*)st->cx + lo;
  src.cy = (const T*)st->cy + lo;
  src.mfx = (const T*)st->mfx + lo;
  src.mfy = (const T*)st->mfy + lo;
  src.err = st->err;
  CHECK(launch_area_flux<T>((T*)st->cxs + lo, (T*)st->cys + lo, (T*)st->xfx + lo, (T*)st->yfx + lo,
                            (T*)st->mfxs + lo, (T*)st->mfys + lo, (const T*)st->dxa, (const T*)st->dya,
                            (const T*)st->dx, (const T*)st->dy, (const T*)st->sin4, st->plane * st->npz, st->plane,
                            st->plane, st->plane, st->pg, 1, st->n, 1, st->n, st->nt, nk, frac, s, src));
  CHECK(mark(st, K_PROLOGUE, s, 1));
  return 0;
}

// The substeps of tracer_2d for tracers [g0, g0+ng) (every tracer is
// advected independently; the layer thicknesses they write are the same).
// Levels [k0, k0+nk) (nk < 0: every level); the level range needs the cube
// without edge reconciliation.
template <typename T>
int substeps_t(fv3g_state* st, int nsplt, int g0, int ng, cudaStream_t s, int k0 = 0, int nk = -1) {
  if (nk < 0) nk = st->npz;
  const bool part = nk < st->npz;
  if (part && (!st->cube || st->eflux != nullptr))
    return set_error(FV3G_E_ARG, "a level range of the substeps needs the cube without edge reconciliation");
  // a CTA advances one tracer per warp: no wider than the group
  const int warps = std::min(ng, st->d.warps_per_cta > 0 ? st->d.warps_per_cta : (st->fp64 ? 5 : 10));
  // element offset of the group and the first level in a tile
  const long long gofs = (long long)g0 * st->plane * st->npz + (long long)k0 * st->plane;
  const long long lo = (long long)k0 * st->plane;  // first level's offset in the per-level fields
  int src = 0, dpi = 0;
  for (int it = 0; it < nsplt; ++it) {
    const int dst = (src == 1) ? 2 : 1;
    const int dpo = (dpi == 1) ? 2 : 1;
    AdvArgs<T> a = adv_args<T>(st, src, dst, dpi, dpo);
    a.q_in += gofs;
    a.q_out += gofs;
    if (part) {
      a.cx += lo; a.cy += lo; a.xfx += lo; a.yfx += lo; a.mfx += lo; a.mfy += lo;
      a.dp1 += lo;
      a.dp2 += lo;
      a.npz = nk;
    }
    a.nq = ng;
    a.warps_ring = std::min(a.warps_ring, ng);
    if (st->cube) {
      CHECK(launch_cube_halo<T>((T*)st->q[src] + gofs, a.sQt, st->plane, ng * nk, st->pg, st->n, st->topo, s, nk,
                                (long long)st->plane * st->npz));
      CHECK(mark(st, K_HALO, s));
    } else if (src != 0) {  // the prescribed ring of the home buffer, held over the step
      CHECK(launch_copy_halo_ring<T>((T*)st->q[src] + gofs, (const T*)st->q[0] + gofs, st->plane, ng * st->npz,
                                     a.sQt, st->nt,
                                     st->pg, st->n, s));
      CHECK(mark(st, K_HALO, s));
    }
    CHECK(launch_substep<T>(a, st->d.hord, false, warps, s));
    const bool damp = it == 0 && st->d.trdm > 1e-4;  // upstream damps the first substep only
    if (damp) {
      a.del6_u = (const T*)st->del6u;
      a.del6_v = (const T*)st->del6v;
      a.damp = T(damp_coefficient(st->d.trdm, st->da_min, st->d.nord_tr));
      a.nord = st->d.nord_tr;
      a.damp_mass = 1;
      CHECK(launch_damp<T>(a, false, s));
    }
    {
      const BlockMap bm = block_map(a.is, a.ie, a.js, a.je, a.npx, a.npy, a.nested);
      const int nint = bm.nbxi * bm.nbyi;
      CHECK(mark(st, K_SUBSTEP, s, (nint > 0) + (bm.nbx * bm.nby > nint) + (damp ? 1 : 0)));
    }
    if (st->cube && st->eflux != nullptr) {
      CHECK(launch_edge_fix<T>(a, st->n, s));
      CHECK(mark(st, K_EDGEFIX, s));
    }
    st->dp_start = dpi;
    src = dst;
    dpi = dpo;
  }
  st->q_cur = src;
  st->dp_end = dpi;
  return 0;
}

// The substep count of a tracer_2d call: q_split when it is given, else
// tracer_2d's int(1 + max |Courant|) over every tile's compute cells (the
// unscaled inputs), read back once; non-finite Courant numbers and counts
// above 64 are errors.
int resolve_nsplt(fv3g_state* st, int q_split, cudaStream_t s, int* nsplt) {
  if (q_split < 0 || q_split > 64) return set_error(FV3G_E_ARG, "q_split must be 0..64 on the batched path");
  if (q_split > 0) {
    *nsplt = q_split;
    return 0;
  }
  FV3G_CUDA(cudaMemsetAsync(st->cmax, 0, sizeof(unsigned long long), s));
  if (st->fp64)
    CHECK(launch_max_courant<double>((const double*)st->cx, (const double*)st->cy, st->plane * st->npz, st->plane,
                                     st->pg, 1, st->n, 1, st->n, st->nt, st->npz, st->cmax, s));
  else
    CHECK(launch_max_courant<float>((const float*)st->cx, (const float*)st->cy, st->plane * st->npz, st->plane,
                                    st->pg, 1, st->n, 1, st->n, st->nt, st->npz, st->cmax, s));
  unsigned long long bits = 0;
  FV3G_CUDA(cudaMemcpyAsync(&bits, st->cmax, sizeof bits, cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  double cmax;
  memcpy(&cmax, &bits, sizeof cmax);
  if (!std::isfinite(cmax)) return set_error(FV3G_E_NONFINITE, "non-finite Courant number");
  const int n = (int)(1.0 + cmax);
  if (n > 64) return set_error(FV3G_E_COURANT, "Courant number too large (nsplt=%d > 64)", n);
  *nsplt = n;
  return 0;
}

template <typename T>
int tracer_2d_t(fv3g_state* st, int nsplt, cudaStream_t s) {
  CHECK(prologue_t<T>(st, nsplt, s));
  return substeps_t<T>(st, nsplt, 0, st->nq, s);
}

// Global-mass arguments of tracers [g0, g0+ng) of field q on thickness dp.
template <typename T>
MassArgs<T> mass_args(const fv3g_state* st, const void* q, const void* dp, int g0) {
  MassArgs<T> m{};
  m.sQk = st->plane;
  m.sQq = st->plane * st->npz;
  m.sQt = m.sQq * st->nq;
  m.q = (const T*)q + (long long)g0 * m.sQq;
  m.dp = (const T*)dp;
  m.sFk = st->plane;
  m.sFt = st->plane * st->npz;
  m.area = (const T*)st->area;
  m.sMt = st->plane;
  m.pg = st->pg;
  m.i1 = 1; m.j1 = 1; m.ni = st->n; m.nj = st->n;
  m.npz = st->npz;
  m.ntiles = st->nt;
  m.partials = st->partials;
  return m;
}

// Mass fixer (desc.mass_fix), around the remap of tracers [g0, g0+ng): the
// step-start mass from the home buffer and the Lagrangian thickness before
// the remap overwrites it (with each tracer's largest exponent), then after
// the remap the remapped mass with its small-value class and the correction
// of each tracer back to its step-start mass.  Scratch: mass0 holds the
// step-start masses [0, nq), the remapped masses [nq, 4nq) (three per
// tracer, by group) and the first pass's moved masses [4nq, 6nq) (two per
// tracer, by group).
template <typename T>
int mass_fix_pre(fv3g_state* st, cudaStream_t s, int g0, int ng) {
  MassArgs<T> m = mass_args<T>(st, st->q[0], st->dp[0], g0);
  if (!st->fp64) {
    FV3G_CUDA(cudaMemsetAsync(st->emax + g0, 0, sizeof(int) * ng, s));
    m.emax_out = st->emax + g0;
  }
  return launch_mass<T>(m, ng, st->mass0 + g0, s);
}
template <typename T>
int mass_fix_post(fv3g_state* st, cudaStream_t s, int g0, int ng) {
  const MassArgs<T> m = mass_args<T>(st, st->q[0], st->dp_eul, g0);
  MassArgs<T> mc = m;
  if (!st->fp64) mc.cls_emax = st->emax + g0;
  double* m1c = st->mass0 + st->nq + 3 * g0;
  double* dm = st->mass0 + 4 * st->nq + 2 * g0;
  CHECK(launch_mass<T>(mc, ng, m1c, s));
  return launch_mass_fix<T>(m, (T*)st->q[0] + (long long)g0 * m.sQq, ng, g0, st->mass0 + g0, m1c, dm,
                            st->fp64 ? nullptr : st->emax + g0, s);
}

// Remap of tracers [g0, g0+ng) of tiles [t0, t0+ntl) from the Lagrangian
// levels onto ak + bk ps.
template <typename T>
int remap_t(fv3g_state* st, cudaStream_t s, int g0 = 0, int ng = -1, int t0 = 0, int ntl = -1) {
  if (!st->levels_set) return set_error(FV3G_E_ARG, "fv3g_state_set_levels has not been called");
  if (ng < 0) ng = st->nq;
  if (ntl < 0) ntl = st->nt;
  const long long tq = (long long)t0 * st->plane * st->npz * st->nq, tf = (long long)t0 * st->plane * st->npz;
  const long long gofs = (long long)g0 * st->plane * st->npz + tq;
  RemapArgs<T> r{};
  r.q_in = (const T*)st->q[st->q_cur] + gofs;
  r.q_out = (T*)st->q[0] + gofs;
  if (st->q_cur == 0) return set_error(FV3G_E_ARG, "remap needs an advected field (run tracer_2d first)");
  r.sQk = st->plane;
  r.sQq = st->plane * st->npz;
  r.sQt = r.sQq * st->nq;
  r.sQqo = r.sQq;
  r.nfield = ng;
  r.dp = (const T*)st->dp[st->dp_end] + tf;
  r.dp_out = (T*)st->dp_eul + tf;
  r.sFk = st->plane;
  r.sFt = st->plane * st->npz;
  r.ak = st->ak;
  r.bk = st->bk;
  r.pg = st->pg;
  r.i1 = 1; r.j1 = 1; r.ni = st->n; r.nj = st->n;
  r.ncol = (long long)ntl * st->n * st->n;
  r.km = st->npz; r.kn = st->npz;
  r.iv = st->d.iv;
  r.q_min = st->d.q_min;
  r.form = st->remap_form;
  const bool whole = t0 == 0 && ntl == st->nt;  // every tile of the tracers: the mass fixer applies here
  if (st->d.mass_fix && whole) CHECK(mass_fix_pre<T>(st, s, g0, ng));
  CHECK(launch_remap<T>(r, st->d.kord, s));
  if (st->d.fill)  // Lagrangian_to_Eulerian's fillz of the remapped tracers
    CHECK(launch_fillz_planes<T>(r.q_out, r.dp_out, st->n, ntl, st->npz, ng, r.sQt, r.sQq, r.sQk, r.sFt, r.sFk,
                                 st->pg, s));
  if (st->d.mass_fix && whole) CHECK(mass_fix_post<T>(st, s, g0, ng));
  // mass fixer: two mass sums (2 launches each), then 3 fixer launches (FP32) or 1 (FP64)
  CHECK(mark(st, K_REMAP, s, (st->d.fill ? 2 : 1) + (st->d.mass_fix && whole ? (st->fp64 ? 5 : 7) : 0)));
  if (t0 + ntl == st->nt) {  // the last tile range of the field: the state now holds the remapped field
    st->q_cur = 0;
    st->remapped = true;
  }
  return 0;
}

// Copy tracers [g0, g0+ng) of tiles [t0, t1) between a host (ntiles, nq,
// npz, nd, nd) array of the state's element type and the planes of q[0].
// Levels [k0, k0+nk) only when nk >= 0 (one copy per tile and tracer).
int q_group_copy(fv3g_state* st, int g0, int ng, void* host, bool to_host, cudaStream_t s, int max_ctas, int t0 = 0,
                 int t1 = -1, int k0 = 0, int nk = -1) {
  const size_t es = st->esz, nd = (size_t)st->nd;
  const size_t hplane = nd * nd * es, dplane = (size_t)st->plane * es;
  if (t1 < 0) t1 = st->nt;
  const bool part = nk >= 0 && nk < st->npz;
  for (int t = t0; t < t1; ++t)
    for (int r = 0; r < (part ? ng : 1); ++r) {
      // first plane of the group (or of tracer g0+r's level range) in tile t, and the planes copied
      const long long p0 = ((long long)t * st->nq + g0 + r) * st->npz + (part ? k0 : 0);
      const long long np = part ? nk : (long long)ng * st->npz;
      char* dev = (char*)st->q[0] + p0 * dplane;
      char* h = (char*)host + p0 * hplane;
      const size_t pitch = (size_t)st->pg.pitch * es;
      if (to_host)
        CHECK(copy_planes(h, nd * es, hplane, dev, pitch, dplane, nd * es, nd, np, cudaMemcpyDeviceToHost, s,
                          max_ctas));
      else
        CHECK(copy_planes(dev, pitch, dplane, h, nd * es, hplane, nd * es, nd, np, cudaMemcpyHostToDevice, s,
                          max_ctas));
    }
  return 0;
}

// Levels [k0, k0+nk) of every tile of a per-level input field from a host
// array in the field's layout.
int level_field_copy(fv3g_state* st, int field, const void* host, cudaStream_t s, int k0, int nk, int max_ctas) {
  FieldShape fs{};
  CHECK(field_shape(st, field, fs, true));
  const size_t es = st->esz;
  const size_t dpl = (size_t)st->plane * es, hpl = (size_t)fs.ni * fs.nj * es;
  for (int t = 0; t < st->nt; ++t) {
    const long long p0 = (long long)t * st->npz + k0;
    char* dev = (char*)fs.dev + p0 * dpl + ((size_t)fs.joff * st->pg.pitch + fs.ioff) * es;
    const char* h = (const char*)host + p0 * hpl;
    CHECK(copy_planes(dev, (size_t)st->pg.pitch * es, dpl, h, (size_t)fs.ni * es, hpl, (size_t)fs.ni * es, fs.nj, nk,
                      cudaMemcpyHostToDevice, s, max_ctas));
  }
  return 0;
}

// ------------------------------------------ tangent-linear and adjoint ---
// Device allocations of one tangent-linear / adjoint call, freed at its end.
struct CallBufs {
  std::vector<void*> p;
  ~CallBufs() {
    for (void* x : p) cudaFree(x);
  }
  template <typename T>
  int take(T** out, size_t count) {
    void* v = nullptr;
    const cudaError_t e = cudaMalloc(&v, count * sizeof(T) + 256);
    if (e != cudaSuccess) {
      cudaGetLastError();
      return set_error(FV3G_E_NOMEM, "tangent-linear / adjoint buffers: %zu bytes: %s", count * sizeof(T),
                       cudaGetErrorString(e));
    }
    p.push_back(v);
    *out = (T*)v;
    return 0;
  }
};

// The trajectory of a linearised step: the forward substeps of the state's
// inputs run with the production kernels, each substep's input (halo strips
// filled) and layer thickness kept as a checkpoint.
struct LinStep {
  int nsplt = 0;
  std::vector<double*> q;   // nsplt + 1 q-shaped checkpoints (the last: the remap's input)
  std::vector<double*> dp;  // nsplt + 1 per-level thicknesses
  LinArgs a{};
  LinTraj tr{};
  LinWork w{};
  long long qn = 0, fn = 0;  // elements of a q-shaped / per-level array
};

int lin_check(fv3g_state* st) {
  if (!st->fp64) return set_error(FV3G_E_UNSUPPORTED, "the tangent-linear / adjoint step needs an FP64 state");
  if (!st->cube) return set_error(FV3G_E_UNSUPPORTED, "the tangent-linear / adjoint step needs the six-tile cube");
  if (!st->levels_set) return set_error(FV3G_E_ARG, "fv3g_state_set_levels has not been called");
  if (st->d.trdm > 1e-4 || st->d.fill || st->d.edge_sync || st->d.mass_fix)
    return set_error(FV3G_E_UNSUPPORTED,
                     "the tangent-linear / adjoint step covers trdm 0, fill 0, edge_sync 0 and mass_fix 0");
  if (st->d.hord != 1 && st->d.hord != 5 && st->d.hord != 8)
    return set_error(FV3G_E_UNSUPPORTED, "hord %d not implemented (1, 5 and 8 are)", st->d.hord);
  return 0;
}

int lin_forward(fv3g_state* st, int q_split, cudaStream_t s, CallBufs& B, LinStep& L) {
  CHECK(lin_check(st));
  if (q_split < 0) {  // no substeps: the remap alone, of the home field on DELP
    L.nsplt = 0;
  } else {
    CHECK(resolve_nsplt(st, q_split, s, &L.nsplt));
    CHECK(prologue_t<double>(st, L.nsplt, s));
  }
  L.qn = (long long)st->nt * st->nq * st->npz * st->plane;
  L.fn = (long long)st->nt * st->npz * st->plane;
  L.q.assign(L.nsplt + 1, nullptr);
  L.dp.assign(L.nsplt + 1, nullptr);
  for (int i = 0; i <= L.nsplt; ++i) {
    CHECK(B.take(&L.q[i], L.qn));
    CHECK(B.take(&L.dp[i], L.fn));
  }
  FV3G_CUDA(cudaMemcpyAsync(L.q[0], st->q[0], sizeof(double) * L.qn, cudaMemcpyDeviceToDevice, s));
  FV3G_CUDA(cudaMemcpyAsync(L.dp[0], st->dp[0], sizeof(double) * L.fn, cudaMemcpyDeviceToDevice, s));
  const int warps = std::min(st->nq, st->d.warps_per_cta > 0 ? st->d.warps_per_cta : 5);
  for (int it = 0; it < L.nsplt; ++it) {
    CHECK(launch_cube_halo<double>(L.q[it], st->plane * st->npz * st->nq, st->plane, st->nq * st->npz, st->pg, st->n,
                                   st->topo, s));
    AdvArgs<double> a = adv_args<double>(st, 0, 0, 0, 0);
    a.q_in = L.q[it];
    a.q_out = L.q[it + 1];
    a.dp1 = L.dp[it];
    a.dp2 = L.dp[it + 1];
    a.eflux = nullptr;
    a.warps_ring = std::min(a.warps_ring, st->nq);
    CHECK(launch_substep<double>(a, st->d.hord, false, warps, s));
  }
  if (L.nsplt > 0) st->last_nsplt = L.nsplt;
  // the linearised substep's arguments and buffers
  LinArgs& a = L.a;
  a = lin_state_args(st->pg, st->plane, st->n, st->nt, st->nq, st->npz, st->d.hord,
                     st->d.lim_fac > 0.0 ? st->d.lim_fac : 1.0, st->topo);
  a.cx = (const double*)st->cxs; a.cy = (const double*)st->cys;
  a.xfx = (const double*)st->xfx; a.yfx = (const double*)st->yfx;
  a.mfx = (const double*)st->mfxs; a.mfy = (const double*)st->mfys;
  a.area = (const double*)st->area; a.rarea = (const double*)st->rarea;
  a.dxa = (const double*)st->dxa; a.dya = (const double*)st->dya;
  double** tq[] = {&L.tr.qc1, &L.tr.qc2, &L.tr.qi, &L.tr.qj, &L.tr.fx2, &L.tr.fy2,
                   &L.w.a1, &L.w.a2, &L.w.ai, &L.w.aj, &L.w.gx, &L.w.gy, &L.w.fx2, &L.w.fy2};
  for (double** b : tq) CHECK(B.take(b, L.qn));
  for (double** b : {&L.tr.wxi, &L.tr.wyi, &L.tr.wxo, &L.tr.wyo}) CHECK(B.take(b, 6 * L.qn));
  return 0;
}

// Copy between a caller's q-shaped device array ((nt nq npz) planes of nd x
// nd, i fastest) and state-layout planes.
int lin_user_copy(fv3g_state* st, double* planes, const double* user, bool to_user, cudaStream_t s) {
  const size_t nd = (size_t)st->nd, es = sizeof(double);
  const size_t hplane = nd * nd * es, dplane = (size_t)st->plane * es, pitch = (size_t)st->pg.pitch * es;
  const long long np = (long long)st->nt * st->nq * st->npz;
  if (to_user)
    return copy_planes(const_cast<double*>(user), nd * es, hplane, planes, pitch, dplane, nd * es, nd, np,
                       cudaMemcpyDeviceToDevice, s);
  return copy_planes(planes, pitch, dplane, user, nd * es, hplane, nd * es, nd, np, cudaMemcpyDeviceToDevice, s);
}

template <typename T>
int remap_fields_t(fv3g_state* st, const void* in, void* out, int nfield, int kind, int iv, int kord,
                          double q_min, int log_p, cudaStream_t s) {
  const int n = st->n, nd = st->nd, km = st->npz;
  const int ni = kind == 2 ? n + 1 : n, nj = kind == 1 ? n + 1 : n;
  const long long nc = (long long)st->nt * ni * nj;
  T* dpl = (T*)st->dp[st->dp_end];  // the Lagrangian thickness of the last tracer_2d (DELP before any)
  if (kind != 0)  // the faces read the columns beside them: the halo strips of the thickness
    CHECK(launch_cube_halo<T>(dpl, st->plane * km, st->plane, km, st->pg, n, st->topo, s));
  CallBufs B;
  double *pe1, *pe2;
  CHECK(B.take(&pe1, (size_t)(km + 1) * nc));
  CHECK(B.take(&pe2, (size_t)(km + 1) * nc));
  CHECK(launch_field_pressures<T>(dpl, st->plane * km, st->plane, st->pg, st->nt, km, ni, nj, kind, log_p, st->ak,
                                  st->bk, pe1, pe2, s));
  RemapArgs<T> r{};
  PlaneGeom up{};  // the caller's planes: nd x nd, i fastest
  up.pitch = nd;
  up.rows = nd;
  up.isd = 1 - NG;
  up.jsd = 1 - NG;
  r.q_in = (const T*)in;
  r.q_out = (T*)out;
  r.sQk = (long long)nd * nd;
  r.sQq = r.sQk * km;
  r.sQt = r.sQq * nfield;
  r.sQqo = r.sQq;
  r.nfield = nfield;
  r.pe1 = pe1;
  r.pe2 = pe2;
  r.pg = up;
  r.i1 = 1; r.j1 = 1; r.ni = ni; r.nj = nj;
  r.ncol = nc;
  r.km = km; r.kn = km;
  r.iv = iv;
  r.q_min = q_min;
  CHECK(launch_remap<T>(r, kord, s));
  FV3G_CUDA(cudaStreamSynchronize(s));  // the pressure buffers are freed on return
  return 0;
}

}  // namespace

int fv3g::state_field_view(fv3g_state* st, int field, bool loading, StateFieldView* v) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  if (field != FV3G_FIELD_Q && field != FV3G_FIELD_DELP)
    return set_error(FV3G_E_ARG, "restart files carry the tracers (FV3G_FIELD_Q) and delp (FV3G_FIELD_DELP)");
  if (loading && field == FV3G_FIELD_Q) {
    if (st->q_cur != 0) {
      FV3G_CUDA(cudaMemcpyAsync(st->q[0], st->q[st->q_cur], (size_t)st->nt * st->nq * st->npz * st->plane * st->esz,
                                cudaMemcpyDeviceToDevice, st->stream));
      st->q_cur = 0;
    }
    st->remapped = false;
  }
  FieldShape fs{};
  CHECK(field_shape(st, field, fs, loading));
  v->dev = fs.dev;
  v->esz = (int)st->esz;
  v->pg = st->pg;
  v->plane = st->plane;
  v->n = st->n;
  v->npz = st->npz;
  v->nq = st->nq;
  v->ntiles = st->nt;
  v->stream = st->stream;
  return 0;
}

extern "C" {

int fv3g_version(void) { return 100; }

int fv3g_last_error(char* buf, int len) {
  if (!buf || len <= 0) return FV3G_E_ARG;
  snprintf(buf, (size_t)len, "%s", g_last_error);
  return 0;
}

int fv3g_device_info(char* buf, int len) {
  int dev = 0;
  cudaDeviceProp p;
  FV3G_CUDA(cudaGetDevice(&dev));
  FV3G_CUDA(cudaGetDeviceProperties(&p, dev));
  if (buf && len > 0) snprintf(buf, (size_t)len, "%s sm_%d%d SMs=%d", p.name, p.major, p.minor, p.multiProcessorCount);
  return 0;
}

int fv3g_state_create(const fv3g_state_desc* desc, fv3g_state** out) {
  if (!desc || !out) return set_error(FV3G_E_ARG, "null argument");
  *out = nullptr;
  const fv3g_state_desc& d = *desc;
  if (d.independent_tiles ? (d.ntiles < 1 || d.ntiles > 1024) : (d.ntiles != 6 && d.ntiles != 1))
    return set_error(FV3G_E_UNSUPPORTED,
                     "batched state supports ntiles 6 (cube), 1 (one face, prescribed halo) or, with "
                     "independent_tiles, 1..1024 single faces (got %d)", d.ntiles);
  if (d.n < 12 || d.npz < 2 || d.npz > KMAX || d.nq < 1)
    return set_error(FV3G_E_ARG, "bad sizes n=%d npz=%d nq=%d (n>=12, 2<=npz<=%d, nq>=1)", d.n, d.npz, d.nq, KMAX);
  if (d.precision != FV3G_FP64 && d.precision != FV3G_MIXED) return set_error(FV3G_E_ARG, "bad precision %d", d.precision);
  if (d.hord != 1 && d.hord != 5 && d.hord != 8)
    return set_error(FV3G_E_UNSUPPORTED, "hord %d not implemented (1, 5 and 8 are)", d.hord);
  if (d.lim_fac < 0.0) return set_error(FV3G_E_ARG, "lim_fac must be positive (0 selects 1), got %g", d.lim_fac);
  if (d.trdm > 1e-4 && (d.nord_tr < 0 || d.nord_tr > 2))
    return set_error(FV3G_E_UNSUPPORTED, "tracer damping supports nord_tr 0..2 (got %d)", d.nord_tr);
  if (d.kord != 4 && d.kord != 9) return set_error(FV3G_E_UNSUPPORTED, "kord %d not implemented", d.kord);
  if (d.iv < -1 || d.iv > 1)
    return set_error(FV3G_E_ARG, "iv %d outside -1..1 (iv -2 needs per-column surface values qs)", d.iv);
  fv3g_state* st = new (std::nothrow) fv3g_state();
  if (!st) return set_error(FV3G_E_NOMEM, "host allocation failed");
  st->d = d;
  st->fp64 = d.precision == FV3G_FP64;
  st->esz = st->fp64 ? 8 : 4;
  st->n = d.n;
  st->nd = d.n + 2 * NG;
  st->npz = d.npz;
  st->nq = d.nq;
  st->nt = d.ntiles;
  st->cube = !d.independent_tiles && d.ntiles == 6;
  st->del6_set.assign(d.ntiles, 0);
  st->pg.pitch = ((st->nd + 1 + 7) / 8) * 8;
  st->pg.rows = st->nd + 1;
  st->pg.isd = 1 - NG;
  st->pg.jsd = 1 - NG;
  st->plane = st->pg.plane();
  build_topo(st->topo);
  {
    int prc = prepare_kernels();
    if (!prc) prc = prepare_remap_kernels();
    if (prc) {
      delete st;
      return prc;
    }
  }
  cudaError_t e = cudaStreamCreateWithFlags(&st->stream, cudaStreamNonBlocking);
  if (e != cudaSuccess) {
    delete st;
    return cuda_error(e, "cudaStreamCreate");
  }
  const size_t P = (size_t)st->plane * st->esz;
  const size_t nt = (size_t)d.ntiles;
  const size_t qb = P * nt * d.nq * d.npz, fb = P * nt * d.npz;
  int rc = 0;
  for (int b = 0; b < 3 && !rc; ++b) rc = dalloc(st, &st->q[b], qb);
  for (int b = 0; b < 3 && !rc; ++b) rc = dalloc(st, &st->dp[b], fb);
  void** fields[] = {&st->cx, &st->cy, &st->mfx, &st->mfy, &st->cxs, &st->cys, &st->mfxs, &st->mfys,
                     &st->xfx, &st->yfx, &st->dp_eul};
  for (void** f : fields)
    if (!rc) rc = dalloc(st, f, fb);
  void** metrics[] = {&st->area, &st->rarea, &st->dxa, &st->dya, &st->dx, &st->dy, &st->del6u, &st->del6v};
  for (void** m : metrics)
    if (!rc) rc = dalloc(st, m, P * nt);
  if (!rc) rc = dalloc(st, &st->sin4, P * nt * 4);
  if (!rc && st->cube && d.edge_sync)
    rc = dalloc(st, &st->eflux, st->esz * 6 * 4 * (size_t)d.npz * d.nq * d.n);
  if (!rc) rc = dalloc(st, (void**)&st->ak, sizeof(double) * (KMAX + 1));
  if (!rc) rc = dalloc(st, (void**)&st->bk, sizeof(double) * (KMAX + 1));
  if (!rc) rc = dalloc(st, (void**)&st->partials, sizeof(double) * MASS_PARTIALS_PER_TRACER * d.nq);
  if (!rc) rc = dalloc(st, (void**)&st->mass_out, sizeof(double) * d.nq);
  if (!rc) rc = dalloc(st, (void**)&st->mass0, sizeof(double) * 6 * d.nq);
  if (!rc) rc = dalloc(st, (void**)&st->emax, sizeof(int) * d.nq);
  if (!rc) rc = dalloc(st, (void**)&st->cmax, sizeof(unsigned long long));
  if (!rc) rc = dalloc(st, (void**)&st->err, sizeof(int));
  if (!rc) {
    e = cudaStreamSynchronize(st->stream);
    if (e != cudaSuccess) rc = cuda_error(e, "cudaStreamSynchronize");
  }
  if (rc) {
    fv3g_state_destroy(st);
    return rc;
  }
  *out = st;
  return 0;
}

int fv3g_state_destroy(fv3g_state* st) {
  if (!st) return 0;
  if (st->stream) cudaStreamSynchronize(st->stream);
  if (st->gexec) cudaGraphExecDestroy(st->gexec);
  for (cudaEvent_t e : st->ev) cudaEventDestroy(e);
  for (cudaEvent_t e : st->pev) cudaEventDestroy(e);
  if (st->xev) cudaEventDestroy(st->xev);
  if (st->up) cudaStreamDestroy(st->up);
  if (st->down) cudaStreamDestroy(st->down);
  for (void* p : st->allocs) cudaFree(p);
  if (st->stage) cudaFree(st->stage);
  if (st->stream) cudaStreamDestroy(st->stream);
  delete st;
  return 0;
}

int fv3g_state_set_grid(fv3g_state* st, int tile, const fv3g_grid* g) {
  if (!st || !g || tile < 0 || tile >= st->nt) return set_error(FV3G_E_ARG, "bad state/grid/tile");
  const int nd = st->nd;
  struct M { const double* src; void* dst; int ni, nj; long long off; };
  const size_t P = (size_t)st->plane;
  auto at = [&](void* base, long long plane_index) { return (char*)base + plane_index * P * st->esz; };
  M ms[] = {{g->dx, at(st->dx, tile), nd, nd + 1, 0},    {g->dy, at(st->dy, tile), nd + 1, nd, 0},
            {g->dxa, at(st->dxa, tile), nd, nd, 0},      {g->dya, at(st->dya, tile), nd, nd, 0},
            {g->area, at(st->area, tile), nd, nd, 0},    {g->rarea, at(st->rarea, tile), nd, nd, 0}};
  for (const M& m : ms) {
    if (!m.src) return set_error(FV3G_E_ARG, "null metric pointer");
    FieldShape fs{1, m.ni, m.nj, 0, 0, m.dst};
    int rc = st->fp64 ? upload_t<double>(st, fs, m.src, st->stream) : upload_t<float>(st, fs, m.src, st->stream);
    if (rc) return rc;
  }
  if (g->del6_u && g->del6_v) {  // damping metrics (optional unless trdm > 1e-4)
    M dm[] = {{g->del6_u, at(st->del6u, tile), nd, nd + 1, 0}, {g->del6_v, at(st->del6v, tile), nd + 1, nd, 0}};
    for (const M& m : dm) {
      FieldShape fs{1, m.ni, m.nj, 0, 0, m.dst};
      int rc = st->fp64 ? upload_t<double>(st, fs, m.src, st->stream) : upload_t<float>(st, fs, m.src, st->stream);
      if (rc) return rc;
    }
    st->del6_set[tile] = 1;
  }
  if (g->da_min > 0.0) st->da_min = g->da_min;
  if (!g->sin_sg) return set_error(FV3G_E_ARG, "null sin_sg");
  for (int sl = 0; sl < 4; ++sl) {
    FieldShape fs{1, nd, nd, 0, 0, at(st->sin4, (long long)tile * 4 + sl)};
    const double* src = g->sin_sg + (size_t)sl * nd * nd;
    int rc = st->fp64 ? upload_t<double>(st, fs, src, st->stream) : upload_t<float>(st, fs, src, st->stream);
    if (rc) return rc;
  }
  FV3G_CUDA(cudaStreamSynchronize(st->stream));
  return 0;
}

int fv3g_state_set_levels(fv3g_state* st, const double* ak, const double* bk) {
  if (!st || !ak || !bk) return set_error(FV3G_E_ARG, "null argument");
  FV3G_CUDA(cudaMemcpyAsync(st->ak, ak, sizeof(double) * (st->npz + 1), cudaMemcpyHostToDevice, st->stream));
  FV3G_CUDA(cudaMemcpyAsync(st->bk, bk, sizeof(double) * (st->npz + 1), cudaMemcpyHostToDevice, st->stream));
  FV3G_CUDA(cudaStreamSynchronize(st->stream));
  st->levels_set = true;
  return 0;
}

int fv3g_upload(fv3g_state* st, int field, const double* host) {
  if (!st || !host) return set_error(FV3G_E_ARG, "null argument");
  FieldShape fs{};
  CHECK(field_shape(st, field, fs, true));
  if (field == FV3G_FIELD_Q_REMAPPED || field == FV3G_FIELD_DELP_OUT)
    return set_error(FV3G_E_ARG, "field %d is an output", field);
  int rc = st->fp64 ? upload_t<double>(st, fs, host, st->stream) : upload_t<float>(st, fs, host, st->stream);
  if (rc) return rc;
  if (field == FV3G_FIELD_Q) {
    st->q_cur = 0;
    st->remapped = false;
  }
  FV3G_CUDA(cudaStreamSynchronize(st->stream));
  return 0;
}

int fv3g_download(fv3g_state* st, int field, double* host) {
  if (!st || !host) return set_error(FV3G_E_ARG, "null argument");
  FieldShape fs{};
  CHECK(field_shape(st, field, fs, false));
  return st->fp64 ? download_t<double>(st, fs, host, st->stream) : download_t<float>(st, fs, host, st->stream);
}

// Work on a caller's stream s other than the state's (a copy, a step, a mass
// sum): after the work already queued on the state's stream (which may still
// read or write the same fields) and before the work queued there after it.
// A stream under capture is left to whoever builds the graph.
static bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus c = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &c) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return c != cudaStreamCaptureStatusNone;
}
static int xfer_begin(fv3g_state* st, cudaStream_t s) {
  if (s == st->stream || capturing(s)) return 0;
  if (!st->xev) FV3G_CUDA(cudaEventCreateWithFlags(&st->xev, cudaEventDisableTiming));
  FV3G_CUDA(cudaEventRecord(st->xev, st->stream));
  FV3G_CUDA(cudaStreamWaitEvent(s, st->xev, 0));
  return 0;
}
static int xfer_end(fv3g_state* st, cudaStream_t s) {
  if (s == st->stream || capturing(s)) return 0;
  FV3G_CUDA(cudaEventRecord(st->xev, s));
  FV3G_CUDA(cudaStreamWaitEvent(st->stream, st->xev, 0));
  return 0;
}

int fv3g_upload_device(fv3g_state* st, int field, const void* dptr, void* stream) {
  if (!st || !dptr) return set_error(FV3G_E_ARG, "null argument");
  FieldShape fs{};
  CHECK(field_shape(st, field, fs, true));
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  CHECK(xfer_begin(st, s));
  CHECK(plane_copy(st, fs, const_cast<void*>(dptr), false, cudaMemcpyDeviceToDevice, s));
  CHECK(xfer_end(st, s));
  if (field == FV3G_FIELD_Q) {
    st->q_cur = 0;
    st->remapped = false;
  }
  return 0;
}

int fv3g_download_device(fv3g_state* st, int field, void* dptr, void* stream) {
  if (!st || !dptr) return set_error(FV3G_E_ARG, "null argument");
  FieldShape fs{};
  CHECK(field_shape(st, field, fs, false));
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  CHECK(xfer_begin(st, s));
  CHECK(plane_copy(st, fs, dptr, true, cudaMemcpyDeviceToDevice, s));
  CHECK(xfer_end(st, s));
  return 0;
}

int fv3g_field_info(fv3g_state* st, int field, void** dptr, long long* strides4, int* pitch) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  FieldShape fs{};
  CHECK(field_shape(st, field, fs, false));
  if (dptr) *dptr = fs.dev;
  if (pitch) *pitch = st->pg.pitch;
  if (strides4) {
    strides4[0] = st->plane;  // level / plane stride
    strides4[1] = st->plane * st->npz;  // tracer (q) or tile (per-level fields)
    strides4[2] = st->plane * st->npz * st->nq;  // tile stride of q
    strides4[3] = st->pg.rows;
  }
  return 0;
}

int fv3g_tracer_2d_batched(fv3g_state* st, int q_split, void* stream) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  CHECK(xfer_begin(st, s));
  int nsplt = q_split;
  CHECK(resolve_nsplt(st, q_split, s, &nsplt));
  st->last_nsplt = nsplt;
  CHECK(st->fp64 ? tracer_2d_t<double>(st, nsplt, s) : tracer_2d_t<float>(st, nsplt, s));
  return xfer_end(st, s);
}

int fv3g_state_step_tl(fv3g_state* st, int q_split, int parts, const double* dq_in, double* dq_out, void* stream) {
  if (!st || !dq_in || !dq_out) return set_error(FV3G_E_ARG, "null argument");
  if (parts < 1 || parts > 3) return set_error(FV3G_E_ARG, "parts must be 1 (tracer_2d), 2 (remap) or 3 (both)");
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  CallBufs B;
  LinStep L;
  CHECK(lin_forward(st, (parts & 1) ? q_split : -1, s, B, L));
  if ((parts & 2) && st->d.kord != 4 && st->d.kord != 9)
    return set_error(FV3G_E_UNSUPPORTED, "kord %d not implemented", st->d.kord);
  double *dq0, *dq1;
  CHECK(B.take(&dq0, L.qn));
  CHECK(B.take(&dq1, L.qn));
  CHECK(lin_user_copy(st, dq0, dq_in, false, s));
  for (int it = 0; it < L.nsplt; ++it) {
    CHECK(launch_cube_halo<double>(dq0, st->plane * st->npz * st->nq, st->plane, st->nq * st->npz, st->pg, st->n,
                                   st->topo, s));
    L.a.dp1 = L.dp[it];
    L.a.dp2 = L.dp[it + 1];
    CHECK(lin_trajectory(L.a, L.q[it], L.tr, s));
    CHECK(lin_substep_tl(L.a, L.tr, L.w, dq0, dq1, s));
    std::swap(dq0, dq1);
  }
  if (!(parts & 2)) {  // tracer_2d alone: the tangent on the Lagrangian levels
    CHECK(lin_user_copy(st, dq0, dq_out, true, s));
    FV3G_CUDA(cudaStreamSynchronize(s));
    return 0;
  }
  // the remap on (value, tangent) planes: the production kernel's tangent-linear instance
  using D2 = Dual<double>;
  D2 *qd, *qo, *dpd, *scr;
  unsigned char* sched;
  const long long ncol = (long long)st->nt * st->n * st->n;
  CHECK(B.take(&qd, L.qn));
  CHECK(B.take(&qo, L.qn));
  CHECK(B.take(&dpd, L.fn));
  CHECK(B.take(&scr, (size_t)6 * (KMAX + 1) * ncol));
  CHECK(B.take(&sched, (size_t)(KMAX + 1) * ncol));
  CHECK(lin_pack_dual(qd, L.q[L.nsplt], dq0, L.qn, s));
  CHECK(lin_pack_dual(qo, L.q[L.nsplt], nullptr, L.qn, s));
  CHECK(lin_pack_dual(dpd, L.dp[L.nsplt], nullptr, L.fn, s));
  RemapArgs<D2> r{};
  r.q_in = qd;
  r.q_out = qo;
  r.sQk = st->plane;
  r.sQq = st->plane * st->npz;
  r.sQt = r.sQq * st->nq;
  r.sQqo = r.sQq;
  r.nfield = st->nq;
  r.dp = dpd;
  r.sFk = st->plane;
  r.sFt = st->plane * st->npz;
  r.ak = st->ak;
  r.bk = st->bk;
  r.pg = st->pg;
  r.i1 = 1; r.j1 = 1; r.ni = st->n; r.nj = st->n;
  r.ncol = ncol;
  r.km = st->npz; r.kn = st->npz;
  r.iv = st->d.iv;
  r.q_min = st->d.q_min;
  r.scratch = scr;
  r.sched = sched;
  CHECK(launch_remap_tl(r, st->d.kord, s));
  FV3G_CUDA(cudaMemsetAsync(dq1, 0, sizeof(double) * L.qn, s));
  CHECK(lin_unpack_tangent(qo, dq1, L.qn, s));
  CHECK(lin_user_copy(st, dq1, dq_out, true, s));
  FV3G_CUDA(cudaStreamSynchronize(s));  // the call's buffers are freed on return
  return 0;
}

int fv3g_state_step_ad(fv3g_state* st, int q_split, int parts, const double* q_ad_out, double* q_ad_in,
                       void* stream) {
  if (!st || !q_ad_out || !q_ad_in) return set_error(FV3G_E_ARG, "null argument");
  if (parts < 1 || parts > 3) return set_error(FV3G_E_ARG, "parts must be 1 (tracer_2d), 2 (remap) or 3 (both)");
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  CallBufs B;
  LinStep L;
  CHECK(lin_forward(st, (parts & 1) ? q_split : -1, s, B, L));
  if ((parts & 2) && st->d.kord != 4)
    return set_error(FV3G_E_UNSUPPORTED, "the adjoint step's remap is kord 4 (got %d)", st->d.kord);
  double *g, *a0, *a1;
  CHECK(B.take(&g, L.qn));
  CHECK(B.take(&a0, L.qn));
  CHECK(B.take(&a1, L.qn));
  FV3G_CUDA(cudaMemsetAsync(a0, 0, sizeof(double) * L.qn, s));
  if (parts & 2) {
    CHECK(lin_user_copy(st, g, q_ad_out, false, s));
    CHECK(lin_remap_ad(L.q[L.nsplt], L.dp[L.nsplt], st->ak, st->bk, g, a0, st->pg, st->plane, st->n, st->nt, st->nq,
                       st->npz, st->npz, st->d.iv, st->d.q_min, st->d.kord, s));
  } else {
    CHECK(lin_user_copy(st, a0, q_ad_out, false, s));
  }
  for (int it = L.nsplt - 1; it >= 0; --it) {
    L.a.dp1 = L.dp[it];
    L.a.dp2 = L.dp[it + 1];
    CHECK(lin_trajectory(L.a, L.q[it], L.tr, s));
    CHECK(lin_substep_ad(L.a, L.tr, L.w, a0, a1, s));
    std::swap(a0, a1);
  }
  CHECK(lin_user_copy(st, a0, q_ad_in, true, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  return 0;
}

int fv3g_state_remap_fields(fv3g_state* st, const void* fields_in, void* fields_out, int nfield, int kind, int iv,
                            int kord, double q_min, int log_p, void* stream) {
  if (!st || !fields_in || !fields_out) return set_error(FV3G_E_ARG, "null argument");
  if (nfield < 1) return set_error(FV3G_E_ARG, "nfield must be positive");
  if (kind < 0 || kind > 2) return set_error(FV3G_E_ARG, "kind must be 0 (cells), 1 (u faces) or 2 (v faces)");
  if (kind != 0 && !st->cube)
    return set_error(FV3G_E_UNSUPPORTED, "face fields need the six-tile cube (the faces read the neighbouring tiles)");
  if (iv < -1 || iv > 1) return set_error(FV3G_E_ARG, "iv %d outside -1..1", iv);
  if (kord != 4 && kord != 9) return set_error(FV3G_E_UNSUPPORTED, "kord %d not implemented (4 and 9 are)", kord);
  if (!st->levels_set) return set_error(FV3G_E_ARG, "fv3g_state_set_levels has not been called");
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  return st->fp64 ? remap_fields_t<double>(st, fields_in, fields_out, nfield, kind, iv, kord, q_min, log_p, s)
                  : remap_fields_t<float>(st, fields_in, fields_out, nfield, kind, iv, kord, q_min, log_p, s);
}

int fv3g_state_nsplt(fv3g_state* st, int* nsplt) {
  if (!st || !nsplt) return set_error(FV3G_E_ARG, "null argument");
  *nsplt = st->last_nsplt;
  return 0;
}

// Time one substep (interior + edge-ring launches, halo fill and prologue)
// for each candidate CTA width and keep the fastest; then the same for the
// width of the edge-ring launch alone (its CTAs need more registers and
// shared memory, so a narrower CTA can fit twice per SM).  Reads the home
// tracer buffer and writes only scratch buffers; the logical state is
// unchanged.
int fv3g_state_autotune(fv3g_state* st, int* warps_out) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  // candidate widths per mode: one tracer per warp, and (FP32 hord 8) two
  static const int cand[2][7] = {{4, 5, 6, 8, 10, 0, 0}, {3, 4, 5, 6, 8, 10, 12}};
  const int nmode = pairs_allowed(st) ? 2 : 1;
  const int saved_w = st->d.warps_per_cta, saved_r = st->warps_ring, saved_p = st->pairs, q_cur = st->q_cur,
            dp_start = st->dp_start, dp_end = st->dp_end;
  const bool remapped = st->remapped, timing = st->timing;
  st->timing = false;
  cudaEvent_t e0, e1;
  FV3G_CUDA(cudaEventCreate(&e0));
  FV3G_CUDA(cudaEventCreate(&e1));
  int rc = 0;
  // one timed substep at the current widths; returns a negative time when the width does not fit
  auto time_one = [&](float& ms) -> int {
    int r = fv3g_tracer_2d_batched(st, 1, st->stream);  // warm-up; rejects widths that do not fit
    if (r == FV3G_E_ARG) {
      ms = -1.f;
      return 0;
    }
    if (r) return r;
    ms = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, st->stream);
      r = fv3g_tracer_2d_batched(st, 1, st->stream);
      cudaEventRecord(e1, st->stream);
      if (r) return r;
      if (cudaEventSynchronize(e1) == cudaSuccess) {
        float t = 0.f;
        cudaEventElapsedTime(&t, e0, e1);
        ms = std::min(ms, t);
      }
    }
    return 0;
  };
  int best = 0, best_r = 0, best_mode = 0;
  float best_ms = 0.f;
  st->warps_ring = 0;
  for (int mode = 0; mode < nmode && !rc; ++mode) {
    st->pairs = mode;
    for (int w : cand[mode]) {
      if (w == 0) break;
      st->d.warps_per_cta = w;
      float ms;
      if ((rc = time_one(ms))) break;
      if (ms < 0.f) continue;
      if (best == 0 || ms < best_ms) {
        best = w;
        best_mode = mode;
        best_ms = ms;
      }
    }
  }
  if (!rc && best > 0) {
    st->pairs = best_mode;
    st->d.warps_per_cta = best;
    for (int w : cand[best_mode]) {
      if (w == 0) break;
      if (w == best) continue;
      st->warps_ring = w;
      float ms;
      if ((rc = time_one(ms))) break;
      if (ms >= 0.f && ms < best_ms) {
        best_r = w;
        best_ms = ms;
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  st->timing = timing;
  st->q_cur = q_cur;
  st->dp_start = dp_start;
  st->dp_end = dp_end;
  st->remapped = remapped;
  if (rc || best == 0) {
    st->d.warps_per_cta = saved_w;
    st->warps_ring = saved_r;
    st->pairs = saved_p;
    return rc ? rc : set_error(FV3G_E_ARG, "no advection CTA width fits this precision");
  }
  st->d.warps_per_cta = best;
  st->warps_ring = best_r;
  st->pairs = best_mode;
  if (st->gexec) {  // the captured step was built for the old width
    cudaGraphExecDestroy(st->gexec);
    st->gexec = nullptr;
  }
  if (warps_out) *warps_out = best;
  return 0;
}

int fv3g_state_set_tracer_pairs(fv3g_state* st, int on) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  if (on && !pairs_allowed(st))
    return set_error(FV3G_E_UNSUPPORTED, "tracer pairs exist for FP32 states with hord 8 only");
  if (on && st->d.warps_per_cta > PAIR_WIDTH_MAX)
    return set_error(FV3G_E_ARG, "tracer pairs take at most %d warps per CTA", PAIR_WIDTH_MAX);
  st->pairs = on ? 1 : 0;
  if (st->gexec) {
    cudaGraphExecDestroy(st->gexec);
    st->gexec = nullptr;
  }
  return 0;
}

int fv3g_state_tracer_pairs(fv3g_state* st, int* on) {
  if (!st || !on) return set_error(FV3G_E_ARG, "null argument");
  *on = pairs_allowed(st) ? st->pairs : 0;
  return 0;
}

int fv3g_state_set_remap_form(fv3g_state* st, int form) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  if (form != 0 && form != 1) return set_error(FV3G_E_ARG, "remap form %d (0: warp per column, 1: thread per column)", form);
  st->remap_form = form;
  if (st->gexec) {  // the captured step holds the old kernel
    cudaGraphExecDestroy(st->gexec);
    st->gexec = nullptr;
  }
  return 0;
}

int fv3g_state_remap_form(fv3g_state* st, int* form) {
  if (!st || !form) return set_error(FV3G_E_ARG, "null argument");
  *form = st->remap_form;
  return 0;
}

int fv3g_state_set_mass_fix(fv3g_state* st, int on) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  st->d.mass_fix = on ? 1 : 0;
  if (st->gexec) {  // the captured step holds the old kernel list
    cudaGraphExecDestroy(st->gexec);
    st->gexec = nullptr;
  }
  return 0;
}

int fv3g_state_widths(fv3g_state* st, int* warps, int* warps_ring) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  const int w = st->d.warps_per_cta > 0 ? st->d.warps_per_cta : (st->fp64 ? 5 : 10);
  if (warps) *warps = w;
  // the edge-ring launch is capped (8 warps for FP32 states, 10 otherwise)
  if (warps_ring) *warps_ring = std::min(st->warps_ring > 0 ? st->warps_ring : w, ring_max_warps((int)st->esz));
  return 0;
}

// ============================================================= ensemble ====
// Independent states (members of an ensemble, any sizes) advanced together:
// one captured graph forks to a stream per member, runs each member's
// tracer_2d + remap there, and joins, so small members overlap on the GPU.
}  // extern "C"

struct fv3g_ensemble {
  std::vector<fv3g_state*> m;
  std::vector<cudaStream_t> ms;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  cudaGraphExec_t gexec = nullptr;
  int g_qsplit = -1;
};

extern "C" {

int fv3g_ensemble_destroy(fv3g_ensemble* e) {
  if (!e) return 0;
  if (e->gexec) cudaGraphExecDestroy(e->gexec);
  for (cudaStream_t s : e->ms) cudaStreamDestroy(s);
  for (cudaEvent_t v : e->join) cudaEventDestroy(v);
  if (e->fork) cudaEventDestroy(e->fork);
  delete e;
  return 0;
}

int fv3g_ensemble_create(fv3g_state* const* members, int n, fv3g_ensemble** out) {
  if (!members || !out || n < 1) return set_error(FV3G_E_ARG, "ensemble needs at least one member");
  *out = nullptr;
  fv3g_ensemble* e = new (std::nothrow) fv3g_ensemble();
  if (!e) return set_error(FV3G_E_NOMEM, "host allocation failed");
  cudaError_t err = cudaEventCreateWithFlags(&e->fork, cudaEventDisableTiming);
  for (int i = 0; i < n && err == cudaSuccess; ++i) {
    if (!members[i]) {
      fv3g_ensemble_destroy(e);
      return set_error(FV3G_E_ARG, "null member %d", i);
    }
    e->m.push_back(members[i]);
    cudaStream_t s;
    cudaEvent_t v;
    err = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (err == cudaSuccess) {
      e->ms.push_back(s);
      err = cudaEventCreateWithFlags(&v, cudaEventDisableTiming);
      if (err == cudaSuccess) e->join.push_back(v);
    }
  }
  if (err != cudaSuccess) {
    fv3g_ensemble_destroy(e);
    return cuda_error(err, "ensemble streams");
  }
  *out = e;
  return 0;
}

int fv3g_ensemble_step(fv3g_ensemble* e, int q_split, void* stream) {
  if (!e) return set_error(FV3G_E_ARG, "null ensemble");
  // one graph for every member: the count is fixed (no read of the Courant maximum inside a capture)
  if (q_split < 1 || q_split > 64) return set_error(FV3G_E_ARG, "the ensemble step needs q_split 1..64");
  for (fv3g_state* st : e->m) {
    if (!st->levels_set) return set_error(FV3G_E_ARG, "a member has no levels (fv3g_state_set_levels)");
    if (st->timing) return set_error(FV3G_E_ARG, "per-kernel timing is not available inside an ensemble step");
  }
  if (e->gexec == nullptr || e->g_qsplit != q_split) {
    if (e->gexec) {
      cudaGraphExecDestroy(e->gexec);
      e->gexec = nullptr;
    }
    cudaStream_t cs;
    FV3G_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g;
    FV3G_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    int rc = 0;
    cudaError_t ce = cudaEventRecord(e->fork, cs);
    for (size_t i = 0; i < e->m.size() && !rc && ce == cudaSuccess; ++i) {
      ce = cudaStreamWaitEvent(e->ms[i], e->fork, 0);
      if (ce != cudaSuccess) break;
      rc = fv3g_tracer_2d_batched(e->m[i], q_split, e->ms[i]);
      if (!rc) rc = fv3g_remap_batched(e->m[i], e->ms[i]);
      if (!rc) ce = cudaEventRecord(e->join[i], e->ms[i]);
      if (!rc && ce == cudaSuccess) ce = cudaStreamWaitEvent(cs, e->join[i], 0);
    }
    cudaError_t ee = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (rc) return rc;
    if (ce != cudaSuccess) return cuda_error(ce, "ensemble capture");
    if (ee != cudaSuccess) return cuda_error(ee, "cudaStreamEndCapture");
    ee = cudaGraphInstantiate(&e->gexec, g, 0);
    cudaGraphDestroy(g);
    if (ee != cudaSuccess) return cuda_error(ee, "cudaGraphInstantiate");
    e->g_qsplit = q_split;
  }
  cudaStream_t s = stream ? (cudaStream_t)stream : e->ms[0];
  for (fv3g_state* st : e->m) CHECK(xfer_begin(st, s));
  FV3G_CUDA(cudaGraphLaunch(e->gexec, s));
  for (fv3g_state* st : e->m) {
    st->q_cur = 0;
    st->remapped = true;
    CHECK(xfer_end(st, s));
  }
  return 0;
}

// fillz on the remapped tracers of every column (the `fill` option applied
// after the tracer remap in Lagrangian_to_Eulerian).
int fv3g_fillz_batched(fv3g_state* st, void* stream) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  if (!st->remapped) return set_error(FV3G_E_ARG, "fillz acts on the remapped tracers (run the remap first)");
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  const long long sQk = st->plane, sQq = st->plane * st->npz, sQt = sQq * st->nq;
  const long long sFk = st->plane, sFt = st->plane * st->npz;
  CHECK(xfer_begin(st, s));
  if (st->fp64)
    CHECK(launch_fillz_planes<double>((double*)st->q[0], (const double*)st->dp_eul, st->n, st->nt, st->npz, st->nq,
                                      sQt, sQq, sQk, sFt, sFk, st->pg, s));
  else
    CHECK(launch_fillz_planes<float>((float*)st->q[0], (const float*)st->dp_eul, st->n, st->nt, st->npz, st->nq,
                                     sQt, sQq, sQk, sFt, sFk, st->pg, s));
  return xfer_end(st, s);
}

int fv3g_remap_batched(fv3g_state* st, void* stream) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  CHECK(xfer_begin(st, s));
  CHECK(st->fp64 ? remap_t<double>(st, s) : remap_t<float>(st, s));
  return xfer_end(st, s);
}

int fv3g_step(fv3g_state* st, int q_split, int use_graph, void* stream) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  CHECK(xfer_begin(st, s));
  if (q_split == 0) {  // the count first (one read of the Courant maximum), then the step for that count
    CHECK(resolve_nsplt(st, 0, s, &q_split));
  }
  if (!use_graph) {
    st->nev = 0;
    CHECK(mark(st, -1, s));
    CHECK(fv3g_tracer_2d_batched(st, q_split, s));
    return fv3g_remap_batched(st, s);
  }
  if (!st->levels_set) return set_error(FV3G_E_ARG, "fv3g_state_set_levels has not been called");
  if (st->gexec == nullptr || st->g_qsplit != q_split) {
    if (st->gexec) {
      cudaGraphExecDestroy(st->gexec);
      st->gexec = nullptr;
    }
    cudaStream_t cs;
    FV3G_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
    cudaGraph_t g;
    FV3G_CUDA(cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal));
    st->nev = 0;
    int rc = mark(st, -1, cs);
    if (!rc) rc = fv3g_tracer_2d_batched(st, q_split, cs);
    if (!rc) rc = fv3g_remap_batched(st, cs);
    cudaError_t e = cudaStreamEndCapture(cs, &g);
    cudaStreamDestroy(cs);
    if (rc) return rc;
    if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&st->gexec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_error(e, "cudaGraphInstantiate");
    st->g_qsplit = q_split;
  }
  FV3G_CUDA(cudaGraphLaunch(st->gexec, s));
  st->q_cur = 0;
  st->remapped = true;
  st->last_nsplt = q_split;
  return xfer_end(st, s);
}

int fv3g_mass_sum(fv3g_state* st, int which, double* host_out, void* stream) {
  if (!st || !host_out) return set_error(FV3G_E_ARG, "null argument");
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  const void* qf;
  const void* dpf;
  if (which == FV3G_FIELD_Q) {
    qf = st->q[st->q_cur];
    dpf = (st->q_cur != 0) ? st->dp[st->dp_end] : (st->remapped ? st->dp_eul : st->dp[0]);
  }
  else if (which == FV3G_FIELD_Q_REMAPPED) { qf = st->q[0]; dpf = st->dp_eul; }
  else return set_error(FV3G_E_ARG, "mass sum of field %d is not defined", which);
  auto run = [&](auto tag) -> int {
    using T = decltype(tag);
    MassArgs<T> m{};
    m.q = (const T*)qf;
    m.sQk = st->plane;
    m.sQq = st->plane * st->npz;
    m.sQt = m.sQq * st->nq;
    m.dp = (const T*)dpf;
    m.sFk = st->plane;
    m.sFt = st->plane * st->npz;
    m.area = (const T*)st->area;
    m.sMt = st->plane;
    m.pg = st->pg;
    m.i1 = 1; m.j1 = 1; m.ni = st->n; m.nj = st->n;
    m.npz = st->npz;
    m.ntiles = st->nt;
    m.partials = st->partials;
    return launch_mass<T>(m, st->nq, st->mass_out, s);
  };
  CHECK(xfer_begin(st, s));
  int rc = st->fp64 ? run(double{}) : run(float{});
  if (rc) return rc;
  CHECK(xfer_end(st, s));
  FV3G_CUDA(cudaMemcpyAsync(host_out, st->mass_out, sizeof(double) * st->nq, cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  return 0;
}

int fv3g_set_timing(fv3g_state* st, int enable) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  if (st->timing != (enable != 0) && st->gexec) {  // recapture with/without event nodes
    cudaGraphExecDestroy(st->gexec);
    st->gexec = nullptr;
  }
  st->timing = enable != 0;
  if (st->timing) {
    // events exist before any capture: a full step records 3 + 2*64 + 1 at most
    while (st->ev.size() < 2 + 2 * 64 + 2) {
      cudaEvent_t e;
      FV3G_CUDA(cudaEventCreate(&e));
      st->ev.push_back(e);
      st->ev_kind.push_back(0);
      st->ev_nk.push_back(0);
    }
  }
  return 0;
}

int fv3g_kernel_times(fv3g_state* st, double* ms_by_kind, int* launches_by_kind) {
  if (!st || !ms_by_kind) return set_error(FV3G_E_ARG, "null argument");
  for (int k = 0; k < K_NKINDS; ++k) {
    ms_by_kind[k] = 0.0;
    if (launches_by_kind) launches_by_kind[k] = 0;
  }
  if (!st->timing || st->nev < 2) return set_error(FV3G_E_ARG, "no timed step recorded (fv3g_set_timing)");
  FV3G_CUDA(cudaEventSynchronize(st->ev[st->nev - 1]));
  for (int i = 1; i < st->nev; ++i) {
    float ms = 0.f;
    FV3G_CUDA(cudaEventElapsedTime(&ms, st->ev[i - 1], st->ev[i]));
    const int kind = st->ev_kind[i];
    if (kind >= 0 && kind < K_NKINDS) {
      ms_by_kind[kind] += ms;
      if (launches_by_kind) launches_by_kind[kind] += st->ev_nk[i];
    }
  }
  return 0;
}

int fv3g_upload_async(fv3g_state* st, int field, const void* host, int host_f32, void* stream) {
  if (!st || !host) return set_error(FV3G_E_ARG, "null argument");
  if (field == FV3G_FIELD_Q_REMAPPED || field == FV3G_FIELD_DELP_OUT)
    return set_error(FV3G_E_ARG, "field %d is an output", field);
  FieldShape fs{};
  CHECK(field_shape(st, field, fs, true));
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  if ((host_f32 != 0) != !st->fp64 && host_f32) return set_error(FV3G_E_UNSUPPORTED, "FP32 host data into an FP64 state");
  CHECK(xfer_begin(st, s));
  if ((host_f32 != 0) == !st->fp64) {  // same element type: one pitched copy
    CHECK(plane_copy(st, fs, (void*)host, false, cudaMemcpyHostToDevice, s));
  } else {
    CHECK(upload_t<float>(st, fs, (const double*)host, s));
  }
  CHECK(xfer_end(st, s));
  if (field == FV3G_FIELD_Q) {
    st->q_cur = 0;
    st->remapped = false;
  }
  return 0;
}

int fv3g_download_async(fv3g_state* st, int field, void* host, int host_f32, void* stream) {
  if (!st || !host) return set_error(FV3G_E_ARG, "null argument");
  FieldShape fs{};
  CHECK(field_shape(st, field, fs, false));
  cudaStream_t s = stream ? (cudaStream_t)stream : st->stream;
  if ((host_f32 != 0) != !st->fp64) return set_error(FV3G_E_UNSUPPORTED, "host type must match the state precision");
  CHECK(xfer_begin(st, s));
  CHECK(plane_copy(st, fs, host, true, cudaMemcpyDeviceToHost, s));
  CHECK(xfer_end(st, s));
  return 0;
}

// One tracer_2d + remap step from host arrays to host arrays, transfers
// overlapped with compute: the per-level inputs go first, then the tracers in
// groups; group g is advected and remapped on the state's stream while group
// g+1 uploads (a grid-capped copy kernel reading page-locked host memory) and
// group g-1 downloads (copy engine), each on its own stream.
int fv3g_step_host(fv3g_state* st, int q_split, const void* q_in, const void* delp, const void* cx, const void* cy,
                   const void* mfx, const void* mfy, void* q_out, int host_f32, int groups, void* stream) {
  if (!st || !q_in || !delp || !cx || !cy || !mfx || !mfy || !q_out) return set_error(FV3G_E_ARG, "null argument");
  if (q_split < 0 || q_split > 64) return set_error(FV3G_E_ARG, "q_split must be 0..64 on the batched path");
  if ((host_f32 != 0) != !st->fp64) return set_error(FV3G_E_UNSUPPORTED, "host type must match the state precision");
  if (!st->levels_set) return set_error(FV3G_E_ARG, "fv3g_state_set_levels has not been called");
  const int warps = st->d.warps_per_cta > 0 ? st->d.warps_per_cta : (st->fp64 ? 5 : 10);
  // The first group streams in level blocks (a cube state with a fixed q_split and neither edge reconciliation
  // nor the mass fixer): each block's per-level inputs and tracers upload, then its prologue and substeps run
  // while the next block uploads, so the advection starts after one block instead of after every input.
  // Then one group is the default (measured at C384 L127 x20: 177 ms, two groups 180 ms); else groups of
  // one CTA width of tracers.
  const bool stream_lev = st->cube && !st->d.edge_sync && !st->d.mass_fix && q_split > 0 && st->npz >= 16;
  int G = groups > 0 ? groups : (stream_lev ? 1 : std::max(1, st->nq / warps));
  G = std::min(G, st->nq);
  // The copy streams run at the highest priority: a compute kernel's grid is
  // far larger than the GPU, and without priority the copy kernels' CTAs
  // would only be dispatched after the last compute CTA; with it they take
  // the first free slots and then stay resident beside the compute CTAs.
  if (!st->up || !st->down) {
    int least = 0, greatest = 0;
    FV3G_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    if (!st->up) FV3G_CUDA(cudaStreamCreateWithPriority(&st->up, cudaStreamNonBlocking, greatest));
    if (!st->down) FV3G_CUDA(cudaStreamCreateWithPriority(&st->down, cudaStreamNonBlocking, greatest));
  }
  const int NB = stream_lev ? 8 : 0;
  // start, levels, per group: uploaded, each tile remapped; per level block of the first group: uploaded
  const size_t need = 2 + (size_t)G * (1 + st->nt) + NB;
  while (st->pev.size() < need + 1) {
    cudaEvent_t e;
    FV3G_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    st->pev.push_back(e);
  }
  cudaStream_t caller = stream ? (cudaStream_t)stream : st->stream;
  cudaStream_t cs = st->stream, us = st->up, ds = st->down;
  cudaEvent_t ev_start = st->pev[0], ev_lev = st->pev[1], ev_end = st->pev[need];
  // everything after the caller's prior work on its stream
  FV3G_CUDA(cudaEventRecord(ev_start, caller));
  FV3G_CUDA(cudaStreamWaitEvent(us, ev_start, 0));
  FV3G_CUDA(cudaStreamWaitEvent(cs, ev_start, 0));
  FV3G_CUDA(cudaStreamWaitEvent(ds, ev_start, 0));
  st->nev = 0;
  CHECK(mark(st, -1, cs));
  constexpr int kCopyCtas = 152;  // one copy CTA per SM beside the compute kernels
  const int lev_fields[] = {FV3G_FIELD_DELP, FV3G_FIELD_CX, FV3G_FIELD_CY, FV3G_FIELD_MFX, FV3G_FIELD_MFY};
  const void* lev_src[] = {delp, cx, cy, mfx, mfy};
  auto group = [&](int g, int& g0, int& ng) {
    g0 = (int)((long long)st->nq * g / G);
    ng = (int)((long long)st->nq * (g + 1) / G) - g0;
  };
  auto block = [&](int b, int& k0, int& nk) {
    k0 = (int)((long long)st->npz * b / NB);
    nk = (int)((long long)st->npz * (b + 1) / NB) - k0;
  };
  cudaEvent_t* ev_block = st->pev.data() + 2 + (size_t)G * (1 + st->nt);
  if (stream_lev) {
    int g0, ng;
    group(0, g0, ng);
    for (int b = 0; b < NB; ++b) {
      int k0, nk;
      block(b, k0, nk);
      const int ctas = b == 0 ? 0 : kCopyCtas;  // the first block alone at full width
      for (int f = 0; f < 5; ++f) CHECK(level_field_copy(st, lev_fields[f], lev_src[f], us, k0, nk, ctas));
      CHECK(q_group_copy(st, g0, ng, (void*)q_in, false, us, ctas, 0, -1, k0, nk));
      FV3G_CUDA(cudaEventRecord(ev_block[b], us));
    }
  } else {
    for (int f = 0; f < 5; ++f) {
      FieldShape fs{};
      CHECK(field_shape(st, lev_fields[f], fs, true));
      CHECK(plane_copy(st, fs, (void*)lev_src[f], false, cudaMemcpyHostToDevice, us));
    }
    FV3G_CUDA(cudaEventRecord(ev_lev, us));
    // q_split 0: the count from the uploaded Courant numbers (the host waits for the per-level uploads)
    if (q_split == 0) CHECK(resolve_nsplt(st, 0, us, &q_split));
  }
  st->last_nsplt = q_split;
  for (int g = stream_lev ? 1 : 0; g < G; ++g) {
    int g0, ng;
    group(g, g0, ng);
    CHECK(q_group_copy(st, g0, ng, (void*)q_in, false, us, g == 0 ? 0 : kCopyCtas));
    FV3G_CUDA(cudaEventRecord(st->pev[2 + g], us));
  }
  if (stream_lev) {
    int g0, ng;
    group(0, g0, ng);
    for (int b = 0; b < NB; ++b) {
      int k0, nk;
      block(b, k0, nk);
      FV3G_CUDA(cudaStreamWaitEvent(cs, ev_block[b], 0));
      CHECK(st->fp64 ? prologue_t<double>(st, q_split, cs, k0, nk) : prologue_t<float>(st, q_split, cs, k0, nk));
      CHECK(st->fp64 ? substeps_t<double>(st, q_split, g0, ng, cs, k0, nk)
                     : substeps_t<float>(st, q_split, g0, ng, cs, k0, nk));
    }
  } else {
    FV3G_CUDA(cudaStreamWaitEvent(cs, ev_lev, 0));
    CHECK(st->fp64 ? prologue_t<double>(st, q_split, cs) : prologue_t<float>(st, q_split, cs));
  }
  for (int g = 0; g < G; ++g) {
    int g0, ng;
    group(g, g0, ng);
    if (!(stream_lev && g == 0)) {
      FV3G_CUDA(cudaStreamWaitEvent(cs, st->pev[2 + g], 0));
      CHECK(st->fp64 ? substeps_t<double>(st, q_split, g0, ng, cs) : substeps_t<float>(st, q_split, g0, ng, cs));
    }
    // the remap runs tile by tile, each tile's download starting as soon as it is remapped, so only the
    // last tile of the last group waits for its download at the end; with the mass fixer the group's
    // tiles are remapped first and corrected together, then downloaded
    if (st->d.mass_fix) {
      CHECK(st->fp64 ? remap_t<double>(st, cs, g0, ng) : remap_t<float>(st, cs, g0, ng));
      FV3G_CUDA(cudaEventRecord(st->pev[2 + G + (size_t)g * st->nt], cs));
      FV3G_CUDA(cudaStreamWaitEvent(ds, st->pev[2 + G + (size_t)g * st->nt], 0));
      CHECK(q_group_copy(st, g0, ng, q_out, true, ds, kCopyCtas));
      continue;
    }
    for (int t = 0; t < st->nt; ++t) {
      CHECK(st->fp64 ? remap_t<double>(st, cs, g0, ng, t, 1) : remap_t<float>(st, cs, g0, ng, t, 1));
      cudaEvent_t done = st->pev[2 + G + (size_t)g * st->nt + t];
      FV3G_CUDA(cudaEventRecord(done, cs));
      FV3G_CUDA(cudaStreamWaitEvent(ds, done, 0));
      CHECK(q_group_copy(st, g0, ng, q_out, true, ds, kCopyCtas, t, t + 1));
    }
  }
  // join the three streams into the caller's
  FV3G_CUDA(cudaEventRecord(ev_end, ds));
  FV3G_CUDA(cudaStreamWaitEvent(caller, ev_end, 0));
  FV3G_CUDA(cudaEventRecord(ev_end, cs));
  FV3G_CUDA(cudaStreamWaitEvent(caller, ev_end, 0));
  FV3G_CUDA(cudaEventRecord(ev_end, us));
  FV3G_CUDA(cudaStreamWaitEvent(caller, ev_end, 0));
  if (!stream) FV3G_CUDA(cudaStreamSynchronize(caller));
  return 0;
}

int fv3g_stream_sync(fv3g_state* st, void* stream) {
  if (!st) return set_error(FV3G_E_ARG, "null state");
  FV3G_CUDA(cudaStreamSynchronize(stream ? (cudaStream_t)stream : st->stream));
  return 0;
}

int fv3g_state_error(fv3g_state* st, int* code) {
  if (!st || !code) return set_error(FV3G_E_ARG, "null argument");
  // read and clear in order after the work queued on the state's streams (they do not
  // synchronise with the default stream)
  for (cudaStream_t s : {st->up, st->down})
    if (s) FV3G_CUDA(cudaStreamSynchronize(s));
  FV3G_CUDA(cudaMemcpyAsync(code, st->err, sizeof(int), cudaMemcpyDeviceToHost, st->stream));
  FV3G_CUDA(cudaMemsetAsync(st->err, 0, sizeof(int), st->stream));
  FV3G_CUDA(cudaStreamSynchronize(st->stream));
  return 0;
}

}  // extern "C"
