// fv3g_internal.cuh -- shared device/host definitions of the fv3g library.
//
// Device layout ("plane layout"): every 2-D field of a tile lives in a plane
// of `rows` rows of `pitch` elements; element (i, j) of the tile (1-based
// Fortran indices, halo included) sits at (j - jsd) * pitch + (i - isd).
// Cell fields use rows jsd..jed, face fields use up to jed+1 / ied+1, so one
// plane geometry (rows = nd+1, pitch >= nd+1) serves all of them.  Planes are
// stacked [tile][tracer][level] for tracers and [tile][level] for per-level
// fields, matching the Fortran (i, j, k, iq) order inside a tile.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/fv3g.h"

#include "fv3g_dual.cuh"

namespace fv3g {

constexpr int NG = 3;    // halo width
constexpr int TW = 26;   // output cells per CTA tile edge
constexpr int WIN = 32;  // window = TW + 2*NG cells (one warp lane per line)
constexpr int NF = 27;   // faces per line of a CTA tile
constexpr int PQ = 33;   // odd pitch of 32-wide shared arrays
constexpr int PF = 27;   // odd pitch of 27/26-wide shared arrays
constexpr int NO_EDGE = -1000;

// Tile-edge ordinals used by the cube topology and the edge-flux buffers.
enum { EW = 0, EE = 1, ES = 2, EN = 3 };

// Six-tile connectivity: for tile t and edge e the neighbour tile, its edge,
// and whether the along-edge index runs the opposite way there.
struct Topo {
  signed char nbr[6][4];
  signed char nedge[6][4];
  signed char rev[6][4];
};

// Widest edge-ring CTA (warps) of a state's element size: the FP32 ring
// kernel is capped at 128 registers so that two 8-warp CTAs fit an SM.
__host__ __device__ constexpr int ring_max_warps(int element_bytes) { return element_bytes == 4 ? 8 : 10; }

struct PlaneGeom {
  int pitch;  // elements per row
  int rows;   // rows per plane
  int isd, jsd;
  __host__ __device__ __forceinline__ long long at(int i, int j) const {
    return (long long)(j - jsd) * pitch + (i - isd);
  }
  __host__ __device__ __forceinline__ long long plane() const { return (long long)pitch * rows; }
};

// Arguments of one advection substep (tracer_2d inner loop body).
template <typename T>
struct AdvArgs {
  const T* q_in;  // [tile][tracer][level] planes
  T* q_out;
  long long sQt, sQq, sQk;  // plane strides in elements (tile, tracer, level)
  const T* cx;              // [tile][level] planes (scaled by 1/nsplt)
  const T* cy;
  const T* xfx;
  const T* yfx;
  const T* mfx;
  const T* mfy;
  const T* dp1;  // layer thickness at the start of the substep
  T* dp2;        // written: thickness at its end
  long long sFt, sFk;
  const T* area;  // [tile] planes
  const T* rarea;
  const T* dxa;
  const T* dya;
  long long sMt;
  PlaneGeom pg;
  int is, ie, js, je;  // compute domain (tile indices)
  int npx, npy;        // tile size + 1
  int nq;
  int corners;  // bit 0 sw, 1 se, 2 nw, 3 ne: tile corner is a cube corner
  int nested;
  int cube;     // 1: six tiles; halo strips of q_in already filled (k_cube_halo), eflux written
  Topo topo;
  T* eflux;     // cube: outward tile-edge fluxes [tile][edge][level][tracer][n]
  int npz;
  const T* ra_x;  // optional caller-supplied ra_x / ra_y planes (single level)
  const T* ra_y;
  const T* q_in_x;  // optional separate input of the x sweeps, no corner fill (adjoint assembly)
  T* fx_out;    // flux mode: planes [level*nq + tracer] of the tile
  T* fy_out;
  long long sFlux;
  double lim_fac;  // hord 1: 2-dx filter factor (upstream default 1)
  int warps_ring;  // warps per CTA of the edge-ring launch (0: as the interior launch)
  // del-2(nord+1) tracer damping (deln_flux), run after the substep kernel
  const T* del6_u;  // [tile] planes: y-face metric (isd:ied, jsd:jed+1)
  const T* del6_v;  // x-face metric (isd:ied+1, jsd:jed)
  T damp;           // (damp_c da_min)^(nord+1)
  int nord;
  int damp_mass;    // 1: field q, flux weighted by damp times the face mean of dp1; 0: field damp q
  int* err;         // optional sticky error word: FV3G_E_DELP when a compute cell's dp2 is not positive
  int pairs;        // FP32, hord 8: advance the tracers two per warp (k_substep_pair)
  int ntiles;       // tiles the launches cover (0: 6 for the cube, else 1)
};

// tiles a substep launch covers
template <typename T>
__host__ __device__ __forceinline__ int adv_tiles(const AdvArgs<T>& a) {
  return a.ntiles > 0 ? a.ntiles : (a.cube ? 6 : 1);
}

// First error of a batched step into its sticky word (later ones are dropped).
__device__ __forceinline__ void raise_error(int* err, int code) {
  if (err != nullptr) atomicCAS(err, 0, code);
}

// CTA tiles of a substep launch: the interior rectangle [bx0, bx0+nbxi) x
// [by0, by0+nbyi) of the nbx x nby tiles holds those whose 32-cell window
// contains no cube-face edge.
struct BlockMap {
  int nbx, nby, bx0, nbxi, by0, nbyi;
};

// Window face (1..31) of the low / high cube-face edge seen by a CTA tile
// starting at i0, NO_EDGE if its window has none.
__host__ __device__ __forceinline__ int window_edge_lo(int is, int i0, int nested) {
  const int e = 1 - i0 + NG;
  return (!nested && is == 1 && e >= 1 && e <= WIN - 1) ? e : NO_EDGE;
}
__host__ __device__ __forceinline__ int window_edge_hi(int ie, int npx, int i0, int nested) {
  const int e = npx - i0 + NG;
  return (!nested && ie + 1 == npx && e >= 1 && e <= WIN - 1) ? e : NO_EDGE;
}

// ------------------------------------------------------------- helpers ----
template <typename T> __device__ __forceinline__ T tmin(T a, T b) { return a < b ? a : b; }
template <typename T> __device__ __forceinline__ T tmax(T a, T b) { return a > b ? a : b; }
template <typename T> __device__ __forceinline__ T tabs(T a) { return a < T(0) ? -a : a; }
// FP32 and FP64: one min / max instruction, and |x| an operand modifier,
// where the compare-and-select forms above take two or three dependent
// instructions; the results differ only for NaN and in the sign of a zero
__device__ __forceinline__ float tmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float tmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ float tabs(float a) { return fabsf(a); }
__device__ __forceinline__ double tmin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ double tmax(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ double tabs(double a) { return fabs(a); }
// |a| with the sign of b, b == 0 counted positive
template <typename T> __device__ __forceinline__ T tsign(T a, T b) {
  T m = tabs(a);
  return b < T(0) ? -m : m;
}
__device__ __forceinline__ float copysign_t(float a, float b) { return copysignf(a, b); }
__device__ __forceinline__ double copysign_t(double a, double b) { return copysign(a, b); }
// One element from global into shared memory by an asynchronous copy (FP32,
// FP64; other element types by a plain load); stage_wait waits for all of the
// thread's copies.
template <typename T>
__device__ __forceinline__ void copy_async(T* dst, const T* src) {
  if constexpr (sizeof(T) == 4 || sizeof(T) == 8) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    if constexpr (sizeof(T) == 4) asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src));
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src));
  } else {
    *dst = *src;
  }
}
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
// three-input min / max (one instruction for f32 on sm_100 and later)
__device__ __forceinline__ float tmax3(float a, float b, float c) {
  float r;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float tmin3(float a, float b, float c) {
  float r;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ double tmax3(double a, double b, double c) { return fmax(fmax(a, b), c); }
__device__ __forceinline__ double tmin3(double a, double b, double c) { return fmin(fmin(a, b), c); }
template <typename T> __device__ __forceinline__ T clamp2(T a, T x0, T x1) {
  return tmin(tmax(a, tmin(x0, x1)), tmax(x0, x1));
}

// Colella & Woodward (1984) eq. 1.10 in perturbation form (bl = aL - q, br = aR - q).
template <typename T> __device__ __forceinline__ void cw84(T& bl, T& br) {
  if (bl * br >= T(0)) {
    bl = T(0);
    br = T(0);
    return;
  }
  T d = br - bl;
  T t = T(3) * d * (bl + br);
  T d2 = d * d;
  if (-t > d2) bl = T(-2) * br;
  else if (t > d2) br = T(-2) * bl;
}

// Monotonized central slope in half-increment form.
template <typename T> __device__ __forceinline__ T vl_slope(T xm, T x0, T xp) {
  T xt = T(0.25) * (xp - xm);
  T smax = tmax(tmax(xm, x0), xp) - x0;
  T smin = x0 - tmin(tmin(xm, x0), xp);
  return tsign(tmin(tmin(tabs(xt), smax), smin), xt);
}

// Upwind integral of the sub-grid parabola over the swept fraction.
template <typename T>
__device__ __forceinline__ T ppm_flux(T c, T xl, T bll, T brl, T xr, T blr, T brr) {
  if (c > T(0)) return xl + (T(1) - c) * (brl - c * (bll + brl));
  return xr + (T(1) + c) * (blr + c * (blr + brr));
}

int set_error(int code, const char* fmt, ...);
int cuda_error(cudaError_t e, const char* what);

// A field of a batched state as the restart reader and writer see it: planes
// of the state's element type (esz 4 or 8) stacked [tile][tracer][level] (Q)
// or [tile][level] (DELP), the compute domain at pg.at(1..n, 1..n).
struct StateFieldView {
  void* dev;
  int esz;
  PlaneGeom pg;
  long long plane;
  int n, npz, nq, ntiles;
  cudaStream_t stream;
};
// loading: the field is about to be overwritten in part (Q: the latest tracer
// buffer becomes the home buffer first, so tracers not loaded keep their
// values); otherwise the field's latest values are viewed for writing out.
int state_field_view(fv3g_state* st, int field, bool loading, StateFieldView* v);

#define FV3G_CUDA(call)                                         \
  do {                                                          \
    cudaError_t e__ = (call);                                   \
    if (e__ != cudaSuccess) return ::fv3g::cuda_error(e__, #call); \
  } while (0)

// fillz over the interior columns of a state's planes (fv3g_l2e.cu)
template <typename T>
int launch_fillz_planes(T* q, const T* dp, int n, int ntiles, int km, int nq, long long sQt, long long sQq,
                        long long sQk, long long sFt, long long sFk, PlaneGeom pg, cudaStream_t s);

// Advection substep kernels, one translation unit per hord (fv3g_substep_h*.cu)
template <typename T, int HORD>
int launch_substep_hord(const AdvArgs<T>& a, bool flux_mode, int warps, cudaStream_t s);
template <int HORD>
int launch_substep_tl_hord(const AdvArgs<Dual<double>>& a, cudaStream_t s);
template <int HORD>
void prepare_substep_hord(cudaError_t& err);

// Tracer damping (fv3g_damp.cu): adds the deln_flux fluxes of a substep's
// input q_in (a.damp, a.nord) to the fluxes (flux mode) or to q_out and the
// tile-edge fluxes; runs after the substep kernel on the same stream.
template <typename T>
int launch_damp(const AdvArgs<T>& a, bool flux_mode, cudaStream_t s);
int launch_damp_tl(const AdvArgs<Dual<double>>& a, cudaStream_t s);  // nord 0, flux mode
// damp = (damp_c da_min)^(nord+1), as the product upstream's integer power is
double damp_coefficient(double damp_c, double da_min, int nord);

// Host launchers (fv3g_advect.cu)
template <typename T>
int launch_copy_halo_ring(T* dst, const T* src, long long splane, int nplanes, long long sQt, int ntiles,
                          PlaneGeom pg, int n, cudaStream_t s);
int launch_substep_tl(const AdvArgs<Dual<double>>& a, int hord, cudaStream_t s);
template <typename T>
int launch_cube_halo(T* q, long long sQt, long long splane, int nplanes, PlaneGeom pg, int n, const Topo& topo,
                     cudaStream_t s, int nlev = 0, long long sQq = 0);  // nlev > 0: planes of nlev levels, sQq apart
template <typename T>
int launch_substep(const AdvArgs<T>& a, int hord, bool flux_mode, int warps, cudaStream_t s);
int launch_substep_pair(const AdvArgs<float>& a, int warps, cudaStream_t s);
constexpr int PAIR_WIDTH_MAX = 12;  // warps (tracer pairs) per CTA of the paired substep
template <typename T>
int launch_edge_fix(const AdvArgs<T>& a, int n, cudaStream_t s);
// Unscaled Courant numbers and mass fluxes to read instead of scaling in place.
template <typename T>
struct AreaFluxSrc {
  const T* cx = nullptr;
  const T* cy = nullptr;
  const T* mfx = nullptr;
  const T* mfy = nullptr;
  // optional sticky error word: FV3G_E_NONFINITE for a non-finite Courant number or mass flux on a compute
  // face, FV3G_E_COURANT for a scaled Courant number above 1 in magnitude
  int* err = nullptr;
};
// xfx, yfx from the Courant numbers with the upwind metrics, and cx, cy, mfx,
// mfy scaled by frac (tracer_2d's prologue); with src, read from src and write
// the scaled values into cx.. (copies) instead of scaling in place.
template <typename T>
int launch_area_flux(T* cx, T* cy, T* xfx, T* yfx, T* mfx, T* mfy, const T* dxa, const T* dya,
                     const T* dx, const T* dy, const T* sin_sg, long long sFt, long long sFk,
                     long long sMt, long long sSin, PlaneGeom pg, int is, int ie, int js, int je,
                     int ntiles, int npz, T frac, cudaStream_t s, AreaFluxSrc<T> src = AreaFluxSrc<T>{});
template <typename T>
int launch_max_courant(const T* cx, const T* cy, long long sFt, long long sFk, PlaneGeom pg, int is,
                       int ie, int js, int je, int ntiles, int npz, unsigned long long* d_out, cudaStream_t s);

// Copy nplanes planes of width_bytes x height between pitched buffers
// (slice = bytes from one plane to the next); device-to-device and uploads
// from page-locked host memory by a kernel (max_ctas > 0 caps its grid, for
// copies that run beside compute kernels), other host copies staged or in
// chunks of cudaMemcpy3DAsync.
int copy_planes(void* dst, size_t dpitch, size_t dslice, const void* src, size_t spitch, size_t sslice,
                size_t width_bytes, size_t height, long long nplanes, cudaMemcpyKind kind, cudaStream_t s,
                int max_ctas = 0);

int prepare_kernels();
BlockMap block_map(int is, int ie, int js, int je, int npx, int npy, int nested);

}  // namespace fv3g
