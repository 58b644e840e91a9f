// fv3g_hostio.cuh -- shared by the exact-shape (host-array) entries: a
// per-thread stream and device arena, host <-> device plane copies of Fortran
// arrays with explicit bounds, bounds checks and the copy_corners kernel.
// Everything here has internal linkage, one copy per translation unit.
#pragma once

#include <cuda_runtime.h>

#include "fv3g_internal.cuh"

using namespace fv3g;

namespace {

#define CHECK(expr)             \
  do {                          \
    int rc__ = (expr);          \
    if (rc__ != 0) return rc__; \
  } while (0)

// Per-thread stream and a grow-only device arena, released at thread exit.
struct ThreadCtx {
  cudaStream_t stream = nullptr;
  char* arena = nullptr;
  size_t cap = 0, used = 0;
  ~ThreadCtx() {
    if (arena) cudaFree(arena);
    if (stream) cudaStreamDestroy(stream);
  }
  int begin(size_t bytes) {
    if (!stream) FV3G_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    bytes += 64 * 256;
    if (cap < bytes) {
      if (arena) cudaFree(arena);
      arena = nullptr;
      cap = 0;
      FV3G_CUDA(cudaMalloc((void**)&arena, bytes));
      cap = bytes;
    }
    used = 0;
    return 0;
  }
  template <typename T>
  T* take(size_t count) {
    T* p = (T*)(arena + used);
    used += ((count * sizeof(T) + 255) / 256) * 256;
    return p;
  }
};
thread_local ThreadCtx g_ctx;

size_t padded(size_t count, size_t es) { return ((count * es + 255) / 256) * 256; }

// Copy a host Fortran array with bounds (ilo:ihi, jlo:jhi, nplanes) into
// device planes of geometry pg (which must contain those bounds).
int h2d_planes(double* dev, const PlaneGeom& pg, const double* host, int ilo, int ihi, int jlo, int jhi,
               long long nplanes, cudaStream_t s) {
  const int ni = ihi - ilo + 1, nj = jhi - jlo + 1;
  return copy_planes(dev + pg.at(ilo, jlo), (size_t)pg.pitch * 8, (size_t)pg.plane() * 8, host, (size_t)ni * 8,
                     (size_t)ni * nj * 8, (size_t)ni * 8, nj, nplanes, cudaMemcpyHostToDevice, s);
}

int d2h_planes(double* host, const double* dev, const PlaneGeom& pg, int ilo, int ihi, int jlo, int jhi,
               long long nplanes, cudaStream_t s) {
  const int ni = ihi - ilo + 1, nj = jhi - jlo + 1;
  return copy_planes(host, (size_t)ni * 8, (size_t)ni * nj * 8, dev + pg.at(ilo, jlo), (size_t)pg.pitch * 8,
                     (size_t)pg.plane() * 8, (size_t)ni * 8, nj, nplanes, cudaMemcpyDeviceToHost, s);
}

int d2d_planes(double* dst, const double* src, const PlaneGeom& pg, int ilo, int ihi, int jlo, int jhi,
               long long nplanes, cudaStream_t s) {
  const int ni = ihi - ilo + 1, nj = jhi - jlo + 1;
  return copy_planes(dst + pg.at(ilo, jlo), (size_t)pg.pitch * 8, (size_t)pg.plane() * 8, src + pg.at(ilo, jlo),
                     (size_t)pg.pitch * 8, (size_t)pg.plane() * 8, (size_t)ni * 8, nj, nplanes,
                     cudaMemcpyDeviceToDevice, s);
}

__global__ void k_corners(double* q, PlaneGeom pg, int npx, int npy, int corners, int dir, long long nplanes) {
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
  if (i < pg.isd || j < pg.jsd || is < pg.isd || js < pg.jsd || i >= pg.isd + pg.pitch || is >= pg.isd + pg.pitch ||
      j >= pg.jsd + pg.rows || js >= pg.jsd + pg.rows)
    return;
  q[p * pg.plane() + pg.at(i, j)] = q[p * pg.plane() + pg.at(is, js)];
}

__global__ void k_max_abs2(const double* cx, const double* cy, PlaneGeom pg, int is, int ie, int js, int je, int npz,
                           unsigned long long* out) {
  const long long per = (long long)(ie - is + 1) * (je - js + 1);
  double m = 0.0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < per * npz; e += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(e / per);
    const long long r = e % per;
    const int i = is + (int)(r % (ie - is + 1)), j = js + (int)(r / (ie - is + 1));
    const long long p = (long long)k * pg.plane() + pg.at(i, j);
    m = fmax(m, fmax(fabs(cx[p]), fabs(cy[p])));
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

int check_bounds(const fv3g_bounds* bd, int npx, int npy) {
  if (!bd) return set_error(FV3G_E_ARG, "null bounds");
  if (bd->ng != 3) return set_error(FV3G_E_ARG, "halo width ng must be 3 (got %d)", bd->ng);
  if (bd->isd != bd->is - 3 || bd->ied != bd->ie + 3 || bd->jsd != bd->js - 3 || bd->jed != bd->je + 3)
    return set_error(FV3G_E_ARG, "data domain must be the compute domain plus a 3-cell halo");
  if (bd->ie < bd->is || bd->je < bd->js) return set_error(FV3G_E_ARG, "empty compute domain");
  if (bd->is < 1 || bd->js < 1 || bd->ie > npx - 1 || bd->je > npy - 1)
    return set_error(FV3G_E_ARG, "compute domain outside the tile (npx=%d, npy=%d)", npx, npy);
  return 0;
}

PlaneGeom plane_for(const fv3g_bounds* bd) {
  PlaneGeom pg;
  pg.isd = bd->isd;
  pg.jsd = bd->jsd;
  pg.pitch = ((bd->ied - bd->isd + 2 + 7) / 8) * 8;
  pg.rows = bd->jed - bd->jsd + 2;
  return pg;
}

int corner_mask(const fv3g_grid* g) {
  return (g->sw_corner ? 1 : 0) | (g->se_corner ? 2 : 0) | (g->nw_corner ? 4 : 0) | (g->ne_corner ? 8 : 0);
}

}  // namespace
