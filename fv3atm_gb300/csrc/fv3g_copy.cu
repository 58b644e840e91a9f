// fv3g_copy.cu -- pitched copies of stacks of planes.
//
// Device-to-device stacks are moved by a kernel (4-byte words, a warp per
// row).  An upload from page-locked host memory (cudaHostAlloc /
// cudaHostRegister) is the same kernel reading the host array through the
// NVLink-C2C link, with the pitch change on the fly (measured ~180 GB/s,
// also when copy-engine reads of host memory are degraded).  Other dense host
// stacks, and every download, go through a per-thread device staging buffer:
// one large cudaMemcpyAsync per 256 MB chunk (copy engine; faster than SM
// stores for writes to the host) and the pitch change in device memory.
// Non-dense host stacks are issued as cudaMemcpy3DAsync calls of at most
// kChunk planes each.
#include <algorithm>

#include "fv3g_internal.cuh"

namespace fv3g {

namespace {
#define CHECK_RC(expr)          \
  do {                          \
    int rc__ = (expr);          \
    if (rc__ != 0) return rc__; \
  } while (0)

constexpr long long kChunk = 256;

// One warp per row of one plane (rows in a grid-stride loop, one integer
// division per row), the row's words across the lanes: coalesced rows.  Each
// lane loads four words before storing them, so a warp keeps 512 bytes of
// reads in flight (reads of host memory over the link have microseconds of
// latency).
__global__ void k_copy_planes(unsigned* dst, long long dpitch, long long dslice, const unsigned* src, long long spitch,
                              long long sslice, int width, int height, long long nplanes) {
  const long long rows = (long long)height * nplanes;
  const int lane = threadIdx.x & 31;
  const long long w0 = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long r = w0; r < rows; r += nw) {
    const long long p = r / height;
    const long long y = r - p * height;
    unsigned* d = dst + p * dslice + y * dpitch;
    const unsigned* sp = src + p * sslice + y * spitch;
    for (int x0 = 0; x0 < width; x0 += 128) {
      unsigned v[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int x = x0 + 32 * u + lane;
        if (x < width) v[u] = sp[x];
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int x = x0 + 32 * u + lane;
        if (x < width) d[x] = v[u];
      }
    }
  }
}
}  // namespace

namespace {
// Per-thread staging buffer; `done` marks the end of its last use, which a
// copy on any stream waits for before reusing the buffer.
struct Staging {
  void* buf = nullptr;
  size_t cap = 0;
  cudaEvent_t done = nullptr;
  ~Staging() {
    if (buf) cudaFree(buf);
    if (done) cudaEventDestroy(done);
  }
};
thread_local Staging g_staging;
constexpr size_t kStageBytes = size_t(256) << 20;

int device_words(void* dst, size_t dpitch, size_t dslice, const void* src, size_t spitch, size_t sslice,
                 size_t width_bytes, size_t height, long long nplanes, cudaStream_t s, int max_ctas = 0) {
  const long long rows = (long long)height * nplanes;
  const long long cap = max_ctas > 0 ? max_ctas : 152LL * 16;
  const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>((rows + 7) / 8, cap));
  k_copy_planes<<<grid, 256, 0, s>>>((unsigned*)dst, (long long)(dpitch / 4), (long long)(dslice / 4),
                                     (const unsigned*)src, (long long)(spitch / 4), (long long)(sslice / 4),
                                     (int)(width_bytes / 4), (int)height, nplanes);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

// dense host stack <-> pitched device stack through the staging buffer
int staged_copy(void* dst, size_t dpitch, size_t dslice, const void* src, size_t spitch, size_t sslice,
                size_t width_bytes, size_t height, long long nplanes, bool h2d, cudaStream_t s, int max_ctas) {
  Staging& g = g_staging;
  const size_t plane = width_bytes * height;
  const long long per = std::max<long long>(1, (long long)(kStageBytes / plane));
  const size_t need = (size_t)std::min<long long>(per, nplanes) * plane;
  if (g.cap < need) {
    if (g.buf) {
      FV3G_CUDA(cudaEventSynchronize(g.done));
      cudaFree(g.buf);
      g.buf = nullptr;
      g.cap = 0;
    }
    FV3G_CUDA(cudaMalloc(&g.buf, std::max(need, size_t(1) << 20)));
    g.cap = std::max(need, size_t(1) << 20);
  }
  if (!g.done) FV3G_CUDA(cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming));
  FV3G_CUDA(cudaStreamWaitEvent(s, g.done, 0));
  for (long long p0 = 0; p0 < nplanes; p0 += per) {
    const long long np = std::min(per, nplanes - p0);
    if (h2d) {
      FV3G_CUDA(cudaMemcpyAsync(g.buf, (const char*)src + p0 * sslice, np * plane, cudaMemcpyHostToDevice, s));
      CHECK_RC(device_words((char*)dst + p0 * dslice, dpitch, dslice, g.buf, width_bytes, plane, width_bytes, height,
                            np, s, max_ctas));
    } else {
      CHECK_RC(device_words(g.buf, width_bytes, plane, (const char*)src + p0 * sslice, spitch, sslice, width_bytes,
                            height, np, s, max_ctas));
      FV3G_CUDA(cudaMemcpyAsync((char*)dst + p0 * dslice, g.buf, np * plane, cudaMemcpyDeviceToHost, s));
    }
  }
  FV3G_CUDA(cudaEventRecord(g.done, s));
  return 0;
}
}  // namespace

int copy_planes(void* dst, size_t dpitch, size_t dslice, const void* src, size_t spitch, size_t sslice,
                size_t width_bytes, size_t height, long long nplanes, cudaMemcpyKind kind, cudaStream_t s,
                int max_ctas) {
  if (nplanes <= 0 || width_bytes == 0 || height == 0) return 0;
  if (kind == cudaMemcpyDeviceToDevice) {
    if ((dpitch | dslice | spitch | sslice | width_bytes | (size_t)dst | (size_t)src) & 3)
      return set_error(FV3G_E_ARG, "device plane copy needs 4-byte aligned pitches and pointers");
    return device_words(dst, dpitch, dslice, src, spitch, sslice, width_bytes, height, nplanes, s);
  }
  if (kind == cudaMemcpyHostToDevice) {  // page-locked host memory: the GPU reads the host array directly
    cudaPointerAttributes at{};
    const cudaError_t qe = cudaPointerGetAttributes(&at, src);
    if (qe != cudaSuccess) cudaGetLastError();  // pageable memory on older drivers: clear and stage
    const bool aligned = !((dpitch | dslice | spitch | sslice | width_bytes | (size_t)dst | (size_t)src) & 3);
    if (qe == cudaSuccess && at.type == cudaMemoryTypeHost && at.devicePointer != nullptr && aligned)
      return device_words(dst, dpitch, dslice, at.devicePointer, spitch, sslice, width_bytes, height, nplanes, s,
                          max_ctas);
  }
  {  // dense pageable host side: staged
    const bool h2d = kind == cudaMemcpyHostToDevice;
    const size_t hp = h2d ? spitch : dpitch, hs = h2d ? sslice : dslice;
    const size_t dp = h2d ? dpitch : spitch, ds = h2d ? dslice : sslice;
    const void* dev = h2d ? dst : src;
    const bool aligned = !((dp | ds | width_bytes | (size_t)dev) & 3);
    if (hp == width_bytes && hs == width_bytes * height && aligned)
      return staged_copy(dst, dpitch, dslice, src, spitch, sslice, width_bytes, height, nplanes, h2d, s, max_ctas);
  }
  for (long long p0 = 0; p0 < nplanes; p0 += kChunk) {
    const long long np = std::min(kChunk, nplanes - p0);
    cudaMemcpy3DParms p{};
    p.srcPtr = make_cudaPitchedPtr((char*)src + p0 * sslice, spitch, spitch, sslice / spitch);
    p.dstPtr = make_cudaPitchedPtr((char*)dst + p0 * dslice, dpitch, dpitch, dslice / dpitch);
    p.extent = make_cudaExtent(width_bytes, height, (size_t)np);
    p.kind = kind;
    FV3G_CUDA(cudaMemcpy3DAsync(&p, s));
  }
  return 0;
}

}  // namespace fv3g
