// fv3g_copy.cu -- pitched copies of stacks of planes.
//
// Device-to-device stacks are moved by a kernel (4-byte words, one grid-stride
// loop); host<->device stacks are issued as cudaMemcpy3DAsync calls of at most
// kChunk planes each, with every pitched pointer's logical width given in
// bytes.
#include <algorithm>

#include "fv3g_internal.cuh"

namespace fv3g {

namespace {
constexpr long long kChunk = 256;

__global__ void k_copy_planes(unsigned* dst, long long dpitch, long long dslice, const unsigned* src, long long spitch,
                              long long sslice, int width, int height, long long nplanes) {
  const long long tot = (long long)width * height * nplanes;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(e % width);
    const long long r = e / width;
    const int y = (int)(r % height);
    const long long p = r / height;
    dst[p * dslice + (long long)y * dpitch + x] = src[p * sslice + (long long)y * spitch + x];
  }
}
}  // namespace

int copy_planes(void* dst, size_t dpitch, size_t dslice, const void* src, size_t spitch, size_t sslice,
                size_t width_bytes, size_t height, long long nplanes, cudaMemcpyKind kind, cudaStream_t s) {
  if (nplanes <= 0 || width_bytes == 0 || height == 0) return 0;
  if (kind == cudaMemcpyDeviceToDevice) {
    if ((dpitch | dslice | spitch | sslice | width_bytes | (size_t)dst | (size_t)src) & 3)
      return set_error(FV3G_E_ARG, "device plane copy needs 4-byte aligned pitches and pointers");
    const long long words = (long long)(width_bytes / 4) * (long long)height * nplanes;
    const unsigned grid = (unsigned)std::max<long long>(1, std::min<long long>((words + 255) / 256, 152LL * 32));
    k_copy_planes<<<grid, 256, 0, s>>>((unsigned*)dst, (long long)(dpitch / 4), (long long)(dslice / 4),
                                       (const unsigned*)src, (long long)(spitch / 4), (long long)(sslice / 4),
                                       (int)(width_bytes / 4), (int)height, nplanes);
    FV3G_CUDA(cudaGetLastError());
    return 0;
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
