// fv3g_mass.cu -- compensated FP64 global tracer mass, sum(q * delp * area)
// over the compute domain of every tile (the global-sum diagnostic that FV3
// computes with g_sum; MPI_Allreduce analogue at atmos_model.F90:496-502).
//
// Each thread accumulates a strided subset with Neumaier's compensated sum;
// blocks combine (sum, compensation) pairs in a fixed tree order into a
// partials buffer, and a single block reduces the partials per tracer, so
// the result is bitwise reproducible for a given problem size.
#include "fv3g_internal.cuh"
#include "fv3g_mass.cuh"

namespace fv3g {

__device__ __forceinline__ void neumaier(double& s, double& c, double x) {
  const double t = s + x;
  if (fabs(s) >= fabs(x)) c += (s - t) + x;
  else c += (x - t) + s;
  s = t;
}

// One warp per row (tile, level, j) in a grid-stride loop, lanes along i.
// FP64 fields: every term q*dp*area goes through Neumaier's sum.  FP32 fields:
// the term is formed in FP32 and added to a plain FP64 running sum (its
// rounding is random, ~1e-12 of the total over 1e9 terms), which keeps the
// FP64 pipe -- 1/64 of the FP32 rate on this GPU -- out of the inner loop; the
// per-thread partials are then combined with Neumaier's sum.
template <typename T>
__global__ void __launch_bounds__(256) k_mass_partial(const MassArgs<T> a) {
  const int iq = blockIdx.y;
  const int lane = threadIdx.x & 31;
  const int rows = a.ntiles * a.npz * a.nj;
  double s = 0.0, c = 0.0;
  for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < rows; r += gridDim.x * (blockDim.x >> 5)) {
    const int j = r % a.nj;
    const int tk = r / a.nj;
    const int k = tk % a.npz, t = tk / a.npz;
    const long long p0 = a.pg.at(a.i1, a.j1 + j);
    const T* qr = a.q + t * a.sQt + iq * a.sQq + k * a.sQk + p0;
    const T* dr = a.dp + t * a.sFt + k * a.sFk + p0;
    const T* ar = a.area + t * a.sMt + p0;
    if (Single<T>::value) {
      double acc = 0.0;
      for (int i = lane; i < a.ni; i += 32) acc += (double)(qr[i] * dr[i] * ar[i]);
      neumaier(s, c, acc);
    } else {
      for (int i = lane; i < a.ni; i += 32) neumaier(s, c, (double)qr[i] * (double)dr[i] * (double)ar[i]);
    }
  }
  __shared__ double ss[256], sc[256];
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      double s0 = ss[threadIdx.x], c0 = sc[threadIdx.x] + sc[threadIdx.x + o];
      neumaier(s0, c0, ss[threadIdx.x + o]);
      ss[threadIdx.x] = s0;
      sc[threadIdx.x] = c0;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    a.partials[2 * ((long long)iq * gridDim.x + blockIdx.x) + 0] = ss[0];
    a.partials[2 * ((long long)iq * gridDim.x + blockIdx.x) + 1] = sc[0];
  }
}

__global__ void k_mass_final(const double* partials, int nblk, int nq, double* out) {
  const int iq = blockIdx.x;
  __shared__ double ss[256], sc[256];
  double s = 0.0, c = 0.0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
    neumaier(s, c, partials[2 * ((long long)iq * nblk + b)]);
    c += partials[2 * ((long long)iq * nblk + b) + 1];
  }
  ss[threadIdx.x] = s;
  sc[threadIdx.x] = c;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) {
      double s0 = ss[threadIdx.x], c0 = sc[threadIdx.x] + sc[threadIdx.x + o];
      neumaier(s0, c0, ss[threadIdx.x + o]);
      ss[threadIdx.x] = s0;
      sc[threadIdx.x] = c0;
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) out[iq] = ss[0] + sc[0];
}

template <typename T>
int launch_mass(const MassArgs<T>& a, int nq, double* d_out, cudaStream_t s) {
  k_mass_partial<T><<<dim3(MASS_BLOCKS, nq), 256, 0, s>>>(a);
  FV3G_CUDA(cudaGetLastError());
  k_mass_final<<<nq, 256, 0, s>>>(a.partials, MASS_BLOCKS, nq, d_out);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

template int launch_mass<float>(const MassArgs<float>&, int, double*, cudaStream_t);
template int launch_mass<double>(const MassArgs<double>&, int, double*, cudaStream_t);

}  // namespace fv3g
