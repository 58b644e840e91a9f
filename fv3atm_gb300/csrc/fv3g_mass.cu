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

template <typename T>
__global__ void __launch_bounds__(256) k_mass_partial(const MassArgs<T> a) {
  const int iq = blockIdx.y;
  const long long per_tile = (long long)a.npz * a.ni * a.nj;
  const long long tot = per_tile * a.ntiles;
  double s = 0.0, c = 0.0;
  for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const int i = (int)(e % a.ni);
    long long r = e / a.ni;
    const int j = (int)(r % a.nj);
    r /= a.nj;
    const int k = (int)(r % a.npz);
    const int t = (int)(r / a.npz);
    const long long p = a.pg.at(a.i1 + i, a.j1 + j);
    const double q = (double)a.q[t * a.sQt + iq * a.sQq + k * a.sQk + p];
    const double dp = (double)a.dp[t * a.sFt + k * a.sFk + p];
    const double ar = (double)a.area[t * a.sMt + p];
    neumaier(s, c, q * dp * ar);
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
