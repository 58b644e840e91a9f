// fv3g_remap.cuh -- arguments of the column remap kernel.
#pragma once

#include "fv3g_internal.cuh"

namespace fv3g {

constexpr int KMAX = 128;  // most layers per column (source or target)

template <typename T>
struct RemapArgs {
  const T* q_in;  // field planes, [tile][field][level]
  T* q_out;
  long long sQt, sQq, sQk;
  long long sQqo;  // field stride of q_out (kn levels)
  int nfield;
  const T* dp;  // Lagrangian thickness planes [tile][level] (batched mode)
  T* dp_out;    // target thickness (may be null)
  long long sFt, sFk;
  const double* ak;  // device, km+1 / kn+1 (batched mode)
  const double* bk;
  const double* pe1;  // drop-in mode: [k][col] interface pressures (null in batched mode)
  const double* pe2;
  const double* qs;  // [col] surface value for iv == -2 (may be null)
  const double* dp2;  // [k][col] target thicknesses dividing the overlap masses (map1_q2); null: pe2 differences
  PlaneGeom pg;
  int i1, j1, ni, nj;  // column block: i1..i1+ni-1, j1..j1+nj-1 on every tile
  long long ncol;      // ntiles * ni * nj
  int km, kn, iv;
  double q_min;
  // Null: the warp-per-column kernel (no scratch).  Set: the thread-per-column
  // kernel with this caller-owned scratch, 6 * (KMAX+1) * ncol elements and
  // (KMAX+1) * ncol schedule bytes.
  T* scratch;
  unsigned char* sched;
  // 0: the warp-per-column kernel; 1: the FP32 thread-per-column kernel
  // wherever it applies (batched kord 9, iv -1..1, at least 16 layers), else
  // the warp kernel
  int form;
};

template <typename T>
int launch_remap(const RemapArgs<T>& a, int kord, cudaStream_t s);
size_t remap_scratch_bytes(long long ncol, size_t elem_bytes);
// the FP32 thread-per-column kernel of the batched remap (fv3g_remap_col.cu)
bool remap_col_applies(const RemapArgs<float>& a, int kord);
cudaError_t launch_remap_col(const RemapArgs<float>& a, cudaStream_t s);  // scratch + schedule of the scratch kernel
int prepare_remap_kernels();
int launch_remap_tl(const RemapArgs<Dual<double>>& a, int kord, cudaStream_t s);
// interface pressures of the columns of a field kind (cells, u or v faces) for the remap of extra fields
template <typename T>
int launch_field_pressures(const T* dp, long long sFt, long long sFk, PlaneGeom pg, int nt, int km, int ni, int nj,
                           int kind, int log_p, const double* ak, const double* bk, double* pe1, double* pe2,
                           cudaStream_t s);

}  // namespace fv3g
