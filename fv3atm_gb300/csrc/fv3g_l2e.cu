// fv3g_l2e.cu -- the column pieces of Lagrangian_to_Eulerian (fv_mapz.F90)
// around the tracer remap: the fillz negative filler (fv_fill.F90) and the
// recompute of the pressure variables pe, peln, pk, pkz from the remapped
// thickness.  One thread per column (and tracer); consecutive threads own
// consecutive i, so every level is a coalesced row.
//
// fillz, restated: a negative top layer is pushed into the layer below; an
// interior negative borrows first from the layer above, then from the layer
// below, as much as they hold; a negative bottom layer borrows from above;
// where negatives remain, the column's positive layer masses are scaled by
// (total mass)/(positive mass) and the negatives zeroed (no change when the
// total is not positive).  The column mass is conserved throughout.
#include <cuda_runtime.h>

#include <cmath>

#include "fv3g_hostio.cuh"

namespace fv3g {

// One column of one tracer: level k at Q[sq*k], thickness at D[sd*k].
template <typename T>
__device__ void fill_column(T* Q, const T* D, long long sq, long long sd, int km) {
  if (km < 2) return;
  auto qv = [&](int k) -> T& { return Q[sq * k]; };
  auto dv = [&](int k) { return D[sd * k]; };
  if (qv(0) < T(0)) {
    qv(1) += qv(0) * dv(0) / dv(1);
    qv(0) = T(0);
  }
  bool fix = false;
  for (int k = 1; k < km - 1; ++k) {
    if (qv(k) >= T(0)) continue;
    fix = true;
    if (qv(k - 1) > T(0)) {
      const T d = fmin(qv(k - 1) * dv(k - 1), -qv(k) * dv(k));
      qv(k - 1) -= d / dv(k - 1);
      qv(k) += d / dv(k);
    }
    if (qv(k) < T(0) && qv(k + 1) > T(0)) {
      const T d = fmin(qv(k + 1) * dv(k + 1), -qv(k) * dv(k));
      qv(k + 1) -= d / dv(k + 1);
      qv(k) += d / dv(k);
    }
  }
  const int kb = km - 1;
  if (qv(kb) < T(0) && qv(kb - 1) > T(0)) {
    fix = true;
    const T d = fmin(qv(kb - 1) * dv(kb - 1), -qv(kb) * dv(kb));
    qv(kb - 1) -= d / dv(kb - 1);
    qv(kb) += d / dv(kb);
  }
  if (!fix) return;
  double tot = 0.0, pos = 0.0;
  for (int k = 0; k < km; ++k) {
    const double m = (double)qv(k) * (double)dv(k);
    tot += m;
    pos += fmax(m, 0.0);
  }
  if (tot > 0.0 && pos > 0.0 && tot < pos) {
    const double f = tot / pos;
    for (int k = 0; k < km; ++k) qv(k) = T(fmax((double)qv(k), 0.0) * f);
  }
}

// Fortran row layout: q (i, k, iq) at i + sI*k + sQ*iq, dp (i, k) at i + sI*k
template <typename T>
__global__ void k_fillz(T* q, const T* dp, int im, int km, int nq, long long sI, long long sQ) {
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= (long long)im * nq) return;
  const int i = (int)(id % im), iq = (int)(id / im);
  fill_column(q + i + sQ * iq, dp + i, sI, sI, km);
}

// Device planes of a state: the interior columns of every tile and tracer
template <typename T>
__global__ void k_fillz_planes(T* q, const T* dp, int n, int ntiles, int km, int nq, long long sQt, long long sQq,
                               long long sQk, long long sFt, long long sFk, PlaneGeom pg) {
  const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long ncol = (long long)ntiles * n * n;
  if (id >= ncol * nq) return;
  const long long c = id % ncol;
  const int iq = (int)(id / ncol);
  const int i = (int)(c % n), j = (int)((c / n) % n), t = (int)(c / ((long long)n * n));
  const long long p = pg.at(1 + i, 1 + j);
  fill_column(q + t * sQt + iq * sQq + p, dp + t * sFt + p, sQk, sFk, km);
}

__global__ void k_pressure_vars(const double* delp, double* pe, double* peln, double* pk, double* pkz, int im, int km,
                                double ptop, double akap) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= im) return;
  double p = ptop, lp = log(ptop), kp = exp(akap * lp);
  pe[i] = p;
  peln[i] = lp;
  pk[i] = kp;
  for (int k = 0; k < km; ++k) {
    p += delp[i + (long long)im * k];
    const double lp1 = log(p), kp1 = exp(akap * lp1);
    const long long o = i + (long long)im * (k + 1);
    pe[o] = p;
    peln[o] = lp1;
    pk[o] = kp1;
    pkz[i + (long long)im * k] = (kp1 - kp) / (akap * (lp1 - lp));
    lp = lp1;
    kp = kp1;
  }
}

template <typename T>
int launch_fillz(T* q, const T* dp, int im, int km, int nq, long long sI, long long sQ, cudaStream_t s) {
  const long long n = (long long)im * nq;
  k_fillz<T><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(q, dp, im, km, nq, sI, sQ);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

template <typename T>
int launch_fillz_planes(T* q, const T* dp, int n, int ntiles, int km, int nq, long long sQt, long long sQq,
                        long long sQk, long long sFt, long long sFk, PlaneGeom pg, cudaStream_t s) {
  const long long tot = (long long)ntiles * n * n * nq;
  k_fillz_planes<T><<<(unsigned)((tot + 127) / 128), 128, 0, s>>>(q, dp, n, ntiles, km, nq, sQt, sQq, sQk, sFt, sFk,
                                                                   pg);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

template int launch_fillz<double>(double*, const double*, int, int, int, long long, long long, cudaStream_t);
template int launch_fillz_planes<float>(float*, const float*, int, int, int, int, long long, long long, long long,
                                        long long, long long, PlaneGeom, cudaStream_t);
template int launch_fillz_planes<double>(double*, const double*, int, int, int, int, long long, long long, long long,
                                         long long, long long, PlaneGeom, cudaStream_t);

}  // namespace fv3g

extern "C" {

int fv3g_fillz(int im, int km, int nq, double* q, const double* dp) {
  if (im < 1 || km < 1 || nq < 1) return set_error(FV3G_E_ARG, "fillz needs im, km, nq >= 1");
  if (!q || !dp) return set_error(FV3G_E_ARG, "null array argument");
  const size_t nqv = (size_t)im * km * nq, ndp = (size_t)im * km;
  CHECK(g_ctx.begin(padded(nqv, 8) + padded(ndp, 8)));
  cudaStream_t s = g_ctx.stream;
  double* dq = g_ctx.take<double>(nqv);
  double* dd = g_ctx.take<double>(ndp);
  FV3G_CUDA(cudaMemcpyAsync(dq, q, nqv * 8, cudaMemcpyHostToDevice, s));
  FV3G_CUDA(cudaMemcpyAsync(dd, dp, ndp * 8, cudaMemcpyHostToDevice, s));
  CHECK(fv3g::launch_fillz<double>(dq, dd, im, km, nq, im, (long long)im * km, s));
  FV3G_CUDA(cudaMemcpyAsync(q, dq, nqv * 8, cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  return 0;
}

int fv3g_pressure_vars(int im, int km, double ptop, double akap, const double* delp, double* pe, double* peln,
                       double* pk, double* pkz) {
  if (im < 1 || km < 1) return set_error(FV3G_E_ARG, "pressure_vars needs im, km >= 1");
  if (!(ptop > 0.0) || !(akap > 0.0)) return set_error(FV3G_E_ARG, "ptop and akap must be positive");
  if (!delp || !pe || !peln || !pk || !pkz) return set_error(FV3G_E_ARG, "null array argument");
  const size_t nl = (size_t)im * km, ni = (size_t)im * (km + 1);
  CHECK(g_ctx.begin(padded(nl, 8) * 2 + padded(ni, 8) * 3));
  cudaStream_t s = g_ctx.stream;
  double *d_dp = g_ctx.take<double>(nl), *d_pe = g_ctx.take<double>(ni), *d_ln = g_ctx.take<double>(ni);
  double *d_pk = g_ctx.take<double>(ni), *d_pkz = g_ctx.take<double>(nl);
  FV3G_CUDA(cudaMemcpyAsync(d_dp, delp, nl * 8, cudaMemcpyHostToDevice, s));
  fv3g::k_pressure_vars<<<(im + 127) / 128, 128, 0, s>>>(d_dp, d_pe, d_ln, d_pk, d_pkz, im, km, ptop, akap);
  FV3G_CUDA(cudaGetLastError());
  FV3G_CUDA(cudaMemcpyAsync(pe, d_pe, ni * 8, cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaMemcpyAsync(peln, d_ln, ni * 8, cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaMemcpyAsync(pk, d_pk, ni * 8, cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaMemcpyAsync(pkz, d_pkz, nl * 8, cudaMemcpyDeviceToHost, s));
  FV3G_CUDA(cudaStreamSynchronize(s));
  return 0;
}

}  // extern "C"
