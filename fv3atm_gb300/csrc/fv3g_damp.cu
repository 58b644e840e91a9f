// fv3g_damp.cu -- del-2(nord+1) tracer damping of tracer_2d / fv_tp_2d
// (deln_flux of tp_core.F90, GFDL_atmos_cubed_sphere; absent submodule,
// .gitmodules:1-4), as a kernel that runs after the advection substep kernel
// of the same substep, on the same stream.
//
// One CTA per 26 x 26 block of one (tile, level) holds a 32 x 32 window (the
// block and its 3-cell halo) in shared memory and loops over the tracers.
// Per tracer:
//   field d = q (mass-weighted damping) or damp q, on the window;
//   for each of the nord+1 orders: the copy_corners fill of d's cube-corner
//   blocks for an x sweep (nord > 0), x fluxes del6_v (d(i-1) - d(i)); the fill
//   for a y sweep, y fluxes del6_u (d(j-1) - d(j)); between orders d becomes
//   the flux divergence times rarea and the next difference is taken the
//   other way round, so the flux of every order damps;
//   the fluxes of the block's faces, weighted by 0.5 damp (dp1 + dp1') when
//   mass-weighted, are added to the flux planes (flux mode), or their
//   divergence times rarea / dp2 to q_out and, at the tile edges, to the
//   outward edge fluxes that the tile-edge reconciliation reads.
// Each order shrinks the valid part of the window by one cell per side; the
// 3-cell halo holds nord <= 2 (upstream's limit without extra ghosting).
#include <cuda_runtime.h>

#include <mutex>

#include "fv3g_stencil.cuh"

namespace fv3g {

template <typename T>
struct SmemDamp {
  T d[WIN][PQ];    // field on the window
  T fx[WIN][PQ];   // x fluxes [window row][face f], face f between window cells f-1 and f
  T fy[WIN][PQ];   // y fluxes [face f][window column]
  T d6v[WIN][PQ];  // del6_v at the x faces
  T d6u[WIN][PQ];  // del6_u at the y faces
};

template <typename T, int NORD, bool FLUXES>
__global__ void __launch_bounds__(256) k_damp(const AdvArgs<T> a, int nbx) {
  extern __shared__ __align__(16) unsigned char damp_raw[];
  SmemDamp<T>& S = *reinterpret_cast<SmemDamp<T>*>(damp_raw);
  const int t = blockIdx.z, k = blockIdx.y;
  const int bx = blockIdx.x % nbx, by = blockIdx.x / nbx;
  const int i0 = a.is + bx * TW, j0 = a.js + by * TW;
  const int ni = min(TW, a.ie - i0 + 1), nj = min(TW, a.je - j0 + 1);
  const PlaneGeom& pg = a.pg;
  const int tid = threadIdx.x, nth = blockDim.x;
  const T* rarea = a.rarea + t * a.sMt;
  {
    const T* d6u = a.del6_u + t * a.sMt;
    const T* d6v = a.del6_v + t * a.sMt;
    for (int e = tid; e < WIN * WIN; e += nth) {
      const int r = e / WIN, w = e % WIN;
      S.d6v[r][w] = ld_field(d6v, pg, i0 - 3 + w, j0 - 3 + r);
      S.d6u[r][w] = ld_field(d6u, pg, i0 - 3 + w, j0 - 3 + r);
    }
  }
  const bool corner_block = NORD > 0 && !a.nested && a.corners != 0 &&
                            ((i0 - 3 < 1) || (i0 + 28 > a.npx - 1)) && ((j0 - 3 < 1) || (j0 + 28 > a.npy - 1));
  // copy_corners on the window: a cube-corner block cell takes the value of
  // the strip cell its rotation lands on (never a corner cell, so one pass)
  auto fill_corners = [&](int dir) {
    for (int e = tid; e < WIN * WIN; e += nth) {
      const int r = e / WIN, w = e % WIN;
      int i = i0 - 3 + w, j = j0 - 3 + r;
      const bool oi = (i < 1) || (i > a.npx - 1), oj = (j < 1) || (j > a.npy - 1);
      if (!(oi && oj)) continue;
      const int bit = (i < 1 ? 0 : 1) + (j < 1 ? 0 : 2);
      if (!(a.corners & (1 << bit))) continue;
      corner_rotate(i, j, a.npx, a.npy, dir);
      const int ws = i - (i0 - 3), rs = j - (j0 - 3);
      if (ws >= 0 && ws < WIN && rs >= 0 && rs < WIN) S.d[r][w] = S.d[rs][ws];
    }
  };
  const T* mass = a.damp_mass ? a.dp1 + t * a.sFt + k * a.sFk : nullptr;
  const T damp2 = a.damp * T(0.5);
  auto wx = [&](T F, int i, int j) {  // x face i of row j
    return mass ? (damp2 * (ld_field(mass, pg, i - 1, j) + ld_field(mass, pg, i, j))) * F : F;
  };
  auto wy = [&](T F, int i, int j) {  // y face j of column i
    return mass ? (damp2 * (ld_field(mass, pg, i, j - 1) + ld_field(mass, pg, i, j))) * F : F;
  };
  const int n = a.npx - 1;
  const long long efe = (long long)a.npz * a.nq * n;
  const long long efo = (((long long)t * 4) * a.npz + k) * a.nq * n;
  const bool edges = !FLUXES && a.cube && a.eflux != nullptr;

#pragma unroll 1
  for (int iq = 0; iq < a.nq; ++iq) {
    const T* qin = a.q_in + t * a.sQt + iq * a.sQq + k * a.sQk;
    const T f0 = mass ? T(1) : a.damp;
    __syncthreads();  // the previous tracer's fluxes are consumed
    for (int e = tid; e < WIN * WIN; e += nth) {
      const int r = e / WIN, w = e % WIN;
      S.d[r][w] = f0 * ld_field(qin, pg, i0 - 3 + w, j0 - 3 + r);
    }
    __syncthreads();
#pragma unroll 1
    for (int o = 0; o <= NORD; ++o) {
      const T sg = (o == 0) ? T(1) : T(-1);
      if (corner_block) {
        fill_corners(1);
        __syncthreads();
      }
      for (int e = tid; e < WIN * WIN; e += nth) {
        const int r = e / WIN, f = e % WIN;
        if (f >= 1) S.fx[r][f] = sg * (S.d6v[r][f] * (S.d[r][f - 1] - S.d[r][f]));
      }
      __syncthreads();
      if (corner_block) {
        fill_corners(2);
        __syncthreads();
      }
      for (int e = tid; e < WIN * WIN; e += nth) {
        const int f = e / WIN, w = e % WIN;
        if (f >= 1) S.fy[f][w] = sg * (S.d6u[f][w] * (S.d[f - 1][w] - S.d[f][w]));
      }
      __syncthreads();
      if (o < NORD) {
        for (int e = tid; e < WIN * WIN; e += nth) {
          const int r = e / WIN, w = e % WIN;
          if (r >= 1 && r < WIN - 1 && w >= 1 && w < WIN - 1)
            S.d[r][w] = (S.fx[r][w] - S.fx[r][w + 1] + S.fy[r][w] - S.fy[r + 1][w]) *
                        ld_field(rarea, pg, i0 - 3 + w, j0 - 3 + r);
        }
        __syncthreads();
      }
    }
    // ------------------------------------------------------------- output
    if (FLUXES) {
      // each face once: a block owns its west and south faces, the last
      // block of a row or column also the tile's east or north face
      T* fxo = a.fx_out + (long long)(k * a.nq + iq) * a.sFlux;
      T* fyo = a.fy_out + (long long)(k * a.nq + iq) * a.sFlux;
      for (int e = tid; e < TW * NF; e += nth) {
        const int r = e / NF, f = e % NF;
        const int i = i0 + f, j = j0 + r;
        if (r < nj && (f < ni || (f == ni && i == a.ie + 1))) fxo[pg.at(i, j)] += wx(S.fx[r + 3][f + 3], i, j);
      }
      for (int e = tid; e < NF * TW; e += nth) {
        const int f = e / TW, c = e % TW;
        const int i = i0 + c, j = j0 + f;
        if (c < ni && (f < nj || (f == nj && j == a.je + 1))) fyo[pg.at(i, j)] += wy(S.fy[f + 3][c + 3], i, j);
      }
    } else {
      T* qo = a.q_out + t * a.sQt + iq * a.sQq + k * a.sQk;
      const T* dp2 = a.dp2 + t * a.sFt + k * a.sFk;
      for (int e = tid; e < TW * TW; e += nth) {
        const int r = e / TW, c = e % TW;
        if (r >= nj || c >= ni) continue;
        const int i = i0 + c, j = j0 + r;
        const T fxw = wx(S.fx[r + 3][c + 3], i, j), fxe = wx(S.fx[r + 3][c + 4], i + 1, j);
        const T fys = wy(S.fy[r + 3][c + 3], i, j), fyn = wy(S.fy[r + 4][c + 3], i, j + 1);
        const long long p = pg.at(i, j);
        qo[p] += (fxw - fxe + fys - fyn) * (rarea[p] / dp2[p]);
        if (edges) {  // outward fluxes of the tile-edge faces
          if (i == 1) a.eflux[efo + iq * (long long)n + (j - 1)] -= fxw;
          if (i == n) a.eflux[efo + efe + iq * (long long)n + (j - 1)] += fxe;
          if (j == 1) a.eflux[efo + 2 * efe + iq * (long long)n + (i - 1)] -= fys;
          if (j == n) a.eflux[efo + 3 * efe + iq * (long long)n + (i - 1)] += fyn;
        }
      }
    }
  }
}

template <typename T>
int launch_damp(const AdvArgs<T>& a, bool flux_mode, cudaStream_t s) {
  if (a.nord < 0 || a.nord > 2)
    return set_error(FV3G_E_UNSUPPORTED, "tracer damping supports nord 0..2 with a 3-cell halo (got %d)", a.nord);
  if (!a.del6_u || !a.del6_v) return set_error(FV3G_E_ARG, "tracer damping needs the del6_u and del6_v metrics");
  if (a.damp_mass && !a.dp1) return set_error(FV3G_E_ARG, "mass-weighted damping needs dp1");
  if (flux_mode && (!a.fx_out || !a.fy_out)) return set_error(FV3G_E_ARG, "flux-mode damping needs flux planes");
  if (!flux_mode && (!a.q_out || !a.dp2)) return set_error(FV3G_E_ARG, "damping of q needs q_out and dp2");
  const int nbx = (a.ie - a.is + TW) / TW, nby = (a.je - a.js + TW) / TW;
  const dim3 grid((unsigned)(nbx * nby), (unsigned)a.npz, (unsigned)adv_tiles(a));
  constexpr size_t smem = sizeof(SmemDamp<T>);
  switch (a.nord * 2 + (flux_mode ? 1 : 0)) {
    case 0: k_damp<T, 0, false><<<grid, 256, smem, s>>>(a, nbx); break;
    case 1: k_damp<T, 0, true><<<grid, 256, smem, s>>>(a, nbx); break;
    case 2: k_damp<T, 1, false><<<grid, 256, smem, s>>>(a, nbx); break;
    case 3: k_damp<T, 1, true><<<grid, 256, smem, s>>>(a, nbx); break;
    case 4: k_damp<T, 2, false><<<grid, 256, smem, s>>>(a, nbx); break;
    default: k_damp<T, 2, true><<<grid, 256, smem, s>>>(a, nbx); break;
  }
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

// Tangent-linear damping fluxes (value/tangent pairs, flux mode) for the
// tangent-linear and adjoint fv_tp_2d: del-2 only, whose stencil (the two
// cells beside a face, no corner fill) lies inside the advection's.
int launch_damp_tl(const AdvArgs<Dual<double>>& a, cudaStream_t s) {
  if (a.nord != 0)
    return set_error(FV3G_E_UNSUPPORTED, "the tangent-linear / adjoint fv_tp_2d damps with nord 0 only (got %d)",
                     a.nord);
  constexpr size_t smem = sizeof(SmemDamp<Dual<double>>);
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    err = cudaFuncSetAttribute(k_damp<Dual<double>, 0, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)smem);
  });
  if (err != cudaSuccess) return cuda_error(err, "cudaFuncSetAttribute(k_damp)");
  if (!a.del6_u || !a.del6_v || !a.fx_out || !a.fy_out || (a.damp_mass && !a.dp1))
    return set_error(FV3G_E_ARG, "tangent-linear damping needs del6_u, del6_v, flux planes and the mass");
  const int nbx = (a.ie - a.is + TW) / TW, nby = (a.je - a.js + TW) / TW;
  const dim3 grid((unsigned)(nbx * nby), (unsigned)a.npz, 1u);
  k_damp<Dual<double>, 0, true><<<grid, 256, smem, s>>>(a, nbx);
  FV3G_CUDA(cudaGetLastError());
  return 0;
}

double damp_coefficient(double damp_c, double da_min, int nord) {
  const double b = damp_c * da_min;
  double r = b;
  for (int o = 0; o < nord; ++o) r *= b;
  return r;
}

template int launch_damp<float>(const AdvArgs<float>&, bool, cudaStream_t);
template int launch_damp<double>(const AdvArgs<double>&, bool, cudaStream_t);

}  // namespace fv3g
