// fv3g_stencil.cuh -- halo and corner sources shared by the stencil kernels
// (advection substep, tracer damping): the copy_corners rotation of a
// cube-corner halo cell, the neighbouring-tile cell behind an edge-halo cell,
// and clamped loads of plane fields.
#pragma once

#include "fv3g_internal.cuh"

namespace fv3g {

// ----------------------------------------------------------- halo source ---
// Rotate a cube-corner halo cell (tile indices) into the halo strip that a
// sweep in direction dir (1 = x, 2 = y) continues: about the corner point,
// +90 deg maps (u,v) -> (-v,u) and -90 deg maps (u,v) -> (v,-u).
__device__ __forceinline__ void corner_rotate(int& i, int& j, int npx, int npy, int dir) {
  const int su = (i < 1) ? -1 : 1, sv = (j < 1) ? -1 : 1;
  const int cx2 = (su < 0) ? 1 : 2 * npx - 1;  // doubled corner coordinates
  const int cy2 = (sv < 0) ? 1 : 2 * npy - 1;
  const int U = 2 * i - cx2, V = 2 * j - cy2;
  const bool plus = (dir == 1) ? (su == -sv) : (su == sv);
  const int U2 = plus ? -V : V, V2 = plus ? U : -U;
  i = (U2 + cx2) / 2;
  j = (V2 + cy2) / 2;
}

// Interior cell of the neighbouring tile that tile t's edge-halo cell (i, j) is.
__device__ __forceinline__ void cube_source(const Topo& tp, int n, int& t, int& i, int& j) {
  int e, d, s;
  if (i < 1) { e = EW; d = 1 - i; s = j - 1; }
  else if (i > n) { e = EE; d = i - n; s = j - 1; }
  else if (j < 1) { e = ES; d = 1 - j; s = i - 1; }
  else { e = EN; d = j - n; s = i - 1; }
  const int nt = tp.nbr[t][e], ne = tp.nedge[t][e];
  const int sb = tp.rev[t][e] ? n - 1 - s : s;
  switch (ne) {
    case EW: i = d; j = sb + 1; break;
    case EE: i = n + 1 - d; j = sb + 1; break;
    case ES: i = sb + 1; j = d; break;
    default: i = sb + 1; j = n + 1 - d; break;
  }
  t = nt;
}

template <typename T>
__device__ __forceinline__ T load_q(const AdvArgs<T>& a, int t, int iq, int k, int i, int j, int dir) {
  const int n = a.npx - 1;
  const bool out_i = (i < 1) || (i > a.npx - 1), out_j = (j < 1) || (j > a.npy - 1);
  if (out_i && out_j && !a.nested) {
    const int bit = (i < 1 ? 0 : 1) + (j < 1 ? 0 : 2);
    if (a.corners & (1 << bit)) corner_rotate(i, j, a.npx, a.npy, dir);
  }
  if (a.cube && (i < 1 || i > n || j < 1 || j > n) && !(((i < 1) || (i > n)) && ((j < 1) || (j > n))))
    cube_source(a.topo, n, t, i, j);
  // stay inside the data domain; clamped cells feed only discarded outputs
  i = min(max(i, a.pg.isd), a.pg.isd + a.pg.pitch - 1);
  j = min(max(j, a.pg.jsd), a.pg.jsd + a.pg.rows - 1);
  return a.q_in[t * a.sQt + iq * a.sQq + k * a.sQk + a.pg.at(i, j)];
}

template <typename T>
__device__ __forceinline__ T ld_field(const T* base, const PlaneGeom& pg, int i, int j) {
  i = min(max(i, pg.isd), pg.isd + pg.pitch - 1);
  j = min(max(j, pg.jsd), pg.jsd + pg.rows - 1);
  return base[pg.at(i, j)];
}

}  // namespace fv3g
