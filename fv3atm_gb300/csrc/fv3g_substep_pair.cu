// fv3g_substep_pair.cu -- the advection substep of FP32 states with hord 8,
// two tracers per warp.
//
// The same fused fv_tp_2d + flux-form update as k_substep (fv3g_substep.cuh:
// the three on-chip stages S1-S3 over a 32 x 32 window of a 26 x 26 CTA tile,
// the Lin 2004 monotonicity constraint, one-sided values at cube-face edges,
// copy_corners rotations), restated for a pair of tracers of the same cell:
// each lane holds the values of both tracers in a packed pair, so the adds,
// subtracts, multiplies and fused multiply-adds of the line march run as one
// f32x2 instruction for both, and the per-face and per-cell fields of the
// level (Courant numbers, area fluxes, mass fluxes, ratios) are read once for
// both.  Min, max and sign tests stay per value.  The slope's sign is taken
// once per cell as +-1 and reused by the two edge deviations one step later
// (a multiply in place of two sign transfers).
//
// Shared memory per warp doubles (the window and q_i hold pairs), so a CTA
// holds up to 12 warps (24 tracers) beside one copy of the level fields.
#include <mutex>

#include "fv3g_pair.cuh"
#include "fv3g_substep.cuh"

namespace fv3g {

struct SmemWarpPair {
  F2 q[WIN][PQ];   // tracer pair window; S2 overwrites each row with q_j (interior columns)
  F2 qi[TW][PQ];   // q_i; then q dp1/rarea + x-flux divergence
};

// Per-warp shared memory; edge CTAs add the edge deviations of two lines of
// pairs, [2][slots][32] (8 or 16 slots as the scalar kernel).
__host__ __device__ constexpr size_t pair_warp_bytes(bool edges, bool two_edges) {
  return sizeof(SmemWarpPair) + (edges ? 2 * (two_edges ? 16 : 8) * 32 * sizeof(F2) : 0);
}
size_t pair_smem_bytes(int warps, bool edges, bool two_edges) {
  return sizeof(SmemLevel<float>) + warps * pair_warp_bytes(edges, two_edges);
}
constexpr int PAIR_MAX_WARPS = 12;       // interior CTAs: 24 tracers, 221 KB
constexpr int PAIR_RING_MAX_WARPS = 8;   // edge-ring CTAs: 8 warps of 16 slots, 226 KB

// edge deviations of both tracers of a line (one scalar pass per tracer)
template <class EX, class ED>
__device__ __forceinline__ void edge_devs_pair(int e, bool east, EX x, ED ed, F2* o) {
  if (e == NO_EDGE) return;
  edge_devs<float, 8, 64>(e, east, [&x](int m) { return x(m).x; }, ed, &o->x);
  edge_devs<float, 8, 64>(e, east, [&x](int m) { return x(m).y; }, ed, &o->y);
}

// One pair of tracers (ia, ib) of one CTA tile through the three stages.
// ib == ia when the tracer count is odd and this is the last pair: the second
// value is then computed and not stored.
template <bool EDGES>
__device__ __forceinline__ void advance_pair(const AdvArgs<float>& a, SmemLevel<float>& L, SmemWarpPair& S,
                                             F2* eds, int ia, int ib, const TileCtx& tc, int lane, long long efo,
                                             long long efe, int nslot) {
  const PlaneGeom& pg = a.pg;
  const int n = a.npx - 1;
  const int t = tc.t, k = tc.k, i0 = tc.i0, j0 = tc.j0, ni = tc.ni, nj = tc.nj;
  const int exA = tc.exA, exB = tc.exB, eyA = tc.eyA, eyB = tc.eyB;
  const bool second = ib != ia;
  auto corner_cells = [&](int dir) {
    const int i = i0 - 3 + lane;
#pragma unroll 1
    for (int r = 0; r < WIN; ++r) {
      const int j = j0 - 3 + r;
      const bool oi = (i < 1) || (i > a.npx - 1), oj = (j < 1) || (j > a.npy - 1);
      if (oi && oj) S.q[r][lane] = F2{load_q(a, t, ia, k, i, j, dir), load_q(a, t, ib, k, i, j, dir)};
    }
  };
  {
    const int ic = min(max(i0 - 3 + lane, pg.isd), pg.isd + pg.pitch - 1);
    const float* sa = a.q_in + t * a.sQt + ia * a.sQq + k * a.sQk + (ic - pg.isd);
    const float* sb = a.q_in + t * a.sQt + ib * a.sQq + k * a.sQk + (ic - pg.isd);
    const int jhi = pg.jsd + pg.rows - 1;
#pragma unroll 8
    for (int r = 0; r < WIN; ++r) {
      const long long o = (long long)(min(max(j0 - 3 + r, pg.jsd), jhi) - pg.jsd) * pg.pitch;
      S.q[r][lane] = F2{sa[o], sb[o]};
    }
  }
  if (tc.corner_block) corner_cells(2);
  __syncwarp();

  F2 fyr[NF];  // inner y flux of this lane's column at faces 3..29 (S1 -> S3)
  const int sbk = nslot - 8;
  const EdgeSel esx = edge_sel(exA, exB, sbk), esy = edge_sel(eyA, eyB, sbk);
  F2* const ed0 = eds + lane;
  F2* const ed1 = eds + nslot * 32 + lane;
  // ------------------------------------------------ S1: inner y, q_i ------
  {
    const int w = lane;
    const F2* qcol = &S.q[0][w];
    if (EDGES) {
      auto ex = [qcol](int m) { return qcol[m * PQ]; };
      auto edA = [&L, w, eyA](int m) { return L.edy[0][m - eyA + 2][w]; };
      auto edB = [&L, w, eyB](int m) { return L.edy[1][m - eyB + 2][w]; };
      edge_devs_pair(eyA, false, ex, edA, ed0);
      edge_devs_pair(eyB, true, ex, edB, ed0 + sbk * 32);
    }
    PairLine ln;
    ln.init();
#pragma unroll
    for (int m = 0; m < 5; ++m) ln.step<EDGES>(m, qcol[m * PQ], 0.f, ed0, esy);
    fyr[0] = ln.step<EDGES>(5, qcol[5 * PQ], L.cy[0][w], ed0, esy);
    F2 fyy_prev = mul2(bc(L.yf[0][w]), fyr[0]);
#pragma unroll
    for (int m = 6; m < WIN; ++m) {
      const int f = m - 2;
      const F2 xrow = ln.xa;  // cell row f-1 = m-3
      fyr[f - 3] = ln.step<EDGES>(m, qcol[m * PQ], L.cy[f - 3][w], ed0, esy);
      const F2 fyy = mul2(bc(L.yf[f - 3][w]), fyr[f - 3]);
      S.qi[f - 4][w] = mul2(sub2(fma2(xrow, bc(L.area[f - 1][w]), fyy_prev), fyy), bc(L.rry[f - 4][w]));
      fyy_prev = fyy;
    }
  }
  __syncwarp();
  if (tc.corner_block) {  // corner blocks for the x sweeps
    corner_cells(1);
    __syncwarp();
  }

  // ---------- S2: inner x -> q_j (into the q row); outer x on q_i -> P -----
  {
    const int r = lane;
    const bool outer = (r >= 3) && (r < 29);
    const int ro = outer ? r - 3 : 0;
    F2* qrow = &S.q[r][0];
    F2* qirow = &S.qi[ro][0];
    if (EDGES) {
      auto exi = [qrow](int m) { return qrow[m]; };
      auto exo = [qirow](int m) { return qirow[m]; };
      auto edA = [&L, r, exA](int m) { return L.edx[0][m - exA + 2][r]; };
      auto edB = [&L, r, exB](int m) { return L.edx[1][m - exB + 2][r]; };
      edge_devs_pair(exA, false, exi, edA, ed0);
      edge_devs_pair(exB, true, exi, edB, ed0 + sbk * 32);
      if (outer) {
        edge_devs_pair(exA, false, exo, edA, ed1);
        edge_devs_pair(exB, true, exo, edB, ed1 + sbk * 32);
      }
    }
    const bool efw = EDGES && a.cube && a.eflux != nullptr && outer && ro < nj;
    auto put_ef = [&](long long o, F2 v) {
      a.eflux[o + ia * (long long)n] = v.x;
      if (second) a.eflux[o + ib * (long long)n] = v.y;
    };
    PairLine li, lo;
    li.init();
    lo.init();
#pragma unroll
    for (int m = 0; m < 5; ++m) {
      li.step<EDGES>(m, qrow[m], 0.f, ed0, esx);
      lo.step<EDGES>(m, qirow[m], 0.f, ed1, esx);
    }
    float c = L.cx[r][0];
    F2 fx2 = li.step<EDGES>(5, qrow[5], c, ed0, esx);
    F2 fo = lo.step<EDGES>(5, qirow[5], c, ed1, esx);
    F2 fxx_prev = mul2(bc(L.xf[r][0]), fx2);
    F2 F_prev = mul2(add2(fo, fx2), bc(L.mx[ro][0]));
    if (efw && i0 == 1) put_ef(efo + (j0 + ro - 1), neg2(F_prev));
#pragma unroll 2
    for (int m = 6; m < WIN; ++m) {
      const int f = m - 2;
      const F2 xcol = li.xa;  // q at window column f-1 of this row
      c = L.cx[r][f - 3];
      fx2 = li.step<EDGES>(m, qrow[m], c, ed0, esx);
      fo = lo.step<EDGES>(m, qirow[m], c, ed1, esx);
      const F2 fxx = mul2(bc(L.xf[r][f - 3]), fx2);
      // q_j of window column f-1 (interior column f-4); column m-6 of this row is consumed
      qrow[f - 4] = mul2(sub2(fma2(xcol, bc(L.area[r][f - 1]), fxx_prev), fxx), bc(L.rrx[r][f - 4]));
      fxx_prev = fxx;
      const F2 F = mul2(add2(fo, fx2), bc(L.mx[ro][f - 3]));
      if (outer) qirow[f - 4] = fma2(xcol, bc(L.dpa[ro][f - 4]), sub2(F_prev, F));  // q dp1/rarea + x divergence
      if (efw && i0 + f - 3 == a.npx) put_ef(efo + efe + (j0 + ro - 1), F);
      F_prev = F;
    }
  }
  __syncwarp();

  // ---------------------------- S3: outer y on q_j, update / write -------
  if (lane >= 3 && lane < 3 + TW) {
    const int c = lane - 3;  // interior column
    const F2* qjcol = &S.q[0][c];
    if (EDGES) {
      auto ex = [qjcol](int m) { return qjcol[m * PQ]; };
      auto edA = [&L, c, eyA](int m) { return L.edy[0][m - eyA + 2][c + 3]; };
      auto edB = [&L, c, eyB](int m) { return L.edy[1][m - eyB + 2][c + 3]; };
      edge_devs_pair(eyA, false, ex, edA, ed0);
      edge_devs_pair(eyB, true, ex, edB, ed0 + sbk * 32);
    }
    const int ig = i0 + c;
    const bool valid_c = c < ni;
    const bool efw = EDGES && a.cube && a.eflux != nullptr && valid_c;
    auto put_ef = [&](long long o, F2 v) {
      a.eflux[o + ia * (long long)n] = v.x;
      if (second) a.eflux[o + ib * (long long)n] = v.y;
    };
    float* qa = a.q_out + t * a.sQt + ia * a.sQq + k * a.sQk + pg.at(ig, j0);
    float* qb = a.q_out + t * a.sQt + ib * a.sQq + k * a.sQk + pg.at(ig, j0);
    PairLine ln;
    ln.init();
#pragma unroll
    for (int m = 0; m < 5; ++m) ln.step<EDGES>(m, qjcol[m * PQ], 0.f, ed0, esy);
    F2 Fprev = mul2(add2(ln.step<EDGES>(5, qjcol[5 * PQ], L.cy[0][c + 3], ed0, esy), fyr[0]), bc(L.my[0][c]));
    if (efw && j0 == 1) put_ef(efo + 2 * efe + (ig - 1), neg2(Fprev));
#pragma unroll
    for (int m = 6; m < WIN; ++m) {
      const int f = m - 2;
      const F2 F =
          mul2(add2(ln.step<EDGES>(m, qjcol[m * PQ], L.cy[f - 3][c + 3], ed0, esy), fyr[f - 3]), bc(L.my[f - 3][c]));
      const int ir = f - 4;  // interior row between faces f-1 and f
      if (ir < nj && valid_c) {
        const F2 v = mul2(sub2(add2(S.qi[ir][c], Fprev), F), bc(L.ub[ir][c]));
        qa[(long long)ir * pg.pitch] = v.x;
        if (second) qb[(long long)ir * pg.pitch] = v.y;
      }
      if (efw && j0 + f - 3 == a.npy) put_ef(efo + 3 * efe + (ig - 1), F);
      Fprev = F;
    }
  }
  __syncwarp();
}

template <bool EDGES>
__global__ void __launch_bounds__(32 * PAIR_MAX_WARPS) k_substep_pair(const AdvArgs<float> a, const BlockMap bm) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  SmemLevel<float>& L = *reinterpret_cast<SmemLevel<float>*>(smem_raw);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, W = blockDim.x >> 5;
  const bool two = EDGES && windows_hold_two_edges(a.is, a.ie, a.js, a.je);
  unsigned char* wbase = smem_raw + sizeof(SmemLevel<float>) + warp * pair_warp_bytes(EDGES, two);
  SmemWarpPair& S = *reinterpret_cast<SmemWarpPair*>(wbase);
  F2* eds = reinterpret_cast<F2*>(wbase + sizeof(SmemWarpPair));
  const TileCtx tc = tile_of<float, EDGES>(a, bm);
  stage_level<float, EDGES>(a, L, tc);
  const int n = a.npx - 1;
  // edge-flux index (((t*4 + e)*npz + k)*nq + iq)*n + s = efo + e*efe + iq*n + s
  const long long efe = (long long)a.npz * a.nq * n;
  const long long efo = (((long long)tc.t * 4) * a.npz + tc.k) * a.nq * n;
  const int npairs = (a.nq + 1) / 2;
  for (int p = warp; p < npairs; p += W)
    advance_pair<EDGES>(a, L, S, eds, 2 * p, min(2 * p + 1, a.nq - 1), tc, lane, efo, efe, two ? 16 : 8);
}

int prepare_substep_pair() {
  static std::once_flag once;
  static cudaError_t err = cudaSuccess;
  std::call_once(once, [] {
    cudaError_t e0 = cudaFuncSetAttribute(k_substep_pair<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)pair_smem_bytes(PAIR_MAX_WARPS, false, false));
    cudaError_t e1 = cudaFuncSetAttribute(k_substep_pair<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)pair_smem_bytes(PAIR_RING_MAX_WARPS, true, true));
    err = e0 != cudaSuccess ? e0 : e1;
  });
  return err == cudaSuccess ? 0 : cuda_error(err, "cudaFuncSetAttribute(k_substep_pair)");
}

// One substep of an FP32 hord-8 state with the tracers in pairs: the interior
// CTAs and the edge-ring CTAs, `warps` (interior) and a.warps_ring (ring, 0:
// as the interior, capped at PAIR_RING_MAX_WARPS) pairs wide, no wider than
// the pairs there are.
int launch_substep_pair(const AdvArgs<float>& a, int warps, cudaStream_t s) {
  {
    const int prc = prepare_substep_pair();
    if (prc) return prc;
  }
  const int npairs = (a.nq + 1) / 2;
  if (warps < 1 || warps > PAIR_MAX_WARPS || a.warps_ring < 0 || a.warps_ring > PAIR_RING_MAX_WARPS)
    return set_error(FV3G_E_ARG, "paired advection supports 1..%d warps per CTA and 1..%d per edge-ring CTA (got %d, %d)",
                     PAIR_MAX_WARPS, PAIR_RING_MAX_WARPS, warps, a.warps_ring);
  if (a.q_in_x != nullptr || a.fx_out != nullptr) return set_error(FV3G_E_ARG, "paired advection has no flux mode");
  const int w = std::min(warps, npairs);
  const int wr = std::min(std::min(a.warps_ring > 0 ? a.warps_ring : warps, PAIR_RING_MAX_WARPS), npairs);
  const BlockMap bm = block_map(a.is, a.ie, a.js, a.je, a.npx, a.npy, a.nested);
  const int nint = bm.nbxi * bm.nbyi, nring = bm.nbx * bm.nby - nint;
  const int nt = adv_tiles(a);
  const bool two = windows_hold_two_edges(a.is, a.ie, a.js, a.je);
  if (nint > 0) {
    k_substep_pair<false><<<dim3(nint, a.npz, nt), 32 * w, pair_smem_bytes(w, false, false), s>>>(a, bm);
    FV3G_CUDA(cudaGetLastError());
  }
  if (nring > 0) {
    k_substep_pair<true><<<dim3(nring, a.npz, nt), 32 * wr, pair_smem_bytes(wr, true, two), s>>>(a, bm);
    FV3G_CUDA(cudaGetLastError());
  }
  return 0;
}

}  // namespace fv3g
