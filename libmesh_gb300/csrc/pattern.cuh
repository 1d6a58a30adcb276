// Per-pattern HIERARCHIC element matrices: the arguments and the work of one
// CTA tile, shared by the per-system kernel (hier3.cu) and the persistent
// batch kernel (batch_persistent.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "df.cuh"
#include "../../include/libmesh_gb300.h"

namespace lmg {

constexpr int H3T = 256;  // threads of a tile CTA

struct H3Args {
  int64_t n_batch;
  const int32_t *batch;     // [n_batch][3]: pattern, first index in order, count
  const int32_t *order;     // element ids sorted by pattern
  const double *xyz;
  const int32_t *conn;      // [n_elem][npe], the G map nodes first
  int npe;
  const double *coef;       // [n_elem] or null
  const double *nodal_f;    // [n_nodes] or null
  const uint64_t *cmask;    // [n_elem] constrained local dofs, or null (no mask)
  const float2 *D;          // [P][6][N*N] double-float pairs
  const float *Df;          // [P][6][N*N] FP32 (mixed form)
  const double *M;          // [P][N][G]
  const double *gd0;        // [G][3]
  void *Kraw;               // [n_elem][N][N] element matrices: double (FP64 drop-in) or float (mixed)
  double *Fraw;             // [n_elem][N]
  int *status;
  unsigned long long *bad_elem;
};

// Shared memory of one tile of up to B elements with G map nodes.
template <int G, int B>
struct PatSmem {
  double sA[B][8];   // A_0..A_5, detJ
  DF sA2[B][6];
  double sf[B][G];
  double sX[B][3 * G];  // map node coordinates of each warp's element
  double sJ[B][9];      // map derivatives J[m*3+d] = dx_d/dxi_m
  uint64_t sm[B];
  int32_t se[B];
};

// N dofs and G map nodes per element (cubic hexes 64 / 27, cubic tets 20 / 14,
// quadratic and cubic prisms 18 / 6 and 40 / 6).
// FP64 drop-in (MIXED false): the contraction in double-float, each entry
// rounded to FP64 once; mixed form: the contraction in FP32.  The map is FP64
// in both.
// One tile bi (a batch of at most B elements of one pattern), all threads of
// the CTA (H3T) taking part.
template <int N, int G, bool MIXED, int B>
__device__ __forceinline__ void pattern_tile(const H3Args &a, int64_t bi, PatSmem<G, B> &S) {
  static_assert(N <= 64 && G <= 32, "one mask word per element, one lane per map node");
  auto &sA = S.sA;
  auto &sA2 = S.sA2;
  auto &sf = S.sf;
  auto &sX = S.sX;
  auto &sJ = S.sJ;
  auto &sm = S.sm;
  auto &se = S.se;
  const int t = threadIdx.x, lane = t & 31;
  constexpr int H3B = B;
  const int p = a.batch[3 * bi], first = a.batch[3 * bi + 1], cnt = a.batch[3 * bi + 2];
  __syncthreads();
  for (int w = t >> 5; w < cnt; w += H3T / 32) {  // warp: geometry of the tile's element w (compute_affine_map)
    const int32_t e = a.order[first + w];
    if (lane < G) {
      const int64_t nd = a.conn[(int64_t)e * a.npe + lane];
      sX[w][3 * lane] = a.xyz[3 * nd];
      sX[w][3 * lane + 1] = a.xyz[3 * nd + 1];
      sX[w][3 * lane + 2] = a.xyz[3 * nd + 2];
      sf[w][lane] = a.nodal_f ? a.nodal_f[nd] : 0.0;
    }
    __syncwarp();
    // J[m][d] = sum_g dphi_g/dxi_m x_g[d] in node order, every product and
    // sum rounded separately, as compute_affine_map forms it (fe_map.C:980-1044):
    // lane j < 9 forms entry j
    if (lane < 9) {
      const int m = lane / 3, d = lane - 3 * m;
      double acc = 0.0;
      for (int g = 0; g < G; ++g) acc = __dadd_rn(acc, __dmul_rn(a.gd0[3 * g + m], sX[w][3 * g + d]));
      sJ[w][lane] = acc;
    }
    __syncwarp();
    double jp[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) jp[k] = sJ[w][k];
    if (lane == 0) {
      // jp[3m+d] = dx_d/dxi_m; G[3m+d] = dxi_m/dx_d (fe_map.C:1046-1068)
      auto cof = [](double a, double b, double c, double d) { return __dsub_rn(__dmul_rn(a, b), __dmul_rn(c, d)); };
      const double c0 = cof(jp[4], jp[8], jp[5], jp[7]), c1 = cof(jp[5], jp[6], jp[3], jp[8]),
                   c2 = cof(jp[3], jp[7], jp[4], jp[6]);
      const double det = __dadd_rn(__dadd_rn(__dmul_rn(jp[0], c0), __dmul_rn(jp[1], c1)), __dmul_rn(jp[2], c2));
      const double inv = __ddiv_rn(1.0, det);
      double G[9];
      G[0] = __dmul_rn(c0, inv);
      G[1] = __dmul_rn(c1, inv);
      G[2] = __dmul_rn(c2, inv);
      G[3] = __dmul_rn(cof(jp[2], jp[7], jp[1], jp[8]), inv);
      G[4] = __dmul_rn(cof(jp[0], jp[8], jp[2], jp[6]), inv);
      G[5] = __dmul_rn(cof(jp[1], jp[6], jp[0], jp[7]), inv);
      G[6] = __dmul_rn(cof(jp[1], jp[5], jp[2], jp[4]), inv);
      G[7] = __dmul_rn(cof(jp[2], jp[3], jp[0], jp[5]), inv);
      G[8] = __dmul_rn(cof(jp[0], jp[4], jp[1], jp[3]), inv);
      if (!(det > 0.0)) {
        atomicCAS(a.status, 0, LMG_ERR_DEGENERATE);
        atomicMin(a.bad_elem, (unsigned long long)e);
      }
      const double kap = (a.coef ? a.coef[e] : 1.0) * det;
      sA[w][0] = kap * (G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
      sA[w][1] = kap * (G[3] * G[3] + G[4] * G[4] + G[5] * G[5]);
      sA[w][2] = kap * (G[6] * G[6] + G[7] * G[7] + G[8] * G[8]);
      sA[w][3] = kap * (G[0] * G[3] + G[1] * G[4] + G[2] * G[5]);
      sA[w][4] = kap * (G[0] * G[6] + G[1] * G[7] + G[2] * G[8]);
      sA[w][5] = kap * (G[3] * G[6] + G[4] * G[7] + G[5] * G[8]);
      sA[w][6] = det;
#pragma unroll
      for (int k = 0; k < 6; ++k) sA2[w][k] = df_split(sA[w][k]);
      sm[w] = a.cmask ? a.cmask[e] : 0ull;
      se[w] = e;
    }
  }
  __syncthreads();
  // K_ij = sum_k A_k D_k[i][j] in double-float arithmetic (FP32 pipe)
  const float2 *Dp = a.D + (size_t)p * 6 * (N * N);
  const float *Dfp = a.Df + (size_t)p * 6 * (N * N);
  for (int idx = t; idx < N * N; idx += H3T) {
    const int i = idx / N, j = idx - i * N;
    DF d[6];
#pragma unroll
    for (int k = 0; k < 6; ++k) {
      if constexpr (MIXED) {
        d[k] = DF{Dfp[k * (N * N) + idx], 0.f};
      } else {
        const float2 x = Dp[k * (N * N) + idx];
        d[k] = DF{x.x, x.y};
      }
    }
    for (int b = 0; b < cnt; ++b) {
      const bool msk = ((sm[b] >> i) | (sm[b] >> j)) & 1ull;
      if constexpr (MIXED) {
        float v = 0.f;
#pragma unroll
        for (int k = 0; k < 6; ++k) v = fmaf(sA2[b][k].hi, d[k].hi, v);
        if (msk) v = (i == j) ? 1.f : 0.f;
        static_cast<float *>(a.Kraw)[(int64_t)se[b] * (N * N) + idx] = v;
      } else {
        DF v = {0.f, 0.f};
#pragma unroll
        for (int k = 0; k < 6; ++k) v = df_fma_lazy(v, sA2[b][k], d[k]);
        v = df_norm(v);
        if (msk) v = DF{(i == j) ? 1.f : 0.f, 0.f};
        static_cast<double *>(a.Kraw)[(int64_t)se[b] * (N * N) + idx] = df_to_double(v);
      }
    }
  }
  const double *Mp = a.M + (size_t)p * N * G;
  for (int idx = t; idx < N * cnt; idx += H3T) {
    const int b = idx / N, i = idx - b * N;
    double s = 0.0;
    for (int g = 0; g < G; ++g) s += Mp[i * G + g] * sf[b][g];
    a.Fraw[(int64_t)se[b] * N + i] = ((sm[b] >> i) & 1ull) ? 0.0 : sA[b][6] * s;
  }
}

}  // namespace lmg
