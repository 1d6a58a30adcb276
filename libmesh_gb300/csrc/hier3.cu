// Cubic HIERARCHIC hexahedra (FEType{THIRD, HIERARCHIC} on HEX27): element
// matrices of the Poisson form on the general path.
//
//   element loop, FEBase::reinit, weak form    introduction_ex4.C:440-540
//   compute_affine_map                          src/fe/fe_map.C:1167-1245
//   fe_hierarchic_3D_shape / cube_indices        src/fe/fe_hierarchic_shape_3D.C:166-760, 2249-2290
//
// Each element's 64 shapes are variants of the tensor hierarchic basis (which
// reference coordinate feeds each 1-D factor and with which sign follows from
// the element's edge and face orientation).  The host tabulates the affine
// reference tensors per orientation pattern (the element's 64 variants) in
// the element's own shape order, D_k[i][j], and the load table M[i][g]
// (shape x HEX27 map basis), and groups the elements by pattern into batches
// of at most eight.  Per batch one CTA forms, for its elements,
//   K_ij = sum_k A_k D_k[i][j],  A = coef detJ (G G^T) (6 entries),
//   F_i  = detJ sum_g M[i][g] f_g,
// reading every table entry once for the whole batch, and writes the full
// 64 x 64 matrices into the general path's element buffer.  The map is formed
// in FP64 in the reference's node order.  For the FP64 drop-in the contraction
// runs in double-float arithmetic on the FP32 pipe (the tables are stored as
// hi + lo pairs; GB300's FP64 rate is 1/64 of FP32) and each entry is rounded
// to FP64; the mixed form contracts in FP32.  Without
// constraint rows the homogeneous Dirichlet rows are applied here (zero row
// and column, 1 on the diagonal, zero load: constrain_element_matrix_and_vector
// with empty rows) and the constraint kernel is skipped; with rows the
// constraint kernel applies C^T K C.  The gather sums the entries in FP64.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "context_internal.cuh"
#include "df.cuh"
#include "general.cuh"

namespace lmg {

namespace {

constexpr int H3T = 256;

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

// N dofs and G map nodes per element (cubic hexes 64 / 27, cubic tets 20 / 14,
// quadratic and cubic prisms 18 / 6 and 40 / 6).
// FP64 drop-in (MIXED false): the contraction in double-float, each entry
// rounded to FP64 once; mixed form: the contraction in FP32.  The map is FP64
// in both.
template <int N, int G, bool MIXED, int H3B>
__global__ void __launch_bounds__(H3T) k_elem_pattern(H3Args a) {
  static_assert(N <= 64 && G <= 32, "one mask word per element, one lane per map node");
  __shared__ double sA[H3B][8];   // A_0..A_5, detJ
  __shared__ DF sA2[H3B][6];
  __shared__ double sf[H3B][G];
  __shared__ double sX[H3B][3 * G];  // map node coordinates of each warp's element
  __shared__ double sJ[H3B][9];      // map derivatives J[m*3+d] = dx_d/dxi_m
  __shared__ uint64_t sm[H3B];
  __shared__ int32_t se[H3B];
  const int t = threadIdx.x, lane = t & 31;
  for (int64_t bi = blockIdx.x; bi < a.n_batch; bi += gridDim.x) {
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
}

}  // namespace

void hier3_free(lmg_ctx *c) {
  dfree(c->d_h3batch);
  dfree(c->d_h3order);
  dfree(c->d_h3D);
  dfree(c->d_h3Df);
  dfree(c->d_h3M);
  dfree(c->d_h3gd);
  c->h3_nbatch = 0;
}

// lmg_form_set for the per-pattern HIERARCHIC elements.
int pattern_fe_dofs(int elem_type, int fe_order) {
  if (fe_order == (3 | LMG_HIERARCHIC))
    return elem_type == LMG_HEX27 ? 64 : (elem_type == LMG_TET14 ? 20 : (elem_type == LMG_PRISM21 ? 40 : 0));
  if (fe_order == (2 | LMG_HIERARCHIC) && elem_type == LMG_PRISM18) return 18;
  return 0;
}

lmg_status hier3_form_set(lmg_ctx *c, int32_t form, int32_t q_order, const double *elem_coef,
                          const double *nodal_f) {
  if (form != LMG_POISSON || c->n_vars != 1 || c->nl > 64)
    return fail(c, LMG_ERR_UNSUPPORTED,
                "form_set: per-pattern HIERARCHIC elements are built for POISSON (HEX27 / TET14 / PRISM21 "
                "THIRD, PRISM18 SECOND)");
  if (!c->h_gen.empty())
    return fail(c, LMG_ERR_UNSUPPORTED, "form_set: per-pattern HIERARCHIC elements take affine elements only");
  Hier3Tables h;
  const int order = c->elem_type == LMG_PRISM18 ? 2 : 3;
  std::string err =
      c->elem_type == LMG_TET14
          ? build_tet3_tables(h, q_order, c->n_elem, c->h_xyz.data(), c->h_conn.data())
          : (c->elem_type == LMG_HEX27
                 ? build_hier3_tables(h, q_order, c->n_elem, c->h_xyz.data(), c->h_conn.data())
                 : build_prism_tables(h, order, q_order, c->n_elem, c->h_xyz.data(), c->h_conn.data(), c->npe));
  if (!err.empty()) return fail(c, LMG_ERR_UNSUPPORTED, "form_set: " + err);
  hier3_free(c);
  LMG_CUDA(c, dupload(c, c->d_h3order, h.order.data(), h.order.size()));
  c->h3_order = h.order;
  c->h3_pid.assign((size_t)c->n_elem, 0);
  for (size_t b = 0; b + 2 < h.batch.size(); b += 3)
    for (int32_t k = 0; k < h.batch[b + 2]; ++k) c->h3_pid[(size_t)(h.batch[b + 1] + k)] = h.batch[b];
  std::vector<float2> dp(h.Dp.size());
  std::vector<float> df(h.Dp.size());
  for (size_t i = 0; i < dp.size(); ++i) {
    const DF x = df_split(h.Dp[i]);
    dp[i] = make_float2(x.hi, x.lo);
    df[i] = x.hi;
  }
  LMG_CUDA(c, dupload(c, c->d_h3D, dp.data(), dp.size()));
  LMG_CUDA(c, dupload(c, c->d_h3Df, df.data(), df.size()));
  LMG_CUDA(c, dupload(c, c->d_h3M, h.Mp.data(), h.Mp.size()));
  LMG_CUDA(c, dupload(c, c->d_h3gd, h.gd0.data(), h.gd0.size()));
  c->h3_patterns = h.P;
  if (lmg_status st = hier3_set_tile(c, c->h3_tile)) return st;
  FETables t;
  t.elem_type = c->elem_type;
  t.fe_order = order;
  t.q_order = q_order;
  t.family = 1;
  t.n = h.N;
  t.q = h.q;
  t.n_geo = h.G;
  c->tab = t;
  c->form = form;
  c->fe_order = order;
  c->q_order = q_order;
  c->kappa = 0.0;
  c->n_modes = 0;
  if (!c->general) c->gen_plan = false;
  c->general = true;
  dfree(c->d_coef);
  dfree(c->d_f);
  dfree(c->d_f2);
  if (elem_coef) LMG_CUDA(c, dupload(c, c->d_coef, elem_coef, (size_t)c->n_elem));
  if (nodal_f) LMG_CUDA(c, dupload(c, c->d_f, nodal_f, (size_t)c->n_nodes));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_form = true;
  return LMG_OK;
}

bool hier3_masks(const lmg_ctx *c) { return c->hier3 && !c->has_rows; }

lmg_status hier3_set_tile(lmg_ctx *c, int tile) {
  if (tile != 4 && tile != 8 && tile != 16 && tile != 32) return fail(c, LMG_ERR_ARG, "pattern tile must be 4, 8, 16 or 32");
  std::vector<int32_t> batch;
  const int64_t n = (int64_t)c->h3_order.size();
  for (int64_t i = 0; i < n;) {
    const int32_t p = c->h3_pid[(size_t)i];
    int64_t j = i;
    while (j < n && j - i < tile && c->h3_pid[(size_t)j] == p) ++j;
    batch.push_back(p);
    batch.push_back((int32_t)i);
    batch.push_back((int32_t)(j - i));
    i = j;
  }
  LMG_CUDA(c, dupload(c, c->d_h3batch, batch.data(), batch.size()));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  c->h3_nbatch = (int64_t)batch.size() / 3;
  c->h3_tile = tile;
  return LMG_OK;
}

namespace {
template <int B>
void launch_tiles(lmg_ctx *c, bool mixed, const H3Args &a, int grid) {
  if (c->tab.n == 20) {
    if (mixed) k_elem_pattern<20, 14, true, B><<<grid, H3T, 0, c->stream>>>(a);
    else k_elem_pattern<20, 14, false, B><<<grid, H3T, 0, c->stream>>>(a);
  } else if (c->tab.n == 18) {
    if (mixed) k_elem_pattern<18, 6, true, B><<<grid, H3T, 0, c->stream>>>(a);
    else k_elem_pattern<18, 6, false, B><<<grid, H3T, 0, c->stream>>>(a);
  } else if (c->tab.n == 40) {
    if (mixed) k_elem_pattern<40, 6, true, B><<<grid, H3T, 0, c->stream>>>(a);
    else k_elem_pattern<40, 6, false, B><<<grid, H3T, 0, c->stream>>>(a);
  } else {
    if (mixed) k_elem_pattern<64, 27, true, B><<<grid, H3T, 0, c->stream>>>(a);
    else k_elem_pattern<64, 27, false, B><<<grid, H3T, 0, c->stream>>>(a);
  }
}
}  // namespace

void launch_hier3(lmg_ctx *c, bool mixed) {
  H3Args a{};
  a.n_batch = c->h3_nbatch;
  a.batch = c->d_h3batch;
  a.order = c->d_h3order;
  a.xyz = c->d_xyz;
  a.conn = c->d_conn;
  a.npe = c->npe;
  a.coef = c->d_coef;
  a.nodal_f = c->d_f;
  a.cmask = hier3_masks(c) ? c->d_cmask : nullptr;
  a.D = c->d_h3D;
  a.Df = c->d_h3Df;
  a.M = c->d_h3M;
  a.gd0 = c->d_h3gd;
  a.Kraw = c->d_Ebuf;
  a.Fraw = c->d_Fbuf;
  a.status = c->d_status;
  a.bad_elem = c->d_bad;
  const int64_t want = (int64_t)c->n_sm * 8;
  const int grid = (int)(a.n_batch < want ? a.n_batch : want);
  if (grid <= 0) return;
  switch (c->h3_tile) {
    case 4: launch_tiles<4>(c, mixed, a, grid); break;
    case 16: launch_tiles<16>(c, mixed, a, grid); break;
    case 32: launch_tiles<32>(c, mixed, a, grid); break;
    default: launch_tiles<8>(c, mixed, a, grid); break;
  }
}

}  // namespace lmg
