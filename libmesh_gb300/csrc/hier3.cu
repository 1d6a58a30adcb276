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
#include "pattern.cuh"

namespace lmg {

namespace {

template <int N, int G, bool MIXED, int H3B>
__global__ void __launch_bounds__(H3T) k_elem_pattern(H3Args a) {
  __shared__ PatSmem<G, H3B> S;
  for (int64_t bi = blockIdx.x; bi < a.n_batch; bi += gridDim.x) pattern_tile<N, G, MIXED, H3B>(a, bi, S);
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

// The per-pattern tables of h on the device, the elements grouped into tiles.
lmg_status pattern_upload(lmg_ctx *c, const Hier3Tables &h) {
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
  return hier3_set_tile(c, c->h3_tile);
}

// A block-path Poisson system (one variable, affine elements, Dirichlet rows
// only) in per-pattern form for the persistent batch: one pattern, the
// symmetrised reference tensors of its FE tables, the load table M and the
// map derivatives at the first point (isoparametric: G = N nodes).
lmg_status pattern_from_block(lmg_ctx *c) {
  const FETables &t = c->tab;
  const int N = t.n;
  if (c->hier3) return LMG_OK;
  if (c->form != LMG_POISSON || c->n_vars != 1 || c->has_rows || !c->h_gen.empty() || t.n_geo != N ||
      N != c->npe || N > 32 || t.S.size() != (size_t)9 * N * N || t.M.size() != (size_t)N * N)
    return fail(c, LMG_ERR_UNSUPPORTED, "persistent batch: member is not an affine one-variable Poisson system");
  Hier3Tables h;
  h.N = N;
  h.G = N;
  h.q = t.q;
  h.P = 1;
  h.Dp.assign((size_t)6 * N * N, 0.0);
  const int pm[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
  auto S = [&](int m, int k, int a, int b) { return t.S[(((size_t)(3 * m + k) * N) + a) * N + b]; };
  for (int k = 0; k < 6; ++k)
    for (int a = 0; a < N; ++a)
      for (int b = 0; b < N; ++b) {
        const int m0 = pm[k][0], m1 = pm[k][1];
        h.Dp[((size_t)k * N + a) * N + b] = (m0 == m1) ? S(m0, m0, a, b) : S(m0, m1, a, b) + S(m1, m0, a, b);
      }
  h.Mp = t.M;
  h.gd0.assign(t.gdphi.begin(), t.gdphi.begin() + (size_t)N * 3);
  h.order.resize((size_t)c->n_elem);
  for (int64_t e = 0; e < c->n_elem; ++e) h.order[(size_t)e] = (int32_t)e;
  h.batch = {0, 0, (int32_t)c->n_elem};
  c->persist_pattern = true;
  return pattern_upload(c, h);
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
  if (lmg_status st = pattern_upload(c, h)) return st;
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
