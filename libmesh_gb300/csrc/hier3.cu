// Cubic HIERARCHIC hexahedra (FEType{THIRD, HIERARCHIC} on HEX27): element
// matrices of the Poisson form on the general path.
//
//   element loop, FEBase::reinit, weak form    introduction_ex4.C:440-540
//   compute_affine_map                          src/fe/fe_map.C:1167-1245
//   fe_hierarchic_3D_shape / cube_indices        src/fe/fe_hierarchic_shape_3D.C:166-760, 2249-2290
//
// Each element's 64 shapes are variants of the tensor hierarchic basis (which
// reference coordinate feeds each 1-D factor and with which sign follows from
// the element's edge and face orientation).  The host tabulates, over the
// variants that occur, D_k[v][w] (affine reference tensors) and M[v][g]
// (shape x HEX27 map basis); the kernel forms, per affine element,
//   K_ij = sum_k A_k D_k[var_i][var_j],  A = coef detJ (G G^T) (6 entries),
//   F_i  = detJ sum_g M[var_i][g] f_g,
// and writes the full 64 x 64 matrix into the general path's element buffer,
// where the constraint kernel and the slot gather take over.  One CTA per
// element at a time (grid-stride); 256 threads cover the 4096 entries with
// coalesced stores; the variant tables stay in L2.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "context_internal.cuh"
#include "general.cuh"

namespace lmg {

namespace {

constexpr int H3N = 64, H3T = 256;

struct H3Args {
  int64_t n_elem;
  const double *xyz;
  const int32_t *conn;      // [n_elem][27]
  const double *coef;       // [n_elem] or null
  const double *nodal_f;    // [n_nodes] or null
  const uint16_t *var;      // [n_elem][64]
  const double *D;          // [V][V][6]
  const double *M;          // [V][27]
  const double *gd0;        // [27][3]
  int V;
  double *Kraw;             // [n_elem][64][64]
  double *Fraw;             // [n_elem][64]
  int *status;
  unsigned long long *bad_elem;
};

__global__ void __launch_bounds__(H3T) k_elem_hier3(H3Args a) {
  __shared__ double sJ[27][9];
  __shared__ double sA[8];   // A_0..A_5, detJ
  __shared__ double sf[27];
  __shared__ uint16_t sv[H3N];
  const int t = threadIdx.x;
  for (int64_t e = blockIdx.x; e < a.n_elem; e += gridDim.x) {
    // compute_affine_map: J = sum_g X_g (x) dphi_g(qp 0), per-node partials reduced below
    if (t < 27) {
      const int64_t nd = a.conn[e * 27 + t];
      const double x[3] = {a.xyz[3 * nd], a.xyz[3 * nd + 1], a.xyz[3 * nd + 2]};
#pragma unroll
      for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int d = 0; d < 3; ++d) sJ[t][3 * m + d] = x[d] * a.gd0[3 * t + m];
      sf[t] = a.nodal_f ? a.nodal_f[nd] : 0.0;
    }
    if (t < H3N) sv[t] = a.var[e * H3N + t];
    __syncthreads();
    if (t == 0) {
      double jp[9];
#pragma unroll
      for (int k = 0; k < 9; ++k) {
        double s = 0.0;
        for (int g = 0; g < 27; ++g) s += sJ[g][k];
        jp[k] = s;
      }
      // jp[3m+d] = dx_d/dxi_m; G[3m+d] = dxi_m/dx_d (fe_map.C:1046-1068)
      const double c0 = jp[4] * jp[8] - jp[5] * jp[7], c1 = jp[5] * jp[6] - jp[3] * jp[8],
                   c2 = jp[3] * jp[7] - jp[4] * jp[6];
      const double det = jp[0] * c0 + jp[1] * c1 + jp[2] * c2;
      const double inv = 1.0 / det;
      double G[9];
      G[0] = c0 * inv;
      G[1] = c1 * inv;
      G[2] = c2 * inv;
      G[3] = (jp[2] * jp[7] - jp[1] * jp[8]) * inv;
      G[4] = (jp[0] * jp[8] - jp[2] * jp[6]) * inv;
      G[5] = (jp[1] * jp[6] - jp[0] * jp[7]) * inv;
      G[6] = (jp[1] * jp[5] - jp[2] * jp[4]) * inv;
      G[7] = (jp[2] * jp[3] - jp[0] * jp[5]) * inv;
      G[8] = (jp[0] * jp[4] - jp[1] * jp[3]) * inv;
      if (!(det > 0.0)) {
        atomicCAS(a.status, 0, LMG_ERR_DEGENERATE);
        atomicMin(a.bad_elem, (unsigned long long)e);
      }
      const double kap = (a.coef ? a.coef[e] : 1.0) * det;
      sA[0] = kap * (G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
      sA[1] = kap * (G[3] * G[3] + G[4] * G[4] + G[5] * G[5]);
      sA[2] = kap * (G[6] * G[6] + G[7] * G[7] + G[8] * G[8]);
      sA[3] = kap * (G[0] * G[3] + G[1] * G[4] + G[2] * G[5]);
      sA[4] = kap * (G[0] * G[6] + G[1] * G[7] + G[2] * G[8]);
      sA[5] = kap * (G[3] * G[6] + G[4] * G[7] + G[5] * G[8]);
      sA[6] = det;
    }
    __syncthreads();
    const double A0 = sA[0], A1 = sA[1], A2 = sA[2], A3 = sA[3], A4 = sA[4], A5 = sA[5];
    double *Ko = a.Kraw + e * (H3N * H3N);
    for (int idx = t; idx < H3N * H3N; idx += H3T) {
      const int i = idx >> 6, j = idx & 63;
      const double *d = a.D + ((size_t)sv[i] * a.V + sv[j]) * 6;
      Ko[idx] = A0 * d[0] + A1 * d[1] + A2 * d[2] + A3 * d[3] + A4 * d[4] + A5 * d[5];
    }
    if (t < H3N) {
      const double *mv = a.M + (size_t)sv[t] * 27;
      double s = 0.0;
      for (int g = 0; g < 27; ++g) s += mv[g] * sf[g];
      a.Fraw[e * H3N + t] = sA[6] * s;
    }
    __syncthreads();
  }
}

}  // namespace

void hier3_free(lmg_ctx *c) {
  dfree(c->d_h3var);
  dfree(c->d_h3D);
  dfree(c->d_h3M);
  dfree(c->d_h3gd);
  c->h3V = 0;
}

// lmg_form_set for FEType{THIRD, HIERARCHIC} on HEX27.
lmg_status hier3_form_set(lmg_ctx *c, int32_t form, int32_t q_order, const double *elem_coef,
                          const double *nodal_f) {
  if (form != LMG_POISSON || c->n_vars != 1 || c->elem_type != LMG_HEX27)
    return fail(c, LMG_ERR_UNSUPPORTED, "form_set: THIRD HIERARCHIC is built for POISSON on HEX27");
  if (!c->h_gen.empty())
    return fail(c, LMG_ERR_UNSUPPORTED, "form_set: THIRD HIERARCHIC takes affine elements only");
  Hier3Tables h;
  std::string err = build_hier3_tables(h, q_order, c->n_elem, c->h_xyz.data(), c->h_conn.data());
  if (!err.empty()) return fail(c, LMG_ERR_UNSUPPORTED, "form_set: " + err);
  hier3_free(c);
  LMG_CUDA(c, dupload(c, c->d_h3var, h.var.data(), h.var.size()));
  LMG_CUDA(c, dupload(c, c->d_h3D, h.D.data(), h.D.size()));
  LMG_CUDA(c, dupload(c, c->d_h3M, h.M.data(), h.M.size()));
  LMG_CUDA(c, dupload(c, c->d_h3gd, h.gd0.data(), h.gd0.size()));
  c->h3V = h.V;
  FETables t;
  t.elem_type = LMG_HEX27;
  t.fe_order = 3;
  t.q_order = q_order;
  t.family = 1;
  t.n = H3N;
  t.q = h.q;
  t.n_geo = 27;
  c->tab = t;
  c->form = form;
  c->fe_order = 3;
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

void launch_hier3(lmg_ctx *c) {
  H3Args a{};
  a.n_elem = c->n_elem;
  a.xyz = c->d_xyz;
  a.conn = c->d_conn;
  a.coef = c->d_coef;
  a.nodal_f = c->d_f;
  a.var = c->d_h3var;
  a.D = c->d_h3D;
  a.M = c->d_h3M;
  a.gd0 = c->d_h3gd;
  a.V = c->h3V;
  a.Kraw = c->d_Ebuf;
  a.Fraw = c->d_Fbuf;
  a.status = c->d_status;
  a.bad_elem = c->d_bad;
  const int64_t want = (int64_t)c->n_sm * 8;
  const int grid = (int)(c->n_elem < want ? c->n_elem : want);
  if (grid > 0) k_elem_hier3<<<grid, H3T, 0, c->stream>>>(a);
}

}  // namespace lmg
