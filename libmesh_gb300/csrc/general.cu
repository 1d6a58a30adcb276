// General scalar assembly path: full (nonsymmetric) element matrices, the
// constraint product C^T K C for elements that touch constrained dofs, and a
// deterministic gather into the CSR values.  Used for the convection-diffusion
// form and for systems with constraint rows (hanging nodes).
//
//   element loop, FEBase::reinit, weak form     adaptivity_ex2.C:580-690 (steady part),
//                                                introduction_ex4.C:440-540
//   DofMap::constrain_element_matrix_and_vector  src/base/dof_map_constraints.C:2439-2515
//   DofMap::build_constraint_matrix              src/base/dof_map_constraints.C:3433-3540
//   SparseMatrix::add_matrix / add_vector        src/numerics/petsc_matrix.C:735-755
//
// Element kernel: one warp per element, lane b computes column b of Ke, in
// double-float arithmetic on the FP32 pipe (geometry and transport velocity in
// FP64); element matrices are stored as double-float pairs.
// Affine hexahedra only: the diffusion block is the reference-tensor
// contraction K_ab = sum_k A_k D^k_ab (D = symmetrized sum_q w dphi_m dphi_n
// tables), the convection block C_ab = sum_q phi_a(q) sum_m beta_m(q) dphi_m,b(q)
// with beta_m(q) = w_q detJ (dxi_m/dx . b(x_q)), summed over q by sum
// factorization (phi_a(q) is a product of 1-D shapes on the tensor Gauss
// rule).
//
// Constraint kernel: one CTA per constrained element.  K' = C^T K C over the
// element's dofs followed by its constraining dofs (sorted), with C given by
// its columns (row index, coefficient) in ascending row order, evaluated in
// the reference's order: L_pj = sum_i C_ip K_ij, K'_pq = sum_j L_pj C_jq.
// Constrained rows become e_i^T with -c_ij at their constraining dofs; F' = C^T F.
#include <cuda_runtime.h>

#include "df.cuh"
#include "general.cuh"
#include "../../include/libmesh_gb300.h"

namespace lmg {

namespace {

constexpr int WARPS = 8;

// sin and cos of x, the series in double-float arithmetic (FP32 pipe).  Cody
// and Waite's reduction in FP64, x = k pi/2 + r, k = rint(x 2/pi),
// r = ((x - k P1) - k P2) - k P3 with pi/2 = P1 + P2 + P3 as doubles, each
// step one FMA (one rounding), so that r keeps the absolute accuracy of x;
// then r as a double-float pair and the Taylor series of sin and cos in r^2 on
// |r| <= pi/4 (9 and 10 terms: the first neglected term is below 2^-54 of the
// leading one) by Horner in double-float, and the quadrant's signs.  The
// coefficients (-1)^i / (2i+1)! and (-1)^i / (2i)! are stored as float pairs.
__device__ __forceinline__ void df_sincos(double xd, DF &s, DF &c) {
  constexpr float SIN[9][2] = {{1.0f, 0.f},
                               {-0.1666666716337204f, 4.967053879312289e-09f},
                               {0.008333333767950535f, -4.34617203337595e-10f},
                               {-0.00019841270113829523f, 2.725596874933456e-12f},
                               {2.7557318844628753e-06f, 3.793571224297229e-14f},
                               {-2.5052107943679403e-08f, -4.4176230446483665e-16f},
                               {1.6059044372074283e-10f, -5.352526511562726e-18f},
                               {-7.647163609812713e-13f, -1.2200710471178288e-20f},
                               {2.8114573589663704e-15f, -1.0462084739763658e-22f}};
  constexpr float COS[10][2] = {{1.0f, 0.f},
                                {-0.5f, 0.f},
                                {0.0416666679084301f, -1.2417634698280722e-09f},
                                {-0.0013888889225199819f, 3.3631094437103215e-11f},
                                {2.4801587642286904e-05f, -3.40699609366682e-13f},
                                {-2.755731998149713e-07f, 7.575112209051195e-15f},
                                {2.0876755879584152e-09f, 1.1082839147459852e-16f},
                                {-1.147074536050896e-11f, -2.372207689231238e-19f},
                                {4.7794772561329454e-14f, 7.62544404448643e-22f},
                                {-1.5619206814541513e-16f, -1.5404471465941993e-24f}};
  const double kd = rint(xd * 0.6366197723675814);
  const double rd = fma(-kd, -1.4973849048591698e-33, fma(-kd, 6.123233995736766e-17, fma(-kd, 1.5707963267948966, xd)));
  const DF r = df_split(rd);
  const float k = (float)kd;
  const DF r2 = df_mul(r, r);
  DF ps = DF{SIN[8][0], SIN[8][1]};
#pragma unroll
  for (int i = 7; i >= 0; --i) ps = df_add(df_mul(ps, r2), DF{SIN[i][0], SIN[i][1]});
  const DF sr = df_mul(ps, r);
  DF pc = DF{COS[9][0], COS[9][1]};
#pragma unroll
  for (int i = 8; i >= 0; --i) pc = df_add(df_mul(pc, r2), DF{COS[i][0], COS[i][1]});
  const DF nsr = DF{-sr.hi, -sr.lo}, npc = DF{-pc.hi, -pc.lo};
  switch (((int)k) & 3) {
    case 0: s = sr; c = pc; break;
    case 1: s = pc; c = nsr; break;
    case 2: s = nsr; c = npc; break;
    default: s = npc; c = sr; break;
  }
}

// Tensor indices of a hex node in the 1-D Lagrange bases (0 at -1, 1 at +1,
// 2 at 0), packed as i + 3 j + 9 k: HEX27 node order of cell_hex27.C, HEX8
// node order of cell_hex8.C.
__host__ __device__ constexpr int hex_tensor(int n, int a) {
  if (n == 8) {
    switch (a) {
      case 0: return 0;  case 1: return 1;  case 2: return 4;  case 3: return 3;
      case 4: return 9;  case 5: return 10; case 6: return 13; default: return 12;
    }
  }
  switch (a) {
    case 0: return 0;   case 1: return 1;   case 2: return 4;   case 3: return 3;   case 4: return 9;
    case 5: return 10;  case 6: return 13;  case 7: return 12;  case 8: return 2;   case 9: return 7;
    case 10: return 5;  case 11: return 6;  case 12: return 18; case 13: return 19; case 14: return 22;
    case 15: return 21; case 16: return 11; case 17: return 16; case 18: return 14; case 19: return 15;
    case 20: return 8;  case 21: return 20; case 22: return 25; case 23: return 23; case 24: return 24;
    case 25: return 17; default: return 26;
  }
}

// C_rb = sum_q phi_r(q) P(q) for the tensor-product element: phi_r(q) =
// L_i(x_q1) L_j(x_q2) L_k(x_q3), q = q1 + Q1 (q2 + Q1 q3); three 1-D passes,
// in double-float arithmetic (FP32 pipe), every inner sum renormalised once.
template <int N1, int Q1>
__device__ __forceinline__ void tensor_contract_df(const DF *L1, const DF *P, DF *Cc) {
  DF T1[N1 * Q1 * Q1];
#pragma unroll
  for (int i = 0; i < N1; ++i)
#pragma unroll
    for (int r = 0; r < Q1 * Q1; ++r) {
      DF t = {0.f, 0.f};
#pragma unroll
      for (int q1 = 0; q1 < Q1; ++q1) t = df_fma_lazy(t, L1[i * Q1 + q1], P[q1 + Q1 * r]);
      T1[i * Q1 * Q1 + r] = df_norm(t);
    }
  DF T2[N1 * N1 * Q1];
#pragma unroll
  for (int i = 0; i < N1; ++i)
#pragma unroll
    for (int j = 0; j < N1; ++j)
#pragma unroll
      for (int q3 = 0; q3 < Q1; ++q3) {
        DF t = {0.f, 0.f};
#pragma unroll
        for (int q2 = 0; q2 < Q1; ++q2) t = df_fma_lazy(t, L1[j * Q1 + q2], T1[i * Q1 * Q1 + q2 + Q1 * q3]);
        T2[(i * N1 + j) * Q1 + q3] = df_norm(t);
      }
#pragma unroll
  for (int i = 0; i < N1; ++i)
#pragma unroll
    for (int j = 0; j < N1; ++j)
#pragma unroll
      for (int k = 0; k < N1; ++k) {
        DF t = {0.f, 0.f};
#pragma unroll
        for (int q3 = 0; q3 < Q1; ++q3) t = df_fma_lazy(t, L1[k * Q1 + q3], T2[(i * N1 + j) * Q1 + q3]);
        Cc[i + 3 * j + 9 * k] = df_norm(t);
      }
}

inline __device__ DF ld_df(const float2 *p) {
  const float2 v = *p;
  return DF{v.x, v.y};
}

template <int FORM, int N, int Q>
__global__ void __launch_bounds__(WARPS * 32) k_elem_full(GenElemArgs a) {
  constexpr int N1 = (N == 8) ? 2 : 3, Q1 = (Q == 8) ? 2 : 3;
  extern __shared__ double sm[];
  float2 *sphi = reinterpret_cast<float2 *>(sm);                   // [Q][N] double-float
  float2 *sdphi = sphi + Q * N;                                     // [Q][N][3] double-float
  float2 *sD = sdphi + Q * N * 3;                                   // [6][N][N] double-float
  double *sqw = reinterpret_cast<double *>(sD + 6 * N * N);       // [Q]
  double *sgd = sqw + Q;              // [N][3] mapping derivatives at qp 0
  double *sgp = sgd + N * 3;          // [Q][N] mapping shapes (isoparametric geometry)
  double *smode = sgp + Q * N;        // [7 * n_modes]
  float2 *scurl = reinterpret_cast<float2 *>(smode + 7 * a.n_modes);  // [n_modes][3] k x a, double-float
  double *wbase = reinterpret_cast<double *>(scurl + 3 * a.n_modes);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *sX = wbase + warp * (N * 3 + N + 4 * Q + 8 * a.n_modes);  // [N][3]
  float2 *sf = reinterpret_cast<float2 *>(sX + N * 3);  // [N] nodal load, double-float
  float2 *sbeta = sf + N;                               // [Q][3] double-float
  float2 *sfq = sbeta + 3 * Q;                          // [Q] JxW f(x_q), double-float
  float2 *sE = sfq + Q;                                 // [n_modes][4] (cos, sin), double-float
  for (int i = threadIdx.x; i < Q * N; i += blockDim.x) {
    const DF x = df_split(a.fe.phi[i]);
    sphi[i] = make_float2(x.hi, x.lo);
  }
  for (int i = threadIdx.x; i < Q * N * 3; i += blockDim.x) {
    const DF x = df_split(a.fe.dphi[i]);
    sdphi[i] = make_float2(x.hi, x.lo);
  }
  for (int i = threadIdx.x; i < 6 * N * N; i += blockDim.x) {
    const DF x = df_split(a.D6[i]);
    sD[i] = make_float2(x.hi, x.lo);
  }
  for (int i = threadIdx.x; i < Q; i += blockDim.x) sqw[i] = a.fe.qw[i];
  for (int i = threadIdx.x; i < N * 3; i += blockDim.x) sgd[i] = a.fe.gdphi[i];
  for (int i = threadIdx.x; i < Q * N; i += blockDim.x) sgp[i] = a.fe.gphi[i];
  for (int i = threadIdx.x; i < 7 * a.n_modes; i += blockDim.x) smode[i] = a.modes[i];
  for (int i = threadIdx.x; i < 3 * a.n_modes; i += blockDim.x) {  // b = sum_m cos(.) k_m x a_m
    const double *md = a.modes + 7 * (i / 3);
    const int d = i % 3;
    const double v = d == 0 ? md[4] * md[2] - md[5] * md[1]
                     : d == 1 ? md[5] * md[0] - md[3] * md[2]
                              : md[3] * md[1] - md[4] * md[0];
    const DF x = df_split(v);
    scurl[i] = make_float2(x.hi, x.lo);
  }
  __shared__ DF sL1[9];
  __shared__ DF sJd[WARPS][9];  // map derivatives of each warp's element
  for (int i = threadIdx.x; i < N1 * Q1; i += blockDim.x) sL1[i] = df_split(a.D6[6 * N * N + i]);
  const double gp = a.D6[6 * N * N + N1 * Q1];  // outer 1-D Gauss point (+gp, -gp, and 0 when Q1 = 3)
  __syncthreads();
  const int64_t stride = (int64_t)gridDim.x * WARPS;
  for (int64_t e = (int64_t)blockIdx.x * WARPS + warp; e < a.n_elem; e += stride) {
    // geometry and nodal load of this element
    if (lane < N) {
      const int64_t nd = a.conn[e * N + lane];
      sX[3 * lane] = a.xyz[3 * nd];
      sX[3 * lane + 1] = a.xyz[3 * nd + 1];
      sX[3 * lane + 2] = a.xyz[3 * nd + 2];
      const DF fv = df_split(a.nodal_f ? a.nodal_f[nd] : 0.0);
      sf[lane] = make_float2(fv.hi, fv.lo);
    }
    __syncwarp();
    // The elements here are affine hexahedra (form_set refuses the others), so
    // the constant map derivatives are the edge vectors from vertex 0 to
    // vertices 1, 3 and 4 over the reference edge length 2: the value of
    // compute_affine_map's sum over the nodes, in 9 subtractions.  Lane j < 9
    // forms entry j in FP64 and splits it; the inverse map, detJ and the
    // diffusion tensor then run in double-float on the FP32 pipe.
    if (lane < 9) {
      const int m = lane / 3, d = lane - 3 * m, v = m == 0 ? 1 : (m == 1 ? 3 : 4);
      sJd[warp][lane] = df_split(0.5 * (sX[3 * v + d] - sX[d]));
    }
    __syncwarp();
    DF J[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) J[j] = sJd[warp][j];
    // J[m*3+d] = d x_d / d xi_m; G[3m+d] = d xi_m / d x_d (fe_map.C:1046-1068)
    const DF c0 = df_sub(df_mul(J[4], J[8]), df_mul(J[5], J[7]));
    const DF c1 = df_sub(df_mul(J[5], J[6]), df_mul(J[3], J[8]));
    const DF c2 = df_sub(df_mul(J[3], J[7]), df_mul(J[4], J[6]));
    const DF det = df_add(df_add(df_mul(J[0], c0), df_mul(J[1], c1)), df_mul(J[2], c2));
    const DF inv = df_recip(det);
    DF G[9];
    G[0] = df_mul(c0, inv);
    G[1] = df_mul(c1, inv);
    G[2] = df_mul(c2, inv);
    G[3] = df_mul(df_sub(df_mul(J[2], J[7]), df_mul(J[1], J[8])), inv);
    G[4] = df_mul(df_sub(df_mul(J[0], J[8]), df_mul(J[2], J[6])), inv);
    G[5] = df_mul(df_sub(df_mul(J[1], J[6]), df_mul(J[0], J[7])), inv);
    G[6] = df_mul(df_sub(df_mul(J[1], J[5]), df_mul(J[2], J[4])), inv);
    G[7] = df_mul(df_sub(df_mul(J[2], J[3]), df_mul(J[0], J[5])), inv);
    G[8] = df_mul(df_sub(df_mul(J[0], J[4]), df_mul(J[1], J[3])), inv);
    if (lane == 0 && !(det.hi > 0.f)) {
      atomicCAS(a.status, 0, LMG_ERR_DEGENERATE);
      atomicMin(a.bad_elem, (unsigned long long)e);
    }
    const double coef = a.coef ? a.coef[e] : 1.0;
    const DF kap = df_mul(df_split(FORM == LMG_ADVDIFF ? a.kappa * coef : coef), det);
    auto gg = [&](int m, int n) {
      return df_add(df_add(df_mul(G[3 * m], G[3 * n]), df_mul(G[3 * m + 1], G[3 * n + 1])),
                    df_mul(G[3 * m + 2], G[3 * n + 2]));
    };
    DF A2[6];
    A2[0] = df_mul(kap, gg(0, 0));
    A2[1] = df_mul(kap, gg(1, 1));
    A2[2] = df_mul(kap, gg(2, 2));
    A2[3] = df_mul(kap, gg(0, 1));
    A2[4] = df_mul(kap, gg(0, 2));
    A2[5] = df_mul(kap, gg(1, 2));
    __syncwarp();
    if (FORM == LMG_ADVDIFF) {
      // exp(i (k.x + phase)) at the element centre and exp(i gp k.dx/dxi_m):
      // the phase is affine in xi, so every Gauss point's value is a product
      // of these (angle addition) -- four sincos per mode, one per lane.
      const double xc[3] = {0.5 * (sX[0] + sX[18]), 0.5 * (sX[1] + sX[19]), 0.5 * (sX[2] + sX[20])};
      for (int t = lane; t < 4 * a.n_modes; t += 32) {
        const double *md = smode + 7 * (t >> 2);
        const int w = t & 3;
        double ang;
        if (w == 0) {
          ang = md[3] * xc[0] + md[4] * xc[1] + md[5] * xc[2] + md[6];
        } else {
          const int v = w == 1 ? 1 : (w == 2 ? 3 : 4);  // d x / d xi_{w-1}
          const double j0 = 0.5 * (sX[3 * v] - sX[0]), j1 = 0.5 * (sX[3 * v + 1] - sX[1]),
                       j2 = 0.5 * (sX[3 * v + 2] - sX[2]);
          ang = gp * (md[3] * j0 + md[4] * j1 + md[5] * j2);
        }
        DF s2, c2;
        df_sincos(ang, s2, c2);
        sE[2 * t] = make_float2(c2.hi, c2.lo);
        sE[2 * t + 1] = make_float2(s2.hi, s2.lo);
      }
      __syncwarp();
    }
    // per quadrature point: transport coefficients and the load, in
    // double-float arithmetic (FP32 pipe)
    if (lane < Q) {
      const int q = lane;
      DF fx = {0.f, 0.f};
      for (int c = 0; c < N; ++c) fx = df_fma_lazy(fx, ld_df(sphi + q * N + c), ld_df(sf + c));  // FE-interpolated load
      fx = df_norm(fx);
      const DF jw = df_mul(det, df_split(sqw[q]));
      const DF fq = df_mul(jw, fx);
      sfq[q] = make_float2(fq.hi, fq.lo);
      if (FORM == LMG_ADVDIFF) {
        DF b[3] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
        // offset of this point along each reference axis: -1, 0 or +1 times gp
        const int qi[3] = {q % Q1, (q / Q1) % Q1, q / (Q1 * Q1)};
        for (int m = 0; m < a.n_modes; ++m) {
          const float2 *E = sE + 8 * m;
          DF re = ld_df(E), im = ld_df(E + 1);
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            if (Q1 == 3 && qi[d] == 1) continue;
            const DF c = ld_df(E + 2 * (d + 1));
            DF sn = ld_df(E + 2 * (d + 1) + 1);
            if (qi[d] == 0) sn = DF{-sn.hi, -sn.lo};
            const DF nim = DF{-im.hi, -im.lo};
            const DF r2 = df_norm(df_fma_lazy(df_fma_lazy(DF{0.f, 0.f}, re, c), nim, sn));
            im = df_norm(df_fma_lazy(df_fma_lazy(DF{0.f, 0.f}, re, sn), im, c));
            re = r2;
          }
#pragma unroll
          for (int d = 0; d < 3; ++d) b[d] = df_fma_lazy(b[d], re, ld_df(scurl + 3 * m + d));
        }
#pragma unroll
        for (int d = 0; d < 3; ++d) b[d] = df_norm(b[d]);
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          DF t = {0.f, 0.f};
#pragma unroll
          for (int d = 0; d < 3; ++d) t = df_fma_lazy(t, G[3 * m + d], b[d]);
          t = df_mul(jw, df_norm(t));
          sbeta[3 * q + m] = make_float2(t.hi, t.lo);
        }
      }
    }
    __syncwarp();
    if (lane < N) {
      // column b of Ke in double-float arithmetic: convection by sum
      // factorisation, diffusion from the reference tensors
      const int b = lane;
      DF P[Q];
      if (FORM == LMG_ADVDIFF) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const float2 *d = sdphi + (q * N + b) * 3;
          DF t = {0.f, 0.f};
#pragma unroll
          for (int m = 0; m < 3; ++m) t = df_fma_lazy(t, ld_df(sbeta + 3 * q + m), ld_df(d + m));
          P[q] = df_norm(t);
        }
      }
      DF Cc[27];
      if (FORM == LMG_ADVDIFF) {
        DF L1[N1 * Q1];
#pragma unroll
        for (int i = 0; i < N1 * Q1; ++i) L1[i] = sL1[i];
        tensor_contract_df<N1, Q1>(L1, P, Cc);
      }
      float2 *Ke = a.Kraw + e * (N * N);
#pragma unroll
      for (int r = 0; r < N; ++r) {
        DF k = {0.f, 0.f};
#pragma unroll
        for (int t = 0; t < 6; ++t) k = df_fma_lazy(k, A2[t], ld_df(sD + (t * N + r) * N + b));
        k = df_norm(k);
        if (FORM == LMG_ADVDIFF) k = df_add(k, Cc[hex_tensor(N, r)]);
        Ke[r * N + b] = make_float2(k.hi, k.lo);
      }
      DF fe = {0.f, 0.f};
#pragma unroll
      for (int q = 0; q < Q; ++q) fe = df_fma_lazy(fe, ld_df(sfq + q), ld_df(sphi + q * N + b));
      a.Fraw[e * N + b] = df_to_double(df_norm(fe));
    }
    __syncwarp();
  }
}

template <int FORM, int N, int Q>
void launch_full(const GenElemArgs &a, int max_ctas, cudaStream_t s) {
  const size_t smem = sizeof(double) * ((size_t)Q * N * 5 + 6 * N * N + Q + N * 3 + 10 * a.n_modes +
                                        (size_t)WARPS * (N * 3 + N + 4 * Q + 8 * a.n_modes));
  static size_t attr = 0;  // largest dynamic shared memory granted so far
  if (smem > attr) {
    cudaFuncSetAttribute(k_elem_full<FORM, N, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = smem;
  }
  const int64_t need = (a.n_elem + WARPS - 1) / WARPS;
  const int grid = (int)(need < (int64_t)max_ctas ? need : (int64_t)max_ctas);
  if (grid > 0) k_elem_full<FORM, N, Q><<<grid, WARPS * 32, smem, s>>>(a);
}

// Dynamic shared memory: K [N][N] (double-float), F [N], L = C^T K [max_ne][N]
// (double-float), coefficients [max_ent] (FP64 and double-float), column
// pointers [max_ne + 1], row indices [max_ent].  The matrix products run in
// double-float arithmetic on the FP32 pipe; the load in FP64.
__global__ void __launch_bounds__(128) k_constrain(ConsArgs c) {
  extern __shared__ double csm[];
  const int N = c.N;
  float2 *sK = reinterpret_cast<float2 *>(csm);
  double *sF = reinterpret_cast<double *>(sK + N * N);
  float2 *sL = reinterpret_cast<float2 *>(sF + N);
  double *scv = reinterpret_cast<double *>(sL + c.max_ne * N);
  float2 *scv2 = reinterpret_cast<float2 *>(scv + c.max_ent);
  int32_t *scp = reinterpret_cast<int32_t *>(scv2 + c.max_ent);
  uint8_t *sci = reinterpret_cast<uint8_t *>(scp + c.max_ne + 1);
  for (int64_t k = blockIdx.x; k < c.n_cons; k += gridDim.x) {
    const int64_t e = c.elem[k];
    const int ne = c.ne[k];
    const int64_t cb = c.cbase[k], eb = c.ebase[k];
    const uint64_t rows = c.rowmask[k];
    __syncthreads();
    for (int i = threadIdx.x; i < N * N; i += blockDim.x) sK[i] = c.Kraw[e * N * N + i];
    for (int i = threadIdx.x; i < N; i += blockDim.x) sF[i] = c.Fraw[e * N + i];
    for (int i = threadIdx.x; i <= ne; i += blockDim.x) scp[i] = c.ccp[cb + i];
    __syncthreads();
    const int n_ent = scp[ne];
    for (int i = threadIdx.x; i < n_ent; i += blockDim.x) {
      sci[i] = c.ci[eb + i];
      const double v = c.cv[eb + i];
      scv[i] = v;
      const DF x = df_split(v);
      scv2[i] = make_float2(x.hi, x.lo);
    }
    __syncthreads();
    // L_pj = sum_i C_ip K_ij (rows of constrained local dofs are replaced below)
    for (int idx = threadIdx.x; idx < ne * N; idx += blockDim.x) {
      const int p = idx / N, j = idx - p * N;
      DF l = {0.f, 0.f};
      if (!(p < N && ((rows >> p) & 1ull)))
        for (int u = scp[p]; u < scp[p + 1]; ++u) {
          const float2 cv = scv2[u], kv = sK[sci[u] * N + j];
          l = df_fma_lazy(l, DF{cv.x, cv.y}, DF{kv.x, kv.y});
        }
      l = df_norm(l);
      sL[idx] = make_float2(l.hi, l.lo);
    }
    __syncthreads();
    float2 *out = c.Ebuf + c.kout[k];
    for (int idx = threadIdx.x; idx < ne * ne; idx += blockDim.x) {
      const int p = idx / ne, q = idx - p * ne;
      DF v = {0.f, 0.f};
      if (p < N && ((rows >> p) & 1ull)) {
        if (p == q) {
          v = DF{1.f, 0.f};
        } else {
          for (int t = scp[q]; t < scp[q + 1]; ++t)
            if (sci[t] == p) v = DF{-scv2[t].x, -scv2[t].y};
        }
      } else {
        const float2 *lp = sL + p * N;
        for (int t = scp[q]; t < scp[q + 1]; ++t) {
          const float2 lv = lp[sci[t]], cv = scv2[t];
          v = df_fma_lazy(v, DF{lv.x, lv.y}, DF{cv.x, cv.y});
        }
        v = df_norm(v);
      }
      out[idx] = make_float2(v.hi, v.lo);
    }
    double *fo = c.Fbuf + c.fout[k];
    for (int p = threadIdx.x; p < ne; p += blockDim.x) {
      double v = 0.0;
      for (int u = scp[p]; u < scp[p + 1]; ++u) v += scv[u] * sF[sci[u]];
      fo[p] = v;
    }
  }
}

// K[s] = sum of the slot's contributions in element order, over element
// matrices stored as double-float pairs: summed in double-float arithmetic on
// the FP32 pipe and rounded to FP64 once per entry; F likewise per dof in FP64.
__global__ void k_gather_full_df(int64_t nnz, const int64_t *__restrict__ cptr, const uint32_t *__restrict__ coff,
                                 const float2 *__restrict__ E, double *__restrict__ K, int64_t n_dofs,
                                 const int64_t *__restrict__ fptr, const uint32_t *__restrict__ foff,
                                 const double *__restrict__ Fb, double *__restrict__ F) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < nnz + n_dofs; s += stride) {
    if (s < nnz) {
      DF v = {0.f, 0.f};
      for (int64_t t = cptr[s]; t < cptr[s + 1]; ++t) {
        const float2 x = E[coff[t]];
        v = df_add(v, DF{x.x, x.y});
      }
      K[s] = df_to_double(v);
    } else {
      const int64_t d = s - nnz;
      double v = 0.0;
      for (int64_t t = fptr[d]; t < fptr[d + 1]; ++t) v += Fb[foff[t]];
      F[d] = v;
    }
  }
}

}  // namespace

bool gen_elements_built(int form, int n, int q) {
  if (form != LMG_POISSON && form != LMG_ADVDIFF) return false;
  return (n == 8 || n == 27) && (q == 8 || q == 27);
}

void launch_gen_elements(int form, int n, int q, const GenElemArgs &a, int max_ctas, cudaStream_t s) {
#define LMG_G(F, NN, QQ) \
  if (form == F && n == NN && q == QQ) return launch_full<F, NN, QQ>(a, max_ctas, s);
  LMG_G(LMG_POISSON, 8, 8)
  LMG_G(LMG_POISSON, 8, 27)
  LMG_G(LMG_POISSON, 27, 8)
  LMG_G(LMG_POISSON, 27, 27)
  LMG_G(LMG_ADVDIFF, 8, 8)
  LMG_G(LMG_ADVDIFF, 8, 27)
  LMG_G(LMG_ADVDIFF, 27, 8)
  LMG_G(LMG_ADVDIFF, 27, 27)
#undef LMG_G
}

void launch_constrain(const ConsArgs &c, int n_sm, cudaStream_t s) {
  if (c.n_cons <= 0) return;
  const int64_t g = c.n_cons < (int64_t)n_sm * 16 ? c.n_cons : (int64_t)n_sm * 16;
  const size_t smem = sizeof(double) * ((size_t)c.N * c.N + c.N + (size_t)c.max_ne * c.N + 2 * (size_t)c.max_ent) +
                      sizeof(int32_t) * (c.max_ne + 1) + c.max_ent;
  static size_t attr = 0;
  if (smem > attr) {
    cudaFuncSetAttribute(k_constrain, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = smem;
  }
  k_constrain<<<(int)g, 128, smem, s>>>(c);
}

void launch_gather_full_df(int64_t nnz, const int64_t *cptr, const uint32_t *coff, const float2 *E, double *K,
                           int64_t n_dofs, const int64_t *fptr, const uint32_t *foff, const double *Fb, double *F,
                           int n_sm, cudaStream_t s) {
  const int64_t items = nnz + n_dofs;
  const int64_t blocks = (items + 255) / 256;
  const int g = (int)(blocks < (int64_t)n_sm * 16 ? blocks : (int64_t)n_sm * 16);
  k_gather_full_df<<<g, 256, 0, s>>>(nnz, cptr, coff, E, K, n_dofs, fptr, foff, Fb, F);
}

}  // namespace lmg
