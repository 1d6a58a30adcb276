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

// Arithmetic of the element contraction: T = double for the FP64 drop-in,
// T = float for the mixed form.  The map (J, detJ, J^-1) is FP64 in both.
template <typename T> struct GA;
template <> struct GA<double> {
  static __device__ __forceinline__ double fma_(double a, double b, double c) { return fma(a, b, c); }
  static __device__ __forceinline__ void sincos_(double x, double &s, double &c) { sincos(x, &s, &c); }
};
template <> struct GA<float> {
  static __device__ __forceinline__ float fma_(float a, float b, float c) { return fmaf(a, b, c); }
  static __device__ __forceinline__ void sincos_(double x, float &s, float &c) { sincosf((float)x, &s, &c); }
};

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
// L_i(x_q1) L_j(x_q2) L_k(x_q3), q = q1 + Q1 (q2 + Q1 q3); three 1-D passes.
template <int N1, int Q1, typename T>
__device__ __forceinline__ void tensor_contract(const T *L1, const T *P, T *Cc) {
  using A = GA<T>;
  T T1[N1 * Q1 * Q1];
#pragma unroll
  for (int i = 0; i < N1; ++i)
#pragma unroll
    for (int r = 0; r < Q1 * Q1; ++r) {
      T t = 0;
#pragma unroll
      for (int q1 = 0; q1 < Q1; ++q1) t = A::fma_(L1[i * Q1 + q1], P[q1 + Q1 * r], t);
      T1[i * Q1 * Q1 + r] = t;
    }
  T T2[N1 * N1 * Q1];
#pragma unroll
  for (int i = 0; i < N1; ++i)
#pragma unroll
    for (int j = 0; j < N1; ++j)
#pragma unroll
      for (int q3 = 0; q3 < Q1; ++q3) {
        T t = 0;
#pragma unroll
        for (int q2 = 0; q2 < Q1; ++q2) t = A::fma_(L1[j * Q1 + q2], T1[i * Q1 * Q1 + q2 + Q1 * q3], t);
        T2[(i * N1 + j) * Q1 + q3] = t;
      }
#pragma unroll
  for (int i = 0; i < N1; ++i)
#pragma unroll
    for (int j = 0; j < N1; ++j)
#pragma unroll
      for (int k = 0; k < N1; ++k) {
        T t = 0;
#pragma unroll
        for (int q3 = 0; q3 < Q1; ++q3) t = A::fma_(L1[k * Q1 + q3], T2[(i * N1 + j) * Q1 + q3], t);
        Cc[i + 3 * j + 9 * k] = t;
      }
}

// Byte layout of k_elem_full's dynamic shared memory (T = element arithmetic).
template <typename T>
struct FullSmem {
  int N, Q, modes;
  __host__ __device__ size_t al8(size_t x) const { return (x + 7) & ~(size_t)7; }
  __host__ __device__ size_t phi() const { return 0; }                                  // [Q][N] T
  __host__ __device__ size_t dphi() const { return al8(phi() + sizeof(T) * Q * N); }      // [Q][N][3] T
  __host__ __device__ size_t D() const { return al8(dphi() + sizeof(T) * Q * N * 3); }     // [6][N][N] T
  __host__ __device__ size_t curl() const { return al8(D() + sizeof(T) * 6 * N * N); }     // [modes][3] T
  __host__ __device__ size_t qw() const { return al8(curl() + sizeof(T) * 3 * modes); }    // [Q] double
  __host__ __device__ size_t mode() const { return qw() + sizeof(double) * Q; }          // [7 modes] double
  __host__ __device__ size_t warp0() const { return mode() + sizeof(double) * 7 * modes; }
  // per warp: X [N][3] double, then f [N], beta [Q][3], fq [Q], E [modes][4][2] in T
  __host__ __device__ size_t per_warp() const {
    return al8(sizeof(double) * N * 3 + sizeof(T) * (N + 4 * Q + 8 * modes));
  }
  __host__ __device__ size_t bytes(int warps) const { return warp0() + per_warp() * warps; }
};

template <int FORM, int N, int Q, typename T>
__global__ void __launch_bounds__(WARPS * 32) k_elem_full(GenElemArgs a) {
  using A = GA<T>;
  constexpr int N1 = (N == 8) ? 2 : 3, Q1 = (Q == 8) ? 2 : 3;
  extern __shared__ __align__(16) unsigned char gsm[];
  const FullSmem<T> L{N, Q, a.n_modes};
  T *sphi = reinterpret_cast<T *>(gsm + L.phi());
  T *sdphi = reinterpret_cast<T *>(gsm + L.dphi());
  T *sD = reinterpret_cast<T *>(gsm + L.D());
  T *scurl = reinterpret_cast<T *>(gsm + L.curl());
  double *sqw = reinterpret_cast<double *>(gsm + L.qw());
  double *smode = reinterpret_cast<double *>(gsm + L.mode());
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  double *sX = reinterpret_cast<double *>(gsm + L.warp0() + L.per_warp() * warp);  // [N][3]
  T *sf = reinterpret_cast<T *>(sX + N * 3);  // [N] nodal load
  T *sbeta = sf + N;                          // [Q][3] JxW (J^-1 b)
  T *sfq = sbeta + 3 * Q;                     // [Q] JxW f(x_q)
  T *sE = sfq + Q;                            // [n_modes][4] (cos, sin)
  for (int i = threadIdx.x; i < Q * N; i += blockDim.x) sphi[i] = (T)a.fe.phi[i];
  for (int i = threadIdx.x; i < Q * N * 3; i += blockDim.x) sdphi[i] = (T)a.fe.dphi[i];
  for (int i = threadIdx.x; i < 6 * N * N; i += blockDim.x) sD[i] = (T)a.D6[i];
  for (int i = threadIdx.x; i < Q; i += blockDim.x) sqw[i] = a.fe.qw[i];
  for (int i = threadIdx.x; i < 7 * a.n_modes; i += blockDim.x) smode[i] = a.modes[i];
  for (int i = threadIdx.x; i < 3 * a.n_modes; i += blockDim.x) {  // b = sum_m cos(.) k_m x a_m
    const double *md = a.modes + 7 * (i / 3);
    const int d = i % 3;
    scurl[i] = (T)(d == 0 ? md[4] * md[2] - md[5] * md[1]
                   : d == 1 ? md[5] * md[0] - md[3] * md[2]
                            : md[3] * md[1] - md[4] * md[0]);
  }
  __shared__ T sL1[9];
  __shared__ double sG[WARPS][10];  // J^-1 (dxi_m/dx_d at [3m + d]) and detJ of each warp's element
  for (int i = threadIdx.x; i < N1 * Q1; i += blockDim.x) sL1[i] = (T)a.D6[6 * N * N + i];
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
      sf[lane] = (T)(a.nodal_f ? a.nodal_f[nd] : 0.0);
    }
    __syncwarp();
    // The elements here are affine hexahedra (form_set refuses the others):
    // compute_affine_map takes the map at the first quadrature point,
    // J[m][d] = sum_a dphi_a/dxi_m x_a[d] over the N map nodes in node order
    // (fe_map.C:1167-1245, 980-1044), then detJ and J^-1 by cofactors
    // (fe_map.C:1046-1068).  On small elements far from the origin the node
    // sum cancels to a few digits, so it is formed exactly as the reference
    // forms it: FP64, node order, every product and sum rounded separately
    // (no fused multiply-adds).  Lane j < 9 forms J[j]; lane 0 the rest.
    if (lane < 9) {
      const int m = lane / 3, d = lane - 3 * m;
      double acc = 0.0;
      for (int g = 0; g < N; ++g) acc = __dadd_rn(acc, __dmul_rn(a.fe.gdphi[3 * g + m], sX[3 * g + d]));
      sG[warp][lane] = acc;
    }
    __syncwarp();
    if (lane == 0) {
      double J[9];  // J[m*3+d] = d x_d / d xi_m
#pragma unroll
      for (int j = 0; j < 9; ++j) J[j] = sG[warp][j];
      auto cof = [](double a, double b, double c, double d) { return __dsub_rn(__dmul_rn(a, b), __dmul_rn(c, d)); };
      const double c0 = cof(J[4], J[8], J[5], J[7]), c1 = cof(J[5], J[6], J[3], J[8]), c2 = cof(J[3], J[7], J[4], J[6]);
      const double det = __dadd_rn(__dadd_rn(__dmul_rn(J[0], c0), __dmul_rn(J[1], c1)), __dmul_rn(J[2], c2));
      const double inv = __ddiv_rn(1.0, det);
      double *G = sG[warp];
      G[0] = __dmul_rn(c0, inv);
      G[1] = __dmul_rn(c1, inv);
      G[2] = __dmul_rn(c2, inv);
      G[3] = __dmul_rn(cof(J[2], J[7], J[1], J[8]), inv);
      G[4] = __dmul_rn(cof(J[0], J[8], J[2], J[6]), inv);
      G[5] = __dmul_rn(cof(J[1], J[6], J[0], J[7]), inv);
      G[6] = __dmul_rn(cof(J[1], J[5], J[2], J[4]), inv);
      G[7] = __dmul_rn(cof(J[2], J[3], J[0], J[5]), inv);
      G[8] = __dmul_rn(cof(J[0], J[4], J[1], J[3]), inv);
      G[9] = det;
      if (!(det > 0.0)) {
        atomicCAS(a.status, 0, LMG_ERR_DEGENERATE);
        atomicMin(a.bad_elem, (unsigned long long)e);
      }
    }
    __syncwarp();
    const double *G = sG[warp];
    const double det = G[9];
    const double coef = a.coef ? a.coef[e] : 1.0;
    const double kap = (FORM == LMG_ADVDIFF ? a.kappa * coef : coef) * det;
    auto gg = [&](int m, int n) {
      return G[3 * m] * G[3 * n] + G[3 * m + 1] * G[3 * n + 1] + G[3 * m + 2] * G[3 * n + 2];
    };
    T A2[6];
    A2[0] = (T)(kap * gg(0, 0));
    A2[1] = (T)(kap * gg(1, 1));
    A2[2] = (T)(kap * gg(2, 2));
    A2[3] = (T)(kap * gg(0, 1));
    A2[4] = (T)(kap * gg(0, 2));
    A2[5] = (T)(kap * gg(1, 2));
    const bool axis = A2[3] == (T)0 && A2[4] == (T)0 && A2[5] == (T)0;  // axis-aligned element: diagonal tensor
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
        T sn, cs;
        A::sincos_(ang, sn, cs);
        sE[2 * t] = cs;
        sE[2 * t + 1] = sn;
      }
      __syncwarp();
    }
    // per quadrature point: transport coefficients and the load
    if (lane < Q) {
      const int q = lane;
      T fx = 0;
      for (int c = 0; c < N; ++c) fx = A::fma_(sphi[q * N + c], sf[c], fx);  // FE-interpolated load
      const T jw = (T)(det * sqw[q]);
      sfq[q] = jw * fx;
      if (FORM == LMG_ADVDIFF) {
        T b[3] = {0, 0, 0};
        // offset of this point along each reference axis: -1, 0 or +1 times gp
        const int qi[3] = {q % Q1, (q / Q1) % Q1, q / (Q1 * Q1)};
        for (int m = 0; m < a.n_modes; ++m) {
          const T *E = sE + 8 * m;
          T re = E[0], im = E[1];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            if (Q1 == 3 && qi[d] == 1) continue;
            const T c = E[2 * (d + 1)];
            const T sn = qi[d] == 0 ? -E[2 * (d + 1) + 1] : E[2 * (d + 1) + 1];
            const T r2 = A::fma_(re, c, -(im * sn));
            im = A::fma_(re, sn, im * c);
            re = r2;
          }
#pragma unroll
          for (int d = 0; d < 3; ++d) b[d] = A::fma_(re, scurl[3 * m + d], b[d]);
        }
#pragma unroll
        for (int m = 0; m < 3; ++m) {
          T t = 0;
#pragma unroll
          for (int d = 0; d < 3; ++d) t = A::fma_((T)G[3 * m + d], b[d], t);
          sbeta[3 * q + m] = jw * t;
        }
      }
    }
    __syncwarp();
    if (lane < N) {
      // column b of Ke: convection by sum factorisation, diffusion from the reference tensors
      const int b = lane;
      T Cc[27];
      if (FORM == LMG_ADVDIFF) {
        T P[Q];
#pragma unroll
        for (int q = 0; q < Q; ++q) {
          const T *d = sdphi + (q * N + b) * 3;
          T t = 0;
#pragma unroll
          for (int m = 0; m < 3; ++m) t = A::fma_(sbeta[3 * q + m], d[m], t);
          P[q] = t;
        }
        T L1[N1 * Q1];
#pragma unroll
        for (int i = 0; i < N1 * Q1; ++i) L1[i] = sL1[i];
        tensor_contract<N1, Q1, T>(L1, P, Cc);
      }
      T *Ke = reinterpret_cast<T *>(a.Kraw) + e * (N * N);
#pragma unroll
      for (int r = 0; r < N; ++r) {
        T k = 0;
        if (axis) {
#pragma unroll
          for (int t = 0; t < 3; ++t) k = A::fma_(A2[t], sD[(t * N + r) * N + b], k);
        } else {
#pragma unroll
          for (int t = 0; t < 6; ++t) k = A::fma_(A2[t], sD[(t * N + r) * N + b], k);
        }
        if (FORM == LMG_ADVDIFF) k += Cc[hex_tensor(N, r)];
        Ke[r * N + b] = k;
      }
      double fe = 0.0;
#pragma unroll
      for (int q = 0; q < Q; ++q) fe = fma((double)sfq[q], (double)sphi[q * N + b], fe);
      a.Fraw[e * N + b] = fe;
    }
    __syncwarp();
  }
}

template <int FORM, int N, int Q, typename T>
void launch_full(const GenElemArgs &a, int max_ctas, cudaStream_t s) {
  const size_t smem = FullSmem<T>{N, Q, a.n_modes}.bytes(WARPS);
  static size_t attr = 0;  // largest dynamic shared memory granted so far
  if (smem > attr) {
    cudaFuncSetAttribute(k_elem_full<FORM, N, Q, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = smem;
  }
  const int64_t need = (a.n_elem + WARPS - 1) / WARPS;
  const int grid = (int)(need < (int64_t)max_ctas ? need : (int64_t)max_ctas);
  if (grid > 0) k_elem_full<FORM, N, Q, T><<<grid, WARPS * 32, smem, s>>>(a);
}

// Dynamic shared memory: K [N][N] (T), F [N] (FP64), L = C^T K [max_ne][N]
// (T), coefficients [max_ent] (FP64 and T), column pointers [max_ne + 1], row
// indices [max_ent].  The matrix products run in T (FP64 for the drop-in,
// FP32 for the mixed form); the load in FP64.
template <typename T>
__global__ void __launch_bounds__(128) k_constrain(ConsArgs c) {
  using A = GA<T>;
  extern __shared__ double csm[];
  const int N = c.N;
  T *sK = reinterpret_cast<T *>(csm);
  double *sF = reinterpret_cast<double *>(csm + (sizeof(T) * N * N + 7) / 8);
  T *sL = reinterpret_cast<T *>(sF + N);
  double *scv = reinterpret_cast<double *>(reinterpret_cast<unsigned char *>(sL) +
                                           ((sizeof(T) * c.max_ne * N + 7) & ~(size_t)7));
  T *scvT = reinterpret_cast<T *>(scv + c.max_ent);
  int32_t *scp = reinterpret_cast<int32_t *>(reinterpret_cast<unsigned char *>(scvT) +
                                             ((sizeof(T) * c.max_ent + 7) & ~(size_t)7));
  uint8_t *sci = reinterpret_cast<uint8_t *>(scp + c.max_ne + 1);
  const T *Kraw = reinterpret_cast<const T *>(c.Kraw);
  for (int64_t k = blockIdx.x; k < c.n_cons; k += gridDim.x) {
    const int64_t e = c.elem[k];
    const int ne = c.ne[k];
    const int64_t cb = c.cbase[k], eb = c.ebase[k];
    const uint64_t rows = c.rowmask[k];
    __syncthreads();
    for (int i = threadIdx.x; i < N * N; i += blockDim.x) sK[i] = Kraw[e * N * N + i];
    for (int i = threadIdx.x; i < N; i += blockDim.x) sF[i] = c.Fraw[e * N + i];
    for (int i = threadIdx.x; i <= ne; i += blockDim.x) scp[i] = c.ccp[cb + i];
    __syncthreads();
    const int n_ent = scp[ne];
    for (int i = threadIdx.x; i < n_ent; i += blockDim.x) {
      sci[i] = c.ci[eb + i];
      const double v = c.cv[eb + i];
      scv[i] = v;
      scvT[i] = (T)v;
    }
    __syncthreads();
    // L_pj = sum_i C_ip K_ij (rows of constrained local dofs are replaced below)
    for (int idx = threadIdx.x; idx < ne * N; idx += blockDim.x) {
      const int p = idx / N, j = idx - p * N;
      T l = 0;
      if (!(p < N && ((rows >> p) & 1ull)))
        for (int u = scp[p]; u < scp[p + 1]; ++u) l = A::fma_(scvT[u], sK[sci[u] * N + j], l);
      sL[idx] = l;
    }
    __syncthreads();
    T *out = reinterpret_cast<T *>(c.Ebuf) + c.kout[k];
    for (int idx = threadIdx.x; idx < ne * ne; idx += blockDim.x) {
      const int p = idx / ne, q = idx - p * ne;
      T v = 0;
      if (p < N && ((rows >> p) & 1ull)) {
        if (p == q) {
          v = 1;
        } else {
          for (int t = scp[q]; t < scp[q + 1]; ++t)
            if (sci[t] == p) v = -scvT[t];
        }
      } else {
        const T *lp = sL + p * N;
        for (int t = scp[q]; t < scp[q + 1]; ++t) v = A::fma_(lp[sci[t]], scvT[t], v);
      }
      out[idx] = v;
    }
    double *fo = c.Fbuf + c.fout[k];
    for (int p = threadIdx.x; p < ne; p += blockDim.x) {
      double v = 0.0;
      for (int u = scp[p]; u < scp[p + 1]; ++u) v += scv[u] * sF[sci[u]];
      fo[p] = v;
    }
  }
}

// K[s] = sum of the slot's contributions in element order; F likewise per
// dof in FP64.  FP64 drop-in: FP64 sums of the FP64 element entries.  Mixed
// form: the FP32 entries are summed in double-float on the FP32 pipe (TwoSum
// on the high parts, errors collected in the low part, a 48-bit significand)
// and rounded to FP64 once -- widening each entry to FP64 first would put two
// FP64-pipe operations on every contribution.
template <typename T>
__global__ void k_gather_full(int64_t nnz, const int64_t *__restrict__ cptr, const uint32_t *__restrict__ coff,
                              const T *__restrict__ E, double *__restrict__ K, int64_t n_dofs,
                              const int64_t *__restrict__ fptr, const uint32_t *__restrict__ foff,
                              const double *__restrict__ Fb, double *__restrict__ F, int64_t s0, int64_t s1,
                              int64_t d0, int64_t d1) {
  const int64_t stride = (int64_t)gridDim.x * blockDim.x, ns = s1 - s0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < ns + d1 - d0; i += stride) {
    const int64_t s = i < ns ? s0 + i : nnz + d0 + (i - ns);
    if (s < nnz) {
      if constexpr (sizeof(T) == 4) {
        float hi = 0.f, lo = 0.f;
        for (int64_t t = cptr[s]; t < cptr[s + 1]; ++t) {
          const float x = E[coff[t]];
          const float sum = __fadd_rn(hi, x), bb = __fsub_rn(sum, hi);
          lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(sum, bb)), __fsub_rn(x, bb)));
          hi = sum;
        }
        K[s] = (double)hi + (double)lo;
      } else {
        double v = 0.0;
        for (int64_t t = cptr[s]; t < cptr[s + 1]; ++t) v += (double)E[coff[t]];
        K[s] = v;
      }
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

void launch_gen_elements(int form, int n, int q, bool mixed, const GenElemArgs &a, int max_ctas, cudaStream_t s) {
#define LMG_G(F, NN, QQ)                                                        \
  if (form == F && n == NN && q == QQ) {                                        \
    if (mixed) launch_full<F, NN, QQ, float>(a, max_ctas, s);                   \
    else launch_full<F, NN, QQ, double>(a, max_ctas, s);                        \
    return;                                                                     \
  }
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

template <typename T>
void launch_constrain_t(const ConsArgs &c, int n_sm, cudaStream_t s) {
  const int64_t g = c.n_cons < (int64_t)n_sm * 16 ? c.n_cons : (int64_t)n_sm * 16;
  auto r8 = [](size_t x) { return (x + 7) & ~(size_t)7; };
  const size_t smem = r8(sizeof(T) * c.N * c.N) + sizeof(double) * c.N + r8(sizeof(T) * c.max_ne * c.N) +
                      sizeof(double) * c.max_ent + r8(sizeof(T) * c.max_ent) + sizeof(int32_t) * (c.max_ne + 1) +
                      c.max_ent;
  static size_t attr = 0;
  if (smem > attr) {
    cudaFuncSetAttribute(k_constrain<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = smem;
  }
  k_constrain<T><<<(int)g, 128, smem, s>>>(c);
}

void launch_constrain(const ConsArgs &c, bool mixed, int n_sm, cudaStream_t s) {
  if (c.n_cons <= 0) return;
  if (mixed) launch_constrain_t<float>(c, n_sm, s);
  else launch_constrain_t<double>(c, n_sm, s);
}

void launch_gather_full(int64_t nnz, const int64_t *cptr, const uint32_t *coff, const void *E, bool mixed, double *K,
                        int64_t n_dofs, const int64_t *fptr, const uint32_t *foff, const double *Fb, double *F,
                        int n_sm, cudaStream_t s, int64_t s0, int64_t s1, int64_t d0, int64_t d1) {
  const int64_t items = (s1 - s0) + (d1 - d0);
  if (items <= 0) return;
  const int64_t blocks = (items + 255) / 256;
  const int g = (int)(blocks < (int64_t)n_sm * 16 ? blocks : (int64_t)n_sm * 16);
  if (mixed)
    k_gather_full<float><<<g, 256, 0, s>>>(nnz, cptr, coff, static_cast<const float *>(E), K, n_dofs, fptr, foff,
                                            Fb, F, s0, s1, d0, d1);
  else
    k_gather_full<double><<<g, 256, 0, s>>>(nnz, cptr, coff, static_cast<const double *>(E), K, n_dofs, fptr, foff,
                                             Fb, F, s0, s1, d0, d1);
}

}  // namespace lmg
