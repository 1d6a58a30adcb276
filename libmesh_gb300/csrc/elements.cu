// Element kernels: per-element Jacobian, inverse and determinant in FP64 and
// the weak-form contraction, written to a per-element block buffer that the
// gather kernel reduces into CSR values.
//
// What the reference does per element (the user's assembly callback):
//   FE::reinit -> FEMap::compute_affine_map | compute_single_point_map
//     (src/fe/fe_map.C:1167-1245, 980-1078), map_dphi (src/fe/h1_fe_transformation.C:64-195),
//   then Ke(i,j) += JxW dphi_i.dphi_j (introduction_ex4.C:467) or the
//   elasticity form (systems_of_equations_ex6.C:222-230), then
//   constrain_element_matrix_and_vector (src/base/dof_map_constraints.C:2439-2515).
// Here two kernels cover that:
//   * k_elem_affine: elements whose map is affine (Elem::has_affine_map).  The
//     Jacobian is taken once at qp 0 as libMesh does; the quadrature sum is
//     folded into reference tensors S^{mn}_{ab} = sum_q w_q dphi_a/dxi_m dphi_b/dxi_n,
//     so Ke_ab = sum_mn A_mn S^{mn}_ab with an element tensor A built from
//     detJ, J^-1 and the coefficients.  One warp takes 32 elements: lane = element
//     for the geometry, lane = output block for the contraction.
//   * k_elem_general: any element; the Jacobian, detJ and J^-1 at every qp,
//     physical gradients per qp, and accumulation over qps (warp per element).
// Dirichlet rows/columns are applied in the epilogue: a constrained local dof
// gets a zero row and column with 1 on the diagonal and a zero load, which is
// what C^T K C and C^T F give for an empty constraint row.
//
// Both forms are symmetric (K^{ik}_{ab} = K^{ki}_{ba}), so only the n diagonal
// blocks and the n(n-1)/2 strictly upper blocks are computed and stored; the
// gather reads a lower block as the transpose of its upper partner.
// FP64 drop-in: the geometry (J, J^-1, detJ), the element tensor A, the load
// vector and the non-affine path run in native FP64; the affine contraction
// sum_mn A_mn S^{mn}_ab runs in double-float arithmetic (df.cuh) on the FP32
// pipe, which GB300 executes 64x faster than FP64, with a 48-bit significand.
// The mixed form (T = float) contracts only the off-diagonal blocks, in FP32,
// and stores them without the Dirichlet epilogue; the insertion kernel applies
// the constraints and rebuilds every diagonal block of the global matrix as
// minus the (double-float accumulated) sum of its row's off-diagonal blocks.
// That identity is exact in real arithmetic because sum_b dphi_b = 0, and
// enforcing it keeps every rigid translation in the kernel of K.
#include <cuda_runtime.h>

#include <type_traits>

#include "assemble.cuh"
#include "df.cuh"
#include "elem_geom.cuh"
#include "../../include/libmesh_gb300.h"

namespace lmg {

namespace {

constexpr unsigned FULL = 0xffffffffu;

__device__ __forceinline__ void report_bad(const ElemArgs &a, int code, int64_t e) {
  atomicCAS(a.status, 0, code);
  atomicMin(a.bad_elem, (unsigned long long)e);
}

// Strictly upper block index o of (a, b), a < b, and its inverse.
__host__ __device__ constexpr int off_index(int N, int a, int b) { return a * N - a * (a + 1) / 2 + (b - a - 1); }

template <int N>
__device__ __forceinline__ void build_pairs(uint16_t *pair) {
  for (int o = threadIdx.x; o < N * (N - 1) / 2; o += blockDim.x) {
    int a = 0, rem = o;
    while (rem >= N - 1 - a) { rem -= N - 1 - a; ++a; }
    pair[o] = (uint16_t)((a << 8) | (a + 1 + rem));
  }
}

// Dirichlet epilogue of one entry (local rows lr, lc).
__device__ __forceinline__ double masked(double v, uint64_t mask, int lr, int lc) {
  if (((mask >> lr) | (mask >> lc)) & 1ull) return (lr == lc) ? 1.0 : 0.0;
  return v;
}

// Arithmetic of the affine contraction: T = float2 is a double-float pair
// (FP64 drop-in, df.cuh), T = float plain FP32 (mixed form).
template <typename T> struct Ar;
template <> struct Ar<float> {
  using V = float;
  static __device__ __forceinline__ V zero() { return 0.f; }
  static __device__ __forceinline__ V from(double x) { return (float)x; }
  static __device__ __forceinline__ V ld(float x) { return x; }
  static __device__ __forceinline__ V fma(V acc, V a, V b) { return fmaf(a, b, acc); }
  static __device__ __forceinline__ V mul(V a, V b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ V norm(V x) { return x; }
};
template <> struct Ar<float2> {
  using V = DF;
  static __device__ __forceinline__ V zero() { return {0.f, 0.f}; }
  static __device__ __forceinline__ V from(double x) { return df_split(x); }
  static __device__ __forceinline__ V ld(float2 x) { return {x.x, x.y}; }
  static __device__ __forceinline__ V fma(V acc, V a, V b) { return df_fma_lazy(acc, a, b); }
  // a * b as an unevaluated pair: TwoProduct's high part, the rounding error
  // and the cross terms in the low part (df_fma_lazy into zero, without the sum)
  static __device__ __forceinline__ V mul(V a, V b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return {p, e};
  }
  static __device__ __forceinline__ V norm(V x) { return df_norm(x); }
};
__device__ __forceinline__ void st(float &o, float v) { o = v; }
__device__ __forceinline__ void st(float2 &o, DF v) { o = make_float2(v.hi, v.lo); }

// Per-element operands of the affine contraction, in T:
//   POISSON:    A_mn = k detJ (G G^T)_mn                    (9)
//   ELASTICITY: G_mn, lam detJ, mu detJ                     (11)
template <int FORM> struct Geo { static constexpr int NG = (FORM == LMG_POISSON) ? 9 : 11; };

// One element block from the per-element operands gv (Geo<FORM>::NG values)
// and the reference tensors sv = S^{mn}_{ab} (9 values) of the block (a, b):
//   POISSON    K_ab = sum_mn A_mn S^{mn}_ab
//   ELASTICITY K^{ik}_ab = lam' P^{ik} + mu' P^{ki} + d_ik mu' tr P, P = G^T S_ab G.
// Shared by the element kernel and the fused row kernel so that both produce
// the same bits.
template <int FORM, typename R>
__device__ __forceinline__ void contract_block(const typename R::V *gv, const typename R::V *sv,
                                               typename R::V *out) {
  using V = typename R::V;
  // Each chain starts with a plain product; the intermediate pairs stay
  // unnormalised (the lazy products take both parts, so the low parts only
  // need to stay small, and every consumer of the output sums both parts).
  if (FORM == LMG_POISSON) {
    V acc = R::mul(gv[0], sv[0]);
#pragma unroll
    for (int mn = 1; mn < 9; ++mn) acc = R::fma(acc, gv[mn], sv[mn]);
    out[0] = R::norm(acc);
  } else {
    // P = G^T S_ab G (T = S_ab G, then G^T T); K^{ik} = lam' P^{ik} + mu' P^{ki} + d_ik mu' tr P
    V Tm[9];
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
      for (int kk = 0; kk < 3; ++kk) {
        V acc = R::mul(sv[3 * m], gv[kk]);
#pragma unroll
        for (int n = 1; n < 3; ++n) acc = R::fma(acc, sv[3 * m + n], gv[3 * n + kk]);
        Tm[3 * m + kk] = acc;
      }
    V Pm[9];
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int kk = 0; kk < 3; ++kk) {
        V acc = R::mul(gv[i], Tm[kk]);
#pragma unroll
        for (int m = 1; m < 3; ++m) acc = R::fma(acc, gv[3 * m + i], Tm[3 * m + kk]);
        Pm[3 * i + kk] = acc;
      }
    V tr = R::mul(Pm[0], R::from(1.0));
#pragma unroll
    for (int i = 1; i < 3; ++i) tr = R::fma(tr, Pm[4 * i], R::from(1.0));
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
      for (int kk = 0; kk < 3; ++kk) {
        V acc = R::mul(gv[9], Pm[3 * i + kk]);
        acc = R::fma(acc, gv[10], Pm[3 * kk + i]);
        if (i == kk) acc = R::fma(acc, gv[10], tr);
        out[3 * i + kk] = acc;
      }
  }
}

// Load vector of one element, Fe_a^v = detJ sum_b M_ab f_b^v, in double-float
// (M the reference mass matrix as pairs, dd = detJ); constrained local dofs
// (mask bit v*N + a) get 0.  For up to ten nodes the element's nodal values of
// a component are loaded once into registers; the sums are the same either way.
template <int N, int NV>
__device__ __forceinline__ void element_load_df(const float2 *nodal_f2, const int32_t *c, const float2 *sM, DF dd,
                                                uint64_t mask, float2 *Fo) {
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    if constexpr (N <= 10) {
      float2 fb[N];
#pragma unroll
      for (int b = 0; b < N; ++b) fb[b] = nodal_f2 ? nodal_f2[(int64_t)c[b] * NV + v] : float2{0.f, 0.f};
      for (int ai = 0; ai < N; ++ai) {
        DF s = {0.f, 0.f};
        if (nodal_f2)
#pragma unroll
          for (int b = 0; b < N; ++b) {
            const float2 mb = sM[ai * N + b];
            s = df_fma_lazy(s, DF{mb.x, mb.y}, DF{fb[b].x, fb[b].y});
          }
        s = df_norm(df_fma_lazy(DF{0.f, 0.f}, df_norm(s), dd));
        Fo[ai * NV + v] = ((mask >> (v * N + ai)) & 1ull) ? make_float2(0.f, 0.f) : make_float2(s.hi, s.lo);
      }
    } else {
      for (int ai = 0; ai < N; ++ai) {
        DF s = {0.f, 0.f};
        if (nodal_f2)
          for (int b = 0; b < N; ++b) {
            const float2 fb = nodal_f2[(int64_t)c[b] * NV + v], mb = sM[ai * N + b];
            s = df_fma_lazy(s, DF{mb.x, mb.y}, DF{fb.x, fb.y});
          }
        s = df_norm(df_fma_lazy(DF{0.f, 0.f}, df_norm(s), dd));
        Fo[ai * NV + v] = ((mask >> (v * N + ai)) & 1ull) ? make_float2(0.f, 0.f) : make_float2(s.hi, s.lo);
      }
    }
  }
}

// Byte offsets of the affine kernel's dynamic shared memory (4 warps per CTA).
__host__ __device__ constexpr size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }
template <int FORM, int N, int NV, typename T>
struct AffineSmem {
  static constexpr int NG = Geo<FORM>::NG;
  static constexpr int NO = N * (N - 1) / 2;
  static constexpr size_t S = 0;                                        // [9][N][N] T
  static constexpr size_t M = S + al16(sizeof(T) * 9 * N * N);          // [N][N] float2
  static constexpr size_t G = M + al16(sizeof(float2) * N * N);         // [4][32][NG] T
  static constexpr size_t MASK = G + al16(sizeof(T) * 4 * 32 * NG);     // [4][32] u64
  static constexpr size_t PAIR = MASK + al16(sizeof(uint64_t) * 4 * 32);
  static constexpr size_t BYTES = PAIR + al16(sizeof(uint16_t) * (NO > 0 ? NO : 1));
};

template <int FORM, int N, int NV, typename T>
__global__ void __launch_bounds__(128) k_elem_affine(ElemArgs a) {
  using R = Ar<T>;
  using V = typename R::V;
  constexpr bool MIXED = sizeof(T) == 4;
  constexpr int NG = Geo<FORM>::NG;
  constexpr int NB = N * N, NO = N * (N - 1) / 2, B2 = NV * NV;
  constexpr int NWORK = MIXED ? NO : N + NO;  // blocks computed by the contraction
  constexpr int BPL = (NWORK + 31) / 32;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using L = AffineSmem<FORM, N, NV, T>;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  T *sS = reinterpret_cast<T *>(smem_raw + L::S);
  float2 *sM = reinterpret_cast<float2 *>(smem_raw + L::M);
  T *sG = reinterpret_cast<T *>(smem_raw + L::G) + warp * 32 * NG;
  uint64_t *sMask = reinterpret_cast<uint64_t *>(smem_raw + L::MASK) + warp * 32;
  uint16_t *sPair = reinterpret_cast<uint16_t *>(smem_raw + L::PAIR);
  for (int i = threadIdx.x; i < 9 * NB; i += blockDim.x) st(sS[i], R::from(a.fe.S[i]));
  for (int i = threadIdx.x; i < NB; i += blockDim.x) st(sM[i], df_split(a.fe.M[i]));
  build_pairs<N>(sPair);
  __syncthreads();

  const int64_t n_tiles = (a.n_list + 31) / 32;
  for (int64_t tile = (int64_t)blockIdx.x * 4 + warp; tile < n_tiles; tile += (int64_t)gridDim.x * 4) {
    const int64_t li = tile * 32 + lane;
    const int32_t e = (li < a.n_list) ? a.list[li] : -1;
    if (e >= 0) {  // lane = element: FP64 geometry at qp 0 (compute_affine_map)
      const int32_t *c = a.conn + (int64_t)e * a.npe;
      double G[9];
      double det;
      {
        double X[N * 3];
#pragma unroll
        for (int g = 0; g < N; ++g) {
          const double *p = a.xyz + 3 * (int64_t)c[g];
          X[3 * g] = p[0];
          X[3 * g + 1] = p[1];
          X[3 * g + 2] = p[2];
        }
        det = jacobian_affine<N>(X, G);
      }
      if (!(det > 0.0)) report_bad(a, LMG_ERR_DEGENERATE, e);
      const double coef = a.coef ? a.coef[e] : 1.0;
      T *g = sG + lane * NG;
      if (FORM == LMG_POISSON) {
        const double s = coef * det;
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
          for (int n = 0; n < 3; ++n)
            st(g[3 * m + n], R::from(s * (G[3 * m] * G[3 * n] + G[3 * m + 1] * G[3 * n + 1] + G[3 * m + 2] * G[3 * n + 2])));
      } else {
        double lam, mu;
        lame(coef, a.nu, lam, mu);
#pragma unroll
        for (int i = 0; i < 9; ++i) st(g[i], R::from(G[i]));
        st(g[9], R::from(lam * det));
        st(g[10], R::from(mu * det));
      }
      const uint64_t mask = a.cmask[e];
      sMask[lane] = mask;
      // Load vector Fe_a^i = detJ sum_b M_ab f_b^i in double-float (both forms).
      float2 *Fo = a.Fe2 + (int64_t)e * N * NV;
      const DF dd = df_split(det);
      element_load_df<N, NV>(a.nodal_f2, c, sM, dd, mask, Fo);
    }
    __syncwarp();
    for (int t = 0; t < 32; ++t) {  // lane = output block
      const int32_t et = __shfl_sync(FULL, e, t);
      if (et < 0) break;
      const T *gt = sG + t * NG;
      V gv[NG];
#pragma unroll
      for (int i = 0; i < NG; ++i) gv[i] = R::ld(gt[i]);
      const uint64_t mask = sMask[t];
      // not unrolled: one copy of the contraction keeps the hot code within
      // the instruction caches (unrolled, the warps stalled on fetch)
#pragma unroll 1
      for (int k = 0; k < BPL; ++k) {
        const int w = lane + 32 * k;
        if (w < NWORK) {
          int ra, cb, o;
          if (!MIXED && w < N) { ra = cb = w; o = -1; }
          else { o = MIXED ? w : w - N; ra = sPair[o] >> 8; cb = sPair[o] & 0xff; }
          const int blk = ra * N + cb;
          V sv[9];
#pragma unroll
          for (int mn = 0; mn < 9; ++mn) sv[mn] = R::ld(sS[mn * NB + blk]);
          V out[B2];
          contract_block<FORM, R>(gv, sv, out);
#pragma unroll
          for (int ik = 0; ik < B2; ++ik) {
            const int i = ik / NV, kk = ik - i * NV;
            const int lr = i * N + ra, lc = kk * N + cb;
            if constexpr (MIXED) {
              a.Koff32[((int64_t)et * NO + o) * B2 + ik] = out[ik];
            } else {
              float2 v = make_float2(out[ik].hi, out[ik].lo);
              if (((mask >> lr) | (mask >> lc)) & 1ull) v = make_float2(lr == lc ? 1.f : 0.f, 0.f);
              if (o < 0) a.Kdiag2[((int64_t)et * N + ra) * B2 + ik] = v;
              else a.Koff2[((int64_t)et * NO + o) * B2 + ik] = v;
            }
          }
        }
      }
    }
    __syncwarp();
  }
}

// Matrix-free residual R = K u - F without forming K (affine elements, the
// FP64 drop-in's arithmetic): LinearImplicitSystem::assembly's residual
// (src/systems/linear_implicit_system.C:367-381) as a per-element product.
// A warp takes 32 elements: lane = element for the FP64 map, the element's
// operands, its u_e and its load vector (the same code as k_elem_affine);
// then lanes (slot, a) take SL = 32 / N elements at a time, lane a forming
// row block a of K_e from the reference tensors and multiplying it into u_e
// in double-float.  Dirichlet rows / columns as the assembled matrix has them:
// a constrained row gives u_a (its row is e_a), a constrained column adds
// nothing.  R_e goes to Re2 and is summed per dof by the load-vector plan.
template <int FORM, int N, int NV>
struct ResidualSmem {
  static constexpr int NG = Geo<FORM>::NG;
  static constexpr size_t S = 0;                                        // [9][N][N] float2
  static constexpr size_t M = S + al16(sizeof(float2) * 9 * N * N);     // [N][N] float2
  static constexpr size_t G = M + al16(sizeof(float2) * N * N);         // [4][32][NG] float2
  static constexpr size_t MASK = G + al16(sizeof(float2) * 4 * 32 * NG);  // [4][32] u64
  static constexpr size_t U = MASK + al16(sizeof(uint64_t) * 4 * 32);  // [4][32][N*NV] float2
  static constexpr size_t BYTES = U + al16(sizeof(float2) * 4 * 32 * N * NV);
};

template <int FORM, int N, int NV>
__global__ void __launch_bounds__(128) k_residual_affine(ElemArgs a) {
  using R = Ar<float2>;
  using V = DF;
  constexpr int NG = Geo<FORM>::NG, NB = N * N, SL = 32 / N, NL = N * NV;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  using L = ResidualSmem<FORM, N, NV>;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float2 *sS = reinterpret_cast<float2 *>(smem_raw + L::S);
  float2 *sM = reinterpret_cast<float2 *>(smem_raw + L::M);
  float2 *sG = reinterpret_cast<float2 *>(smem_raw + L::G) + warp * 32 * NG;
  uint64_t *sMask = reinterpret_cast<uint64_t *>(smem_raw + L::MASK) + warp * 32;
  float2 *sU = reinterpret_cast<float2 *>(smem_raw + L::U) + warp * 32 * NL;
  for (int i = threadIdx.x; i < 9 * NB; i += blockDim.x) st(sS[i], R::from(a.fe.S[i]));
  for (int i = threadIdx.x; i < NB; i += blockDim.x) st(sM[i], df_split(a.fe.M[i]));
  __syncthreads();
  const int64_t n_tiles = (a.n_list + 31) / 32;
  for (int64_t tile = (int64_t)blockIdx.x * 4 + warp; tile < n_tiles; tile += (int64_t)gridDim.x * 4) {
    const int64_t li = tile * 32 + lane;
    const int32_t e = (li < a.n_list) ? a.list[li] : -1;
    if (e >= 0) {  // lane = element: FP64 geometry at qp 0 (compute_affine_map), u_e, F_e
      const int32_t *c = a.conn + (int64_t)e * a.npe;
      double G[9];
      double det;
      {
        double X[N * 3];
#pragma unroll
        for (int g = 0; g < N; ++g) {
          const double *p = a.xyz + 3 * (int64_t)c[g];
          X[3 * g] = p[0];
          X[3 * g + 1] = p[1];
          X[3 * g + 2] = p[2];
        }
        det = jacobian_affine<N>(X, G);
      }
      if (!(det > 0.0)) report_bad(a, LMG_ERR_DEGENERATE, e);
      const double coef = a.coef ? a.coef[e] : 1.0;
      float2 *g = sG + lane * NG;
      if (FORM == LMG_POISSON) {
        const double s = coef * det;
#pragma unroll
        for (int m = 0; m < 3; ++m)
#pragma unroll
          for (int n = 0; n < 3; ++n)
            st(g[3 * m + n], R::from(s * (G[3 * m] * G[3 * n] + G[3 * m + 1] * G[3 * n + 1] + G[3 * m + 2] * G[3 * n + 2])));
      } else {
        double lam, mu;
        lame(coef, a.nu, lam, mu);
#pragma unroll
        for (int i = 0; i < 9; ++i) st(g[i], R::from(G[i]));
        st(g[9], R::from(lam * det));
        st(g[10], R::from(mu * det));
      }
      const uint64_t mask = a.cmask[e];
      sMask[lane] = mask;
      const int32_t *eb = a.eb + (int64_t)e * N;
      for (int b = 0; b < N; ++b)
#pragma unroll
        for (int v = 0; v < NV; ++v) st(sU[lane * NL + b * NV + v], df_split(a.u[(int64_t)eb[b] * NV + v]));
      // load vector Fe_a^i = detJ sum_b M_ab f_b^i (the element kernel's), into Re2
      float2 *Fo = a.Re2 + (int64_t)e * NL;
      const DF dd = df_split(det);
      element_load_df<N, NV>(a.nodal_f2, c, sM, dd, mask, Fo);
    }
    __syncwarp();
    const int slot = lane / N, ra = lane - slot * N;
    for (int t0 = 0; t0 < 32; t0 += SL) {
      const int t = t0 + slot;
      const int32_t et = __shfl_sync(FULL, e, t < 32 ? t : 0);
      if (slot < SL && t < 32 && et >= 0) {
        const float2 *gt = sG + t * NG;
        V gv[NG];
#pragma unroll
        for (int i = 0; i < NG; ++i) gv[i] = R::ld(gt[i]);
        const uint64_t mask = sMask[t];
        const float2 *ut = sU + t * NL;
        V y[NV];
#pragma unroll
        for (int i = 0; i < NV; ++i) y[i] = R::zero();
#pragma unroll 1  // one copy of the contraction (instruction-cache footprint)
        for (int cb = 0; cb < N; ++cb) {
          V sv[9];
#pragma unroll
          for (int mn = 0; mn < 9; ++mn) sv[mn] = R::ld(sS[mn * NB + ra * N + cb]);
          V out[NV * NV];
          contract_block<FORM, R>(gv, sv, out);
#pragma unroll
          for (int k = 0; k < NV; ++k) {
            if ((mask >> (k * N + cb)) & 1ull) continue;  // constrained column
            const V uk = R::ld(ut[cb * NV + k]);
#pragma unroll
            for (int i = 0; i < NV; ++i) y[i] = df_fma_lazy(y[i], out[i * NV + k], uk);
          }
        }
        float2 *Ro = a.Re2 + (int64_t)et * NL + ra * NV;
#pragma unroll
        for (int i = 0; i < NV; ++i) {
          V r = df_norm(y[i]);
          if ((mask >> (i * N + ra)) & 1ull) r = R::ld(ut[ra * NV + i]);  // row e_a: u_a
          const float2 f = Ro[i];
          r = df_add(r, DF{-f.x, -f.y});
          Ro[i] = make_float2(r.hi, r.lo);
        }
      }
      __syncwarp();
    }
    __syncwarp();
  }
}


template <int FORM, int N, int NV>
void launch_residual_t(const ElemArgs &a, int grid, cudaStream_t s) {
  using L = ResidualSmem<FORM, N, NV>;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_residual_affine<FORM, N, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::BYTES);
    attr = true;
  }
  const int64_t tiles = (a.n_list + 31) / 32, blocks = (tiles + 3) / 4;
  const int g = (int)(blocks < grid ? blocks : grid);
  if (g > 0) k_residual_affine<FORM, N, NV><<<g, 128, L::BYTES, s>>>(a);
}

template <int FORM, int N, int NV, typename T>
__global__ void __launch_bounds__(128) k_elem_general(ElemArgs a) {
  constexpr bool MIXED = sizeof(T) == 4;
  constexpr int NB = N * N, NO = N * (N - 1) / 2, B2 = NV * NV;
  constexpr int BPL = (NB + 31) / 32;
  constexpr int MAXQ = 27;
  __shared__ double sX[4][N * 3];
  __shared__ double sGeo[4][MAXQ][10];  // G (9) and JxW per qp
  __shared__ double sGr[4][N * 3];      // physical gradients at the current qp
  __shared__ double sF[4][N * NV];      // nodal load of the element
  __shared__ double sFq[4][MAXQ * NV];  // the load at every point
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int Q = a.fe.q;
  for (int64_t li = (int64_t)blockIdx.x * 4 + warp; li < a.n_list; li += (int64_t)gridDim.x * 4) {
    const int32_t e = a.list[li];
    const int32_t *c = a.conn + (int64_t)e * a.npe;
    for (int i = lane; i < N * 3; i += 32) sX[warp][i] = a.xyz[3 * (int64_t)c[i / 3] + i % 3];
    for (int i = lane; i < N * NV; i += 32)
      sF[warp][i] = a.nodal_f ? a.nodal_f[(int64_t)c[i / NV] * NV + i % NV] : 0.0;
    __syncwarp();
    const double coef = a.coef ? a.coef[e] : 1.0;
    for (int q = lane; q < Q; q += 32) {
      double G[9];
      const double det = jacobian(sX[warp], a.fe.gdphi + (int64_t)q * N * 3, N, G);
      if (!(det > 0.0)) report_bad(a, LMG_ERR_DEGENERATE, e);
      for (int i = 0; i < 9; ++i) sGeo[warp][q][i] = G[i];
      sGeo[warp][q][9] = det * a.fe.qw[q];
    }
    __syncwarp();
    double lam = 0.0, mu = 0.0;
    if (FORM == LMG_ELASTICITY) lame(coef, a.nu, lam, mu);
    T acc[BPL][B2];
#pragma unroll
    for (int k = 0; k < BPL; ++k)
#pragma unroll
      for (int ik = 0; ik < B2; ++ik) acc[k][ik] = 0;
    for (int q = 0; q < Q; ++q) {
      const double *Gq = sGeo[warp][q];
      for (int i = lane; i < N * 3; i += 32) {
        const int ai = i / 3, d = i - 3 * ai;
        const double *r = a.fe.dphi + ((int64_t)q * N + ai) * 3;
        sGr[warp][i] = r[0] * Gq[d] + r[1] * Gq[3 + d] + r[2] * Gq[6 + d];
      }
      __syncwarp();
      const T jxw = (T)Gq[9];
#pragma unroll
      for (int k = 0; k < BPL; ++k) {
        const int blk = lane + 32 * k;
        if (blk < NB) {
          const int ra = blk / N, cb = blk - ra * N;
          if (ra <= cb) {
            T ga[3], gb[3];
#pragma unroll
            for (int d = 0; d < 3; ++d) { ga[d] = (T)sGr[warp][3 * ra + d]; gb[d] = (T)sGr[warp][3 * cb + d]; }
            const T dot = ga[0] * gb[0] + ga[1] * gb[1] + ga[2] * gb[2];
            if (FORM == LMG_POISSON) {
              acc[k][0] += jxw * (T)coef * dot;
            } else {
#pragma unroll
              for (int i = 0; i < 3; ++i)
#pragma unroll
                for (int kk = 0; kk < 3; ++kk) {
                  T v = (T)lam * ga[i] * gb[kk] + (T)mu * ga[kk] * gb[i];
                  if (i == kk) v += (T)mu * dot;
                  acc[k][3 * i + kk] += jxw * v;
                }
            }
          }
        }
      }

      __syncwarp();
    }
    const uint64_t mask = a.cmask[e];
#pragma unroll
    for (int k = 0; k < BPL; ++k) {
      const int blk = lane + 32 * k;
      if (blk < NB) {
        const int ra = blk / N, cb = blk - ra * N;
        if (ra > cb || (MIXED && ra == cb)) continue;
#pragma unroll
        for (int ik = 0; ik < B2; ++ik) {
          const int i = ik / NV, kk = ik - i * NV;
          if (MIXED) {
            a.Koff32[((int64_t)e * NO + off_index(N, ra, cb)) * B2 + ik] = (float)acc[k][ik];
          } else {
            const DF v = df_split(masked((double)acc[k][ik], mask, i * N + ra, kk * N + cb));
            if (ra == cb) a.Kdiag2[((int64_t)e * N + ra) * B2 + ik] = make_float2(v.hi, v.lo);
            else a.Koff2[((int64_t)e * NO + off_index(N, ra, cb)) * B2 + ik] = make_float2(v.hi, v.lo);
          }
        }
      }
    }
    // load vector in FP64 (element_load: lane (q, v), then lane (a, v))
    element_load<N, NV>(a.fe.phi, sF[warp], &sGeo[warp][0][9], 10, Q, sFq[warp], lane, [&](int ai, int v, double f) {
      const DF s = df_split(((mask >> (v * N + ai)) & 1ull) ? 0.0 : f);
      a.Fe2[((int64_t)e * N + ai) * NV + v] = make_float2(s.hi, s.lo);
    });
  }
}

template <int FORM, int N, int NV, typename T>
void launch_t(bool affine, const ElemArgs &a, int grid, cudaStream_t s) {
  if (a.n_list <= 0) return;
  if (affine) {
    using TA = typename std::conditional<sizeof(T) == 4, float, float2>::type;
    const size_t sm = AffineSmem<FORM, N, NV, TA>::BYTES;
    static bool attr = false;  // set once, before any stream capture of this launch
    if (!attr) {
      cudaFuncSetAttribute(k_elem_affine<FORM, N, NV, TA>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
      attr = true;
    }
    const int64_t tiles = (a.n_list + 31) / 32;
    const int64_t blocks = (tiles + 3) / 4;
    k_elem_affine<FORM, N, NV, TA><<<(int)(blocks < grid ? blocks : grid), 128, sm, s>>>(a);
  } else {
    const int64_t blocks = (a.n_list + 3) / 4;
    k_elem_general<FORM, N, NV, T><<<(int)(blocks < grid ? blocks : grid), 128, 0, s>>>(a);
  }
}


// ---------------------------------------------------------------- fused mixed form
// The mixed form without the element-block buffer: k_geo stores each element's
// FP32 operands (the values the element kernel keeps in shared memory) and its
// double-float load vector; k_rows_mixed then runs one warp per block row P,
// walks the elements touching P in element order (the load-vector plan lists
// them), recomputes the element blocks of P's row with contract_block, and adds
// them in FP32 into a shared-memory row, as the insertion would sum the stored
// blocks.  The epilogue is the mixed insertion's: Dirichlet masking and the
// diagonal rebuilt from double-float row sums.  Same bits as element kernel +
// mixed insertion, without writing and re-reading the blocks.
template <int FORM, int N, int NV>
__global__ void __launch_bounds__(128) k_geo(FusedArgs f) {
  using R = Ar<float>;
  constexpr int NG = Geo<FORM>::NG;
  const ElemArgs &a = f.el;
  __shared__ float2 sM[N * N];  // the mass matrix as double-float pairs, split once per CTA
  for (int i = threadIdx.x; i < N * N; i += blockDim.x) {
    const DF d = df_split(a.fe.M[i]);
    sM[i] = make_float2(d.hi, d.lo);
  }
  __syncthreads();
  for (int64_t li = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; li < a.n_list;
       li += (int64_t)gridDim.x * blockDim.x) {
    const int32_t e = a.list[li];
    const int32_t *c = a.conn + (int64_t)e * a.npe;
    double G[9], det;
    {
      double X[N * 3];
#pragma unroll
      for (int g = 0; g < N; ++g) {
        const double *p = a.xyz + 3 * (int64_t)c[g];
        X[3 * g] = p[0];
        X[3 * g + 1] = p[1];
        X[3 * g + 2] = p[2];
      }
      det = jacobian_affine<N>(X, G);
    }
    if (!(det > 0.0)) report_bad(a, LMG_ERR_DEGENERATE, e);
    const double coef = a.coef ? a.coef[e] : 1.0;
    float *g = f.geo + (int64_t)e * NG;
    if (FORM == LMG_POISSON) {
      const double sc = coef * det;
#pragma unroll
      for (int m = 0; m < 3; ++m)
#pragma unroll
        for (int n = 0; n < 3; ++n)
          g[3 * m + n] = R::from(sc * (G[3 * m] * G[3 * n] + G[3 * m + 1] * G[3 * n + 1] + G[3 * m + 2] * G[3 * n + 2]));
    } else {
      double lam, mu;
      lame(coef, a.nu, lam, mu);
#pragma unroll
      for (int i = 0; i < 9; ++i) g[i] = R::from(G[i]);
      g[9] = R::from(lam * det);
      g[10] = R::from(mu * det);
    }
    // load vector, as the element kernel computes it
    const uint64_t mask = a.cmask[e];
    float2 *Fo = a.Fe2 + (int64_t)e * N * NV;
    const DF dd = df_split(det);
    element_load_df<N, NV>(a.nodal_f2, c, sM, dd, mask, Fo);
  }
}

template <int FORM, int N, int NV>
__global__ void __launch_bounds__(256, 6) k_rows_mixed(FusedArgs f) {
  using R = Ar<float>;
  constexpr int NG = Geo<FORM>::NG, B2 = NV * NV, NPASS = 32 / N, SPL = 32 / B2;
  extern __shared__ __align__(16) float fsm[];
  // reference tensors by block pair: S^{mn}_{ab} at sS[(a N + b) * 12 + mn]
  // (padded to 12 floats: one pair's 9 values are three vector loads)
  float *sS = fsm;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  constexpr int AS = NV == 3 ? 12 : B2;  // floats per slot of the shared-memory row
  float *acc = sS + 12 * N * N + (int64_t)warp * f.max_deg * AS;
  for (int i = threadIdx.x; i < 9 * N * N; i += blockDim.x) {
    const int mn = i / (N * N), ab = i - mn * (N * N);
    sS[ab * 12 + mn] = R::from(f.el.fe.S[i]);
  }
  __syncthreads();
  const int wi = lane / N, bl = lane - wi * N;  // incidence slot and local column node of this lane
  const int js = lane / B2, rem = lane - js * B2;
  const bool act = lane < SPL * B2;
  const int i = rem / NV, k = rem - i * NV;
  for (int64_t P = f.row_begin + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5); P < f.n_brows;
       P += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t rb = f.brow_ptr[P];
    const int deg = (int)(f.brow_ptr[P + 1] - rb);
    const int32_t t0 = f.fptr[P], t1 = f.fptr[P + 1];
    __syncwarp();
    for (int x = lane; x < deg * AS; x += 32) acc[x] = 0.f;
    __syncwarp();
    for (int32_t tg = t0; tg < t1; tg += NPASS) {
      const int32_t t = tg + wi;
      const bool valid = lane < NPASS * N && t < t1;
      const int32_t code = valid ? f.fcontrib[t] : 0;
      const int32_t e = code / N, ae = code - e * N;
      const bool work = valid && bl != ae;
      float out[B2];
      int rel = 0;
      if (work) {
        float gv[NG];
#pragma unroll
        for (int q = 0; q < NG; ++q) gv[q] = f.geo[(int64_t)e * NG + q];
        const int ra = ae < bl ? ae : bl, cb = ae < bl ? bl : ae;
        float sv[9];
        {
          const float4 *s4 = reinterpret_cast<const float4 *>(sS + (ra * N + cb) * 12);
          const float4 x0 = s4[0], x1 = s4[1], x2 = s4[2];
          sv[0] = x0.x; sv[1] = x0.y; sv[2] = x0.z; sv[3] = x0.w;
          sv[4] = x1.x; sv[5] = x1.y; sv[6] = x1.z; sv[7] = x1.w;
          sv[8] = x2.x;
        }
        contract_block<FORM, R>(gv, sv, out);
        if (NV > 1 && bl < ae) {  // the stored block is (b, a): take its transpose
#pragma unroll
          for (int p = 0; p < NV; ++p)
#pragma unroll
            for (int q = p + 1; q < NV; ++q) {
              const float tmp = out[p * NV + q];
              out[p * NV + q] = out[q * NV + p];
              out[q * NV + p] = tmp;
            }
        }
        rel = f.relslot[(int64_t)code * N + bl];
      }
      // element order: the incidences of this pass add one after the other
#pragma unroll
      for (int w = 0; w < NPASS; ++w) {
        if (work && wi == w) {
          if constexpr (NV == 3) {
            // a 3 x 3 block padded to 12 floats: two 16-byte and one 4-byte update
            float4 *a4 = reinterpret_cast<float4 *>(acc + rel * AS);
            float4 x0 = a4[0], x1 = a4[1];
            x0.x = __fadd_rn(x0.x, out[0]);
            x0.y = __fadd_rn(x0.y, out[1]);
            x0.z = __fadd_rn(x0.z, out[2]);
            x0.w = __fadd_rn(x0.w, out[3]);
            x1.x = __fadd_rn(x1.x, out[4]);
            x1.y = __fadd_rn(x1.y, out[5]);
            x1.z = __fadd_rn(x1.z, out[6]);
            x1.w = __fadd_rn(x1.w, out[7]);
            a4[0] = x0;
            a4[1] = x1;
            acc[rel * AS + 8] = __fadd_rn(acc[rel * AS + 8], out[8]);
          } else {
#pragma unroll
            for (int ik = 0; ik < B2; ++ik) acc[rel * AS + ik] = __fadd_rn(acc[rel * AS + ik], out[ik]);
          }
        }
        __syncwarp();
      }
    }
    // epilogue of the mixed insertion, reading the row from shared memory;
    // the Dirichlet flags are read only in rows that touch a constrained dof
    if constexpr (NV == 3) {
      // lane (js3, i3): dof row i3 of the slots js3, js3 + 10, ..., three
      // entries each (written contiguously), with their double-float row sums
      const int js3 = lane / 3, i3 = lane - js3 * 3;
      const bool act3 = lane < 30;
      // dof row 3 P + i3 of the block CSR starts at 9 brow_ptr[P] + 3 i3 deg
      const int32_t rowp = act3 ? (int32_t)(9 * rb + (int64_t)3 * i3 * deg) : 0;
      const bool rc = act3 && f.constrained[3 * P + i3] != 0;
      float rh[3] = {0.f, 0.f, 0.f}, rl[3] = {0.f, 0.f, 0.f};
      int jdiag = -1;
      auto epilogue = [&](auto masks) {
        for (int jj = js3; act3 && jj < deg; jj += 10) {
          const int32_t Q = f.bcol[rb + jj];
          if (Q == (int32_t)P) { jdiag = jj; continue; }
          const float *ar = acc + jj * AS + i3 * 3;
          double *Kr = f.K + rowp + jj * 3;
#pragma unroll
          for (int kk = 0; kk < 3; ++kk) {
            const float kv = ar[kk];
            const float s = __fadd_rn(rh[kk], kv), bb = __fsub_rn(s, rh[kk]);
            rl[kk] = __fadd_rn(rl[kk], __fadd_rn(__fsub_rn(rh[kk], __fsub_rn(s, bb)), __fsub_rn(kv, bb)));
            rh[kk] = s;
            bool msk = false;
            if constexpr (decltype(masks)::value) msk = rc || f.constrained[(int64_t)3 * Q + kk] != 0;
            Kr[kk] = msk ? 0.0 : f2d(kv);
          }
        }
      };
      if (f.rowcons[P]) epilogue(std::true_type{});
      else epilogue(std::false_type{});
      DF r[3];
#pragma unroll
      for (int kk = 0; kk < 3; ++kk) r[kk] = fast_two_sum(rh[kk], rl[kk]);
      // sum over js3 = 0..9 (lanes i3 + 3 js3): pairs, then fours, then eights
#pragma unroll
      for (int d = 1; d < 10; d <<= 1)
#pragma unroll
        for (int kk = 0; kk < 3; ++kk) {
          DF y;
          y.hi = __shfl_sync(0xffffffffu, r[kk].hi, (lane + 3 * d) & 31);
          y.lo = __shfl_sync(0xffffffffu, r[kk].lo, (lane + 3 * d) & 31);
          if (act3 && js3 % (2 * d) == 0 && js3 + d < 10) r[kk] = df_add(r[kk], y);
        }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) jdiag = max(jdiag, __shfl_xor_sync(0xffffffffu, jdiag, o));
      if (lane < 3 && jdiag >= 0) {
#pragma unroll
        for (int kk = 0; kk < 3; ++kk) {
          double v = -(f2d(r[kk].hi) + f2d(r[kk].lo));
          if (rc || f.constrained[3 * P + kk] != 0) v = (i3 == kk) ? (double)(t1 - t0) : 0.0;
          f.K[rowp + jdiag * 3 + kk] = v;
        }
      }
    } else {
      const int32_t rowp = act ? (int32_t)(NV * NV * rb + (int64_t)NV * i * deg) : 0;
      const bool rc = act && f.constrained[NV * P + i] != 0;
      float rh = 0.f, rl = 0.f;  // double-float row sum, normalised after the loop
      int jdiag = -1;
      auto epilogue = [&](auto masks) {
        for (int jj = js; act && jj < deg; jj += SPL) {
          const int32_t Q = f.bcol[rb + jj];
          if (Q == (int32_t)P) { jdiag = jj; continue; }
          const float kv = acc[jj * AS + rem];
          const float s = __fadd_rn(rh, kv), bb = __fsub_rn(s, rh);
          rl = __fadd_rn(rl, __fadd_rn(__fsub_rn(rh, __fsub_rn(s, bb)), __fsub_rn(kv, bb)));
          rh = s;
          bool msk = false;
          if constexpr (decltype(masks)::value) msk = rc || f.constrained[(int64_t)NV * Q + k] != 0;
          f.K[rowp + jj * NV + k] = msk ? 0.0 : f2d(kv);
        }
      };
      if (f.rowcons[P]) epilogue(std::true_type{});
      else epilogue(std::false_type{});
      DF racc = fast_two_sum(rh, rl);
      if constexpr (B2 == 1) {
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          DF y;
          y.hi = __shfl_xor_sync(0xffffffffu, racc.hi, o);
          y.lo = __shfl_xor_sync(0xffffffffu, racc.lo, o);
          racc = (lane & o) ? df_add(y, racc) : df_add(racc, y);
        }
      } else {
#pragma unroll
        for (int t = 1; t < SPL; ++t) {
          DF y;
          y.hi = __shfl_sync(0xffffffffu, racc.hi, (lane + t * B2) & 31);
          y.lo = __shfl_sync(0xffffffffu, racc.lo, (lane + t * B2) & 31);
          if (lane < B2) racc = df_add(racc, y);
        }
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) jdiag = max(jdiag, __shfl_xor_sync(0xffffffffu, jdiag, o));
      if (lane < B2 && jdiag >= 0) {
        double v = -(f2d(racc.hi) + f2d(racc.lo));
        if (rc || f.constrained[NV * P + k] != 0) v = (i == k) ? (double)(t1 - t0) : 0.0;
        f.K[rowp + jdiag * NV + k] = v;
      }
    }
  }
}

template <int FORM, int N, int NV>
void launch_fused_t(const FusedArgs &f, int grid, cudaStream_t s, bool geo, bool rows) {
  const int64_t gb = (f.el.n_list + 127) / 128;
  if (geo && gb > 0) k_geo<FORM, N, NV><<<(int)(gb < grid ? gb : grid), 128, 0, s>>>(f);
  if (!rows) return;
  const size_t smem = sizeof(float) * (12 * N * N + (size_t)8 * f.max_deg * (NV == 3 ? 12 : NV * NV));
  static size_t attr = 0;
  if (smem > attr) {
    cudaFuncSetAttribute(k_rows_mixed<FORM, N, NV>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = smem;
  }
  const int64_t rb = (f.n_brows - f.row_begin + 7) / 8;
  if (rb > 0) k_rows_mixed<FORM, N, NV><<<(int)(rb < grid ? rb : grid), 256, smem, s>>>(f);
  launch_load_vec(NV, f.row_begin, f.n_brows, f.fptr, f.fcontrib, f.el.Fe2, f.F, s);
}

}  // namespace

bool elements_built(int form, int n, int nv) {
  return (form == LMG_POISSON && nv == 1 && (n == 4 || n == 6 || n == 8 || n == 10 || n == 27)) ||
         (form == LMG_ELASTICITY && nv == 3 && (n == 4 || n == 6 || n == 8 || n == 10));
}

bool fused_built(int form, int n, int nv) {
  return (form == LMG_POISSON && nv == 1 && (n == 4 || n == 6 || n == 8 || n == 10 || n == 27)) ||
         (form == LMG_ELASTICITY && nv == 3 && (n == 4 || n == 6 || n == 8 || n == 10));
}

bool fused_fits(int n, int nv, int max_deg) {
  return sizeof(float) * (12 * (size_t)n * n + (size_t)8 * max_deg * (nv == 3 ? 12 : nv * nv)) <= (size_t)200 * 1024;
}

bool launch_fused_mixed(int form, int n, int nv, const FusedArgs &f, int grid, cudaStream_t s, bool geo,
                        bool rows) {
#define LMG_F(F, NN, V)                               \
  if (form == F && n == NN && nv == V) {              \
    launch_fused_t<F, NN, V>(f, grid, s, geo, rows);  \
    return true;                                      \
  }
  LMG_F(LMG_POISSON, 4, 1)
  LMG_F(LMG_POISSON, 6, 1)
  LMG_F(LMG_POISSON, 8, 1)
  LMG_F(LMG_POISSON, 10, 1)
  LMG_F(LMG_POISSON, 27, 1)
  LMG_F(LMG_ELASTICITY, 4, 3)
  LMG_F(LMG_ELASTICITY, 6, 3)
  LMG_F(LMG_ELASTICITY, 8, 3)
  LMG_F(LMG_ELASTICITY, 10, 3)
#undef LMG_F
  return false;
}

bool launch_residual(int form, int n, int nv, const ElemArgs &a, int64_t n_brows, const int32_t *fptr,
                     const int32_t *fcontrib, double *R, int grid, cudaStream_t s) {
#define LMG_R(F, NN, V)                                   \
  if (form == F && n == NN && nv == V) {                  \
    launch_residual_t<F, NN, V>(a, grid, s);              \
    ok = true;                                            \
  }
  bool ok = false;
  LMG_R(LMG_POISSON, 4, 1)
  LMG_R(LMG_POISSON, 6, 1)
  LMG_R(LMG_POISSON, 8, 1)
  LMG_R(LMG_POISSON, 10, 1)
  LMG_R(LMG_POISSON, 27, 1)
  LMG_R(LMG_ELASTICITY, 4, 3)
  LMG_R(LMG_ELASTICITY, 6, 3)
  LMG_R(LMG_ELASTICITY, 8, 3)
  LMG_R(LMG_ELASTICITY, 10, 3)
#undef LMG_R
  if (!ok) return false;
  (void)grid;
  launch_load_vec(nv, 0, n_brows, fptr, fcontrib, a.Re2, R, s);  // per-dof sums in element order
  return true;
}

void launch_elements(int form, int n, int nv, bool affine, bool mixed, const ElemArgs &a, int grid,
                     cudaStream_t s) {
#define LMG_CASE(F, NN, V)                                                      \
  if (form == F && n == NN && nv == V) {                                        \
    if (mixed) launch_t<F, NN, V, float>(affine, a, grid, s);                   \
    else launch_t<F, NN, V, double>(affine, a, grid, s);                        \
    return;                                                                     \
  }
  LMG_CASE(LMG_POISSON, 4, 1)
  LMG_CASE(LMG_POISSON, 6, 1)
  LMG_CASE(LMG_POISSON, 8, 1)
  LMG_CASE(LMG_POISSON, 10, 1)
  LMG_CASE(LMG_POISSON, 27, 1)
  LMG_CASE(LMG_ELASTICITY, 4, 3)
  LMG_CASE(LMG_ELASTICITY, 6, 3)
  LMG_CASE(LMG_ELASTICITY, 8, 3)
  LMG_CASE(LMG_ELASTICITY, 10, 3)
#undef LMG_CASE
}

}  // namespace lmg
