// Mixed-form element matrices on the 5th-generation tensor cores (tcgen05).
//
// The reference assembles every element with the per-quadrature-point form
// (systems_of_equations_ex6.C:222-230, introduction_ex4.C:467):
//   Ke_var[i][k](a,b) += JxW C_ijkl dphi_b(l) dphi_a(j),  C_ijkl = lam d_ij d_kl + mu (d_ik d_jl + d_il d_jk),
//   Ke(a,b)           += JxW k dphi_a . dphi_b.
// Both are Gram matrices: Ke = E^T E with R rows of E per quadrature point and
// one column per element dof u = (i, a) (variable-blocked, u = i N + a):
//   elasticity (R = 7): sqrt(lam JxW) d_i phi_a (divergence), sqrt(2 mu JxW)
//     d_ij d_j phi_a for j = 0..2 (normal strains), sqrt(mu JxW) (d_j phi_a d_il
//     + d_l phi_a d_ij) for (j, l) = (0,1), (0,2), (1,2) (shear strains);
//   Poisson (R = 3): sqrt(k JxW) d_j phi_a.
// Summed over the R rows this is exactly the reference's integrand, so Ke =
// E^T S E is one GEMM per element with K = Q R (77 for TET10 with Keast's 11
// points), S = diag(sign w_q) on each point's rows: a rule with a negative
// weight at its first point (Keast's centre point, -0.01315...) enters with
// sqrt(|w_q| detJ), and the first 16-wide K slab of the B operand, which holds
// that point's rows, is a separate copy with those rows negated.  That is what runs here, for the elements the reference-tensor
// shortcut does not cover (non-affine maps, libMesh's compute_map branch).
//
// A CTA (4 warps) takes 4 elements per tile; their connectivity rows arrive
// in shared memory by one bulk asynchronous copy (cp.async.bulk, completing
// on an mbarrier) when the four are consecutive ids.  Warp w builds element w's E:
// the Jacobian, detJ and J^-1 at every point in FP64 (compute_single_point_map,
// fe_map.C:980-1078), the scale factors in FP64, the physical gradients and E
// in FP32; every entry is split into three BF16 pieces (hi + mid + lo carry
// the FP32 value exactly) stored as rows 32 w + u of three K-major tiles in
// shared memory (the canonical no-swizzle layout: 8-row x 16-byte core
// matrices).  One thread issues the tile's MMAs: D = sum over the six piece
// products (hi hi, hi mid, mid hi, hi lo, mid mid, lo hi) of A_i A_j^T, M = N =
// 128, K = 16 per instruction, FP32 accumulation in tensor memory.  Rows and
// columns 32 w .. 32 w + 31 of D are element w's Ke (the off-diagonal 32 x 32
// blocks pair different elements and are not read).  tcgen05.commit signals an
// mbarrier; after a bounded wait warp w reads its block with tcgen05.ld
// (32x32b, lane u = row u) and writes the strictly upper 3x3 blocks of Ke to
// the mixed form's element-block buffer (the insertion rebuilds the diagonal
// blocks from the row sums).  The load vector is the FP64 path's, bit for bit.
//
// Every wait is bounded: on timeout the kernel records LMG_ERR_CUDA in the
// status word and stops.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "assemble.cuh"
#include "bulk_copy.cuh"
#include "df.cuh"
#include "elem_geom.cuh"
#include "../../include/libmesh_gb300.h"

namespace lmg {

namespace {

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return smem_addr(p); }

// Shared-memory matrix descriptor of a K-major tile without swizzling:
// start address, leading byte offset (between core matrices adjacent in K),
// stride byte offset (between 8-row groups), descriptor version 1.
__device__ __forceinline__ uint64_t umma_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr >> 4) & 0x3fffu) | ((uint64_t)((lbo >> 4) & 0x3fffu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3fffu) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both
// K-major, N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t IDESC_BF16_M128_N128 = (1u << 4) | (1u << 7) | (1u << 10) | (16u << 17) | (8u << 24);

template <int FORM, int N, int NV, int Q>
struct TcShape {
  static constexpr int R = FORM == LMG_ELASTICITY ? 7 : 3;  // rows of E per quadrature point
  static constexpr int NCOL = N * NV;                        // element dofs (columns of E)
  static constexpr int KD = ((Q * R + 15) / 16) * 16;        // K extent, a multiple of the MMA's 16
  static constexpr int KG = KD / 8;                          // core matrices along K
  static constexpr int NO = N * (N - 1) / 2, B2 = NV * NV;
  static constexpr size_t PIECE = (size_t)128 * KD * 2;      // one 128 x KD BF16 tile
  static constexpr size_t SLAB = (size_t)128 * 16 * 2;       // one 128 x 16 BF16 slab (one K step)
  static_assert(R <= 16, "the first point's rows fit the first K step");
  // dynamic shared memory: the three pieces of E, then (signed rules) the
  // three signed slabs of the first K step, then the tables and per-warp data;
  // npc = 3 or 6 (with the slabs)
  __host__ __device__ static size_t dphi(int npc) { return 3 * PIECE + (npc > 3 ? 3 * SLAB : 0); }  // [Q][N][3] float
  __host__ __device__ static size_t phi(int npc) { return (dphi(npc) + sizeof(float) * Q * N * 3 + 15) & ~(size_t)15; }  // [Q][N] double
  __host__ __device__ static size_t warp0(int npc) { return phi(npc) + sizeof(double) * Q * N; }
  // per warp: X [N][3] double, f [N][NV] double, JxW [Q] double, load at the points [Q][NV] double,
  // G [Q][9] float, scales and sign [Q][4] float
  static constexpr size_t PER_WARP =
      ((sizeof(double) * (N * 3 + N * NV + Q + Q * NV) + sizeof(float) * Q * 13) + 15) & ~(size_t)15;
  // at least 60 KB, so that no more than three CTAs share an SM and their
  // accumulators (128 tensor-memory columns each) fit the SM's 512 columns
  __host__ __device__ static size_t bytes(int npc) {
    const size_t b = warp0(npc) + 4 * PER_WARP;
    return b > 61440 ? b : 61440;
  }
  static_assert(NCOL <= 32, "one warp lane per element dof");
  static_assert(PIECE % 1024 == 0, "tiles keep the 1 KB alignment");
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat16 a = __float2bfloat16_rn(lo), b = __float2bfloat16_rn(hi);
  return (uint32_t)__bfloat16_as_ushort(a) | ((uint32_t)__bfloat16_as_ushort(b) << 16);
}

// is_signed: the rule's first point has a negative weight (and no other
// point has); the B operand's first K step then reads the signed slabs.
template <int FORM, int N, int NV, int Q>
__global__ void __launch_bounds__(128) k_elem_tc(ElemArgs a, int is_signed) {
  using S = TcShape<FORM, N, NV, Q>;
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ __align__(8) uint64_t mbar, mbar_tma;
  __shared__ __align__(16) int32_t sConn[4 * N];  // connectivity rows of the tile's elements
  __shared__ int tile_bulk;
  __shared__ uint32_t tmem_base;
  const int t = threadIdx.x, w = t >> 5, lane = t & 31;
  const int npc = is_signed ? 6 : 3;
  float *sdphi = reinterpret_cast<float *>(tsm + S::dphi(npc));
  double *sphi = reinterpret_cast<double *>(tsm + S::phi(npc));
  unsigned char *wb = tsm + S::warp0(npc) + S::PER_WARP * w;
  double *sX = reinterpret_cast<double *>(wb);
  double *sF = sX + N * 3;
  double *sJxW = sF + N * NV;
  double *sFq = sJxW + Q;
  float *sG = reinterpret_cast<float *>(sFq + Q * NV);
  float *sSc = sG + Q * 9;  // [Q][4]: row scales and the sign of the weight
  for (int i = t; i < Q * N * 3; i += blockDim.x) sdphi[i] = (float)a.fe.dphi[i];
  for (int i = t; i < Q * N; i += blockDim.x) sphi[i] = a.fe.phi[i];
  for (size_t i = t; i < S::dphi(npc) / 16; i += blockDim.x) reinterpret_cast<uint4 *>(tsm)[i] = make_uint4(0, 0, 0, 0);
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                 "r"(128));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (t == 0) {
    mbar_init(&mbar, 1);
    mbar_init(&mbar_tma, 1);
    mbar_fence_init();
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = tmem_base;
  uint32_t phase = 0, phase_tma = 0;
  const int64_t n_tiles = (a.n_list + 3) / 4;
  for (int64_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
    const int64_t li = tile * 4 + w;
    const int32_t e = li < a.n_list ? a.list[li] : -1;
    // Connectivity of the tile: when its four elements are consecutive ids
    // with 16-byte aligned rows (a mesh whose elements all take this kernel),
    // one bulk asynchronous copy (TMA) into shared memory; otherwise each
    // warp loads its element's row.
    if (t == 0) {
      const int64_t l0 = tile * 4;
      int bulk = l0 + 3 < a.n_list && a.npe == N;
      const int32_t e0 = bulk ? a.list[l0] : 0;
      for (int j = 1; bulk && j < 4; ++j) bulk = a.list[l0 + j] == e0 + j;
      const uint64_t src = (uint64_t)(a.conn + (int64_t)e0 * N);
      bulk = bulk && (src % 16 == 0) && ((4 * N * sizeof(int32_t)) % 16 == 0);
      tile_bulk = bulk;
      if (bulk) {
        mbar_expect_tx(&mbar_tma, (uint32_t)(4 * N * sizeof(int32_t)));
        bulk_g2s(sConn, (const void *)src, (uint32_t)(4 * N * sizeof(int32_t)), &mbar_tma);
      }
    }
    __syncthreads();
    if (tile_bulk) {
      const uint32_t got = mbar_wait(&mbar_tma, phase_tma, 1 << 24) ? 1u : 0u;
      phase_tma ^= 1u;
      if (!__syncthreads_and((int)got)) {
        if (t == 0) atomicCAS(a.status, 0, LMG_ERR_CUDA);
        break;
      }
    } else if (e >= 0) {
      for (int i = lane; i < N; i += 32) sConn[w * N + i] = a.conn[(int64_t)e * a.npe + i];
    }
    __syncwarp();
    if (e >= 0) {
      const int32_t *c = sConn + w * N;
      for (int i = lane; i < N * 3; i += 32) sX[i] = a.xyz[3 * (int64_t)c[i / 3] + i % 3];
      for (int i = lane; i < N * NV; i += 32) sF[i] = a.nodal_f ? a.nodal_f[(int64_t)c[i / NV] * NV + i % NV] : 0.0;
    }
    __syncwarp();
    if (e >= 0) {
      // FP64 map at every point; FP64 scale factors of E's rows
      const double coef = a.coef ? a.coef[e] : 1.0;
      double lam = 0.0, mu = 0.0;
      if (FORM == LMG_ELASTICITY) lame(coef, a.nu, lam, mu);
      for (int q = lane; q < Q; q += 32) {
        double G[9];
        const double det = jacobian(sX, a.fe.gdphi + (int64_t)q * N * 3, N, G);
        if (!(det > 0.0)) {
          atomicCAS(a.status, 0, LMG_ERR_DEGENERATE);
          atomicMin(a.bad_elem, (unsigned long long)e);
        }
        const double jxw = det * a.fe.qw[q];
        sJxW[q] = jxw;
#pragma unroll
        for (int i = 0; i < 9; ++i) sG[q * 9 + i] = (float)G[i];
        const double aj = fabs(jxw);  // detJ > 0: the sign is the weight's
        if (FORM == LMG_ELASTICITY) {
          sSc[q * 4 + 0] = (float)sqrt(lam * aj);
          sSc[q * 4 + 1] = (float)sqrt(2.0 * mu * aj);
          sSc[q * 4 + 2] = (float)sqrt(mu * aj);
        } else {
          sSc[q * 4] = (float)sqrt(coef * aj);
        }
        sSc[q * 4 + 3] = jxw < 0.0 ? -1.f : 1.f;
      }
    }
    __syncwarp();
    // column u of E (lane u), split into three BF16 pieces, stored as row
    // 32 w + u of the three tiles, 8 K-values (one core-matrix row) at a time
    if (e >= 0 && lane < S::NCOL) {
      const int i = lane / N, aa = lane - i * N, row = 32 * w + lane;
      float col[S::KD];
#pragma unroll
      for (int k = 0; k < S::KD; ++k) col[k] = 0.f;
#pragma unroll
      for (int q = 0; q < Q; ++q) {
        const float *dh = sdphi + (q * N + aa) * 3, *G = sG + q * 9;
        float g[3];
#pragma unroll
        for (int j = 0; j < 3; ++j) g[j] = fmaf(dh[0], G[j], fmaf(dh[1], G[3 + j], dh[2] * G[6 + j]));
        if (FORM == LMG_ELASTICITY) {
          const float sl = sSc[q * 4], sd = sSc[q * 4 + 1], so = sSc[q * 4 + 2];
          float *r = col + q * 7;
          r[0] = sl * g[i];
          r[1] = i == 0 ? sd * g[0] : 0.f;
          r[2] = i == 1 ? sd * g[1] : 0.f;
          r[3] = i == 2 ? sd * g[2] : 0.f;
          r[4] = i == 0 ? so * g[1] : (i == 1 ? so * g[0] : 0.f);
          r[5] = i == 0 ? so * g[2] : (i == 2 ? so * g[0] : 0.f);
          r[6] = i == 1 ? so * g[2] : (i == 2 ? so * g[1] : 0.f);
        } else {
          const float s = sSc[q * 4];
          col[q * 3] = s * g[0];
          col[q * 3 + 1] = s * g[1];
          col[q * 3 + 2] = s * g[2];
        }
      }
      const size_t roff = (size_t)(row >> 3) * S::KG * 128 + (size_t)(row & 7) * 16;
#pragma unroll
      for (int kg = 0; kg < S::KG; ++kg) {
        uint32_t p[3][4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
          float x[2], m[2], l[2];
#pragma unroll
          for (int s2 = 0; s2 < 2; ++s2) {
            const float v = col[kg * 8 + 2 * h + s2];
            const float v0 = __bfloat162float(__float2bfloat16_rn(v));
            const float v1 = __bfloat162float(__float2bfloat16_rn(v - v0));
            x[s2] = v0;
            m[s2] = v1;
            l[s2] = (v - v0) - v1;
          }
          p[0][h] = pack_bf16(x[0], x[1]);
          p[1][h] = pack_bf16(m[0], m[1]);
          p[2][h] = pack_bf16(l[0], l[1]);
        }
#pragma unroll
        for (int pc = 0; pc < 3; ++pc)
          *reinterpret_cast<uint4 *>(tsm + pc * S::PIECE + roff + (size_t)kg * 128) =
              make_uint4(p[pc][0], p[pc][1], p[pc][2], p[pc][3]);
        if (is_signed && kg < 2) {  // B's first K step: sign bit flipped on the first point's rows (k < R)
          uint32_t neg[4];
#pragma unroll
          for (int h = 0; h < 4; ++h) {
            const int k0 = kg * 8 + 2 * h;
            neg[h] = (k0 < S::R ? 0x8000u : 0u) | (k0 + 1 < S::R ? 0x80000000u : 0u);
          }
          const size_t soff = (size_t)(row >> 3) * 256 + (size_t)(row & 7) * 16 + (size_t)kg * 128;
#pragma unroll
          for (int pc = 0; pc < 3; ++pc)
            *reinterpret_cast<uint4 *>(tsm + 3 * S::PIECE + pc * S::SLAB + soff) =
                make_uint4(p[pc][0] ^ neg[0], p[pc][1] ^ neg[1], p[pc][2] ^ neg[2], p[pc][3] ^ neg[3]);
        }
      }
    }
    // load vector, FP64, exactly as the FP64 path forms it
    if (e >= 0) {
      const uint64_t mask = a.cmask[e];
      element_load<N, NV>(sphi, sF, sJxW, 1, Q, sFq, lane, [&](int ai, int v, double f) {
        const DF s = df_split(((mask >> (v * N + ai)) & 1ull) ? 0.0 : f);
        a.Fe2[((int64_t)e * N + ai) * NV + v] = make_float2(s.hi, s.lo);
      });
    }
    // the tile's MMAs: generic-proxy stores made visible to the tensor core
    asm volatile("fence.proxy.async.shared::cta;");
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;");
    if (t == 0) {
      const uint32_t base = smem_u32(tsm);
      const uint32_t sbo = S::KG * 128;
      constexpr int PA[6] = {0, 0, 1, 0, 1, 2}, PB[6] = {0, 1, 0, 2, 1, 0};
#pragma unroll 1
      for (int ks = 0; ks < S::KD / 16; ++ks)
#pragma unroll
        for (int pr = 0; pr < 6; ++pr) {
          const uint64_t da = umma_desc(base + PA[pr] * (uint32_t)S::PIECE + ks * 256, 128, sbo);
          const uint64_t db =
              (is_signed && ks == 0) ? umma_desc(base + 3 * (uint32_t)S::PIECE + PB[pr] * (uint32_t)S::SLAB, 128, 256)
                                     : umma_desc(base + PB[pr] * (uint32_t)S::PIECE + ks * 256, 128, sbo);
          const uint32_t acc = (ks > 0 || pr > 0) ? 1u : 0u;
          asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                       " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                       "l"(da), "l"(db), "r"(IDESC_BF16_M128_N128), "r"(acc));
        }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(&mbar)));
    }
    const uint32_t done = mbar_wait(&mbar, phase, 1 << 24) ? 1u : 0u;
    phase ^= 1u;
    if (!__syncthreads_and((int)done)) {
      if (t == 0) atomicCAS(a.status, 0, LMG_ERR_CUDA);
      break;
    }
    asm volatile("tcgen05.fence::after_thread_sync;");
    // warp w: rows / columns 32 w .. 32 w + 31 of D (lane u holds row u)
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(tmem + ((uint32_t)(32 * w) << 16) + (uint32_t)(32 * w)));
    asm volatile("tcgen05.wait::ld.sync.aligned;");
    if (e >= 0 && lane < S::NCOL) {  // strictly upper 3x3 blocks (a < b) of Ke, entry (i, k)
      const int i = lane / N, aa = lane - i * N;
      for (int b = aa + 1; b < N; ++b) {
        const int o = aa * N - aa * (aa + 1) / 2 + (b - aa - 1);
        float *dst = a.Koff32 + ((int64_t)e * S::NO + o) * S::B2 + i * NV;
#pragma unroll
        for (int k = 0; k < NV; ++k) dst[k] = __uint_as_float(r[k * N + b]);
      }
    }
    asm volatile("tcgen05.fence::before_thread_sync;");
    __syncthreads();  // the next tile overwrites the tiles and the accumulator
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(128));
}

template <int FORM, int N, int NV, int Q>
void launch_tc_t(const ElemArgs &a, bool is_signed, int n_sm, cudaStream_t s) {
  using S = TcShape<FORM, N, NV, Q>;
  const size_t bytes = S::bytes(is_signed ? 6 : 3);
  static size_t attr = 0;  // largest dynamic shared memory granted so far
  if (bytes > attr) {
    cudaFuncSetAttribute(k_elem_tc<FORM, N, NV, Q>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    attr = bytes;
  }
  const int64_t tiles = (a.n_list + 3) / 4;
  const int64_t cap = (int64_t)n_sm * 3;  // at most three CTAs per SM (shared memory and tensor memory)
  const int g = (int)(tiles < cap ? tiles : cap);
  if (g > 0) k_elem_tc<FORM, N, NV, Q><<<g, 128, bytes, s>>>(a, is_signed ? 1 : 0);
}

}  // namespace

bool tc_built(int form, int n, int nv, int q) {
  return (form == LMG_ELASTICITY && n == 10 && nv == 3 && q == 11) ||
         (form == LMG_ELASTICITY && n == 4 && nv == 3 && q == 4) ||
         (form == LMG_POISSON && n == 10 && nv == 1 && q == 11) ||
         (form == LMG_POISSON && n == 8 && nv == 1 && q == 8);
}

bool launch_elements_tc(int form, int n, int nv, int q, bool neg_weights, const ElemArgs &a, int n_sm,
                        cudaStream_t s) {
  if (a.n_list <= 0) return true;
#define LMG_TC(F, NN, V, QQ)                              \
  if (form == F && n == NN && nv == V && q == QQ) {       \
    launch_tc_t<F, NN, V, QQ>(a, neg_weights, n_sm, s);   \
    return true;                                          \
  }
  LMG_TC(LMG_ELASTICITY, 10, 3, 11)
  LMG_TC(LMG_ELASTICITY, 4, 3, 4)
  LMG_TC(LMG_POISSON, 10, 1, 11)
  LMG_TC(LMG_POISSON, 8, 1, 8)
#undef LMG_TC
  return false;
}

}  // namespace lmg
