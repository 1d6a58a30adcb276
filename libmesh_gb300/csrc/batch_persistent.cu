// Persistent batched assembly: every system of a batch in one kernel launch.
//
// libMesh assembles each system through its own System::assemble
// (src/systems/system.C:554-561).  Here the CTAs of one persistent launch pull
// work items from a global queue (one atomicAdd per item): first the element
// tiles of every member (a tile: up to TILE elements of one orientation
// pattern, the per-pattern kernel's work, dispatched on the member's dofs and
// map nodes), then ranges of PB_SLOTS CSR slots of every member's insertion
// (each slot's contributions summed in element order, as k_gather_full sums
// them).  A CTA that takes an insertion range waits for its member's element
// tiles to be done: a counter per member, raised after each tile with a
// device-scope fence.  Every element tile is in the queue before any
// insertion range, so a waited-for tile has already been taken by a running
// CTA and the wait ends; it is bounded all the same (after 2^26 polls the
// status word gets LMG_ERR_CUDA).  Small and large systems, hexes, tets and
// prisms of any order share the GPU without a launch per system.
#include <cuda_runtime.h>

#include "batch_persistent.cuh"
#include "context_internal.cuh"

namespace lmg {

namespace {

constexpr int GMAX = 27;

template <bool MIXED, int TILE>
__device__ __forceinline__ void element_tile(const PMember &m, int64_t bi, unsigned char *sbuf) {
#define LMG_PT(NN, GG)                                                                       \
  if (m.N == NN && m.G == GG) {                                                              \
    pattern_tile<NN, GG, MIXED, TILE>(m.el, bi, *reinterpret_cast<PatSmem<GG, TILE> *>(sbuf)); \
    return;                                                                                  \
  }
  LMG_PT(8, 8)     // HEX8 p1
  LMG_PT(27, 27)   // HEX27 p2
  LMG_PT(4, 4)     // TET4 p1
  LMG_PT(10, 10)   // TET10 p2
  LMG_PT(6, 6)     // PRISM6 p1
  LMG_PT(64, 27)   // HEX27 p3
  LMG_PT(20, 14)   // TET14 p3
  LMG_PT(18, 6)    // PRISM18 p2
  LMG_PT(40, 6)    // PRISM21 p3
#undef LMG_PT
}

template <typename T>
__device__ __forceinline__ void insertion_range(const PMember &m, int64_t item) {
  const int64_t n = m.nnz + m.n_dofs;
  const int64_t s1 = (item + 1) * PB_SLOTS < n ? (item + 1) * PB_SLOTS : n;
  const T *E = static_cast<const T *>(m.el.Kraw);
  for (int64_t s = item * PB_SLOTS + threadIdx.x; s < s1; s += H3T) {
    if (s < m.nnz) {
      if constexpr (sizeof(T) == 4) {  // FP32 entries summed in double-float
        float hi = 0.f, lo = 0.f;
        for (int64_t t = m.cptr[s]; t < m.cptr[s + 1]; ++t) {
          const float x = __ldcg(E + m.coff[t]);
          const float sum = __fadd_rn(hi, x), bb = __fsub_rn(sum, hi);
          lo = __fadd_rn(lo, __fadd_rn(__fsub_rn(hi, __fsub_rn(sum, bb)), __fsub_rn(x, bb)));
          hi = sum;
        }
        m.K[s] = (double)hi + (double)lo;
      } else {
        double v = 0.0;
        for (int64_t t = m.cptr[s]; t < m.cptr[s + 1]; ++t) v += (double)__ldcg(E + m.coff[t]);
        m.K[s] = v;
      }
    } else {
      const int64_t d = s - m.nnz;
      double v = 0.0;
      for (int64_t t = m.fptr[d]; t < m.fptr[d + 1]; ++t) v += __ldcg(m.el.Fraw + m.foff[t]);
      m.F[d] = v;
    }
  }
}

template <bool MIXED, int TILE>
__global__ void __launch_bounds__(H3T) k_batch_persistent(const PMember *__restrict__ mem,
                                                          const PItem *__restrict__ items, int64_t n_items,
                                                          unsigned long long *head, unsigned int *done,
                                                          int *status) {
  __shared__ __align__(16) unsigned char sbuf[sizeof(PatSmem<GMAX, TILE>)];
  __shared__ int64_t s_item;
  for (;;) {
    if (threadIdx.x == 0) s_item = (int64_t)atomicAdd(head, 1ull);
    __syncthreads();
    const int64_t it = s_item;
    __syncthreads();  // every thread has the item before thread 0 takes the next
    if (it >= n_items) break;
    const PItem w = items[it];
    const PMember &m = mem[w.member];
    if (w.kind == 0) {
      element_tile<MIXED, TILE>(m, w.local, sbuf);
      __threadfence();  // this thread's element entries before the member's count
      __syncthreads();
      if (threadIdx.x == 0) atomicAdd(&done[w.member], 1u);
    } else {
      if (threadIdx.x == 0) {
        bool ready = false;
        for (int poll = 0; poll < (1 << 26) && !ready; ++poll) {
          ready = atomicAdd(&done[w.member], 0u) >= (unsigned int)m.n_tiles;
          if (!ready) __nanosleep(128);
        }
        if (!ready) atomicCAS(status, 0, (int)LMG_ERR_CUDA);
        __threadfence();
      }
      __syncthreads();
      if (MIXED) insertion_range<float>(m, w.local);
      else insertion_range<double>(m, w.local);
    }
  }
}

template <bool MIXED, int TILE>
void launch_t(const PMember *mem, const PItem *items, int64_t n_items, unsigned long long *head, unsigned int *done,
              int *status, int grid, cudaStream_t s) {
  k_batch_persistent<MIXED, TILE><<<grid, H3T, 0, s>>>(mem, items, n_items, head, done, status);
}

}  // namespace

bool persistent_kind_built(int N, int G) {
  return (N == G && (N == 8 || N == 27 || N == 4 || N == 10 || N == 6)) || (N == 64 && G == 27) ||
         (N == 20 && G == 14) || (N == 18 && G == 6) || (N == 40 && G == 6);
}

void launch_batch_persistent(const PMember *mem, const PItem *items, int64_t n_items, unsigned long long *head,
                             unsigned int *done, int *status, bool mixed, int tile, int grid, cudaStream_t s) {
#define LMG_PL(M, T) \
  if (mixed == M && tile == T) return launch_t<M, T>(mem, items, n_items, head, done, status, grid, s);
  LMG_PL(false, 4) LMG_PL(false, 8) LMG_PL(false, 16) LMG_PL(false, 32)
  LMG_PL(true, 4) LMG_PL(true, 8) LMG_PL(true, 16) LMG_PL(true, 32)
#undef LMG_PL
}

int persistent_ctas_per_sm(bool mixed, int tile) {
  int n = 1;
#define LMG_PO(M, T) \
  if (mixed == M && tile == T) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_persistent<M, T>, H3T, 0);
  LMG_PO(false, 4) LMG_PO(false, 8) LMG_PO(false, 16) LMG_PO(false, 32)
  LMG_PO(true, 4) LMG_PO(true, 8) LMG_PO(true, 16) LMG_PO(true, 32)
#undef LMG_PO
  return n > 0 ? n : 1;
}

}  // namespace lmg
