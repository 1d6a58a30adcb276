// Device context of the assembly drop-in: uploads, sparsity, scatter plan,
// assemble, and the C-ABI entry points that drive them.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include "context_internal.cuh"
#include "general.cuh"

using namespace lmg;

namespace {

// ---------------------------------------------------------------- kernels
__global__ void k_expand_cols(int64_t n_dofs, int bs, const int64_t *brow_ptr, const int32_t *bcol,
                              const int32_t *row_ptr, int32_t *col) {
  const int lane = threadIdx.x & 31;
  for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n_dofs;
       r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
    const int64_t P = r / bs;
    const int64_t rb = brow_ptr[P];
    const int64_t len = (brow_ptr[P + 1] - rb) * bs;
    int32_t *out = col + row_ptr[r];
    for (int64_t m = lane; m < len; m += 32) out[m] = (int32_t)(bs * bcol[rb + m / bs] + m % bs);
  }
}

// Block slot of every element block pair (e, a, b) by binary search in the
// block row; counts contributions per slot.
__global__ void k_slots(int64_t n_elem, int nb, const int32_t *eb, const int64_t *brow_ptr,
                        const int32_t *bcol, int32_t *slot, int32_t *cnt, int *status) {
  const int64_t total = n_elem * nb * nb;
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < total;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = idx / (nb * nb);
    const int ab = (int)(idx - e * nb * nb);
    const int a = ab / nb, b = ab - a * nb;
    const int32_t P = eb[e * nb + a], Q = eb[e * nb + b];
    int64_t lo = brow_ptr[P], hi = brow_ptr[P + 1];
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (bcol[mid] < Q) lo = mid + 1; else hi = mid;
    }
    if (lo >= brow_ptr[P + 1] || bcol[lo] != Q) {
      atomicCAS(status, 0, LMG_ERR_NEW_NONZERO);
      slot[idx] = -1;
      continue;
    }
    slot[idx] = (int32_t)lo;
    atomicAdd(&cnt[lo], 1);
  }
}

// Slot of block (a, b) relative to the start of block row eb[e][a] (fits a
// byte when every block row has at most 255 slots).
__global__ void k_relslot(int64_t npair, int nb, const int32_t *eb, const int64_t *brow_ptr, const int32_t *slot,
                          uint8_t *rel) {
  for (int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; idx < npair;
       idx += (int64_t)gridDim.x * blockDim.x) {
    const int64_t ea = idx / nb;  // e * nb + a
    rel[idx] = (uint8_t)(slot[idx] - brow_ptr[eb[ea]]);
  }
}

__global__ void k_count_rows(int64_t n, const int32_t *eb, int32_t *cnt) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[eb[i]], 1);
}

__global__ void k_fill(int64_t n, const int32_t *key, const int32_t *ptr, int32_t *cur,
                       int32_t *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int32_t k = key[i];
    if (k < 0) continue;
    out[ptr[k] + atomicAdd(&cur[k], 1)] = (int32_t)i;
  }
}

// Constrained sparsity (find_connected_dofs, src/base/dof_map.C:2915-2970):
// every element couples the union of its dofs and of the dofs their
// constraint rows refer to.  k_enlarge: warp per element, the element's dofs
// and its constrained dofs' row columns gathered into shared memory, bitonic
// sort, duplicates dropped by ballot; PASS 0 records the length (and raises
// `flag` bit 1 when an added dof is itself constrained -- a chain the host
// closure would follow -- or bit 0 when the list outgrows the buffer),
// PASS 1 writes the list padded with INT32_MAX to width W.
constexpr int ENL_CAP = 1024, ENL_WARPS = 4;
template <int PASS>
__global__ void __launch_bounds__(ENL_WARPS * 32) k_enlarge(int64_t n_elem, int nl, const int32_t *ed,
                                                           const int64_t *cons_ptr, const int32_t *cons_col, int W,
                                                           int32_t *len, int32_t *out, int *flag) {
  __shared__ int32_t buf[ENL_WARPS][ENL_CAP];
  __shared__ int32_t sn[ENL_WARPS];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t *b = buf[warp];
  for (int64_t e = (int64_t)blockIdx.x * ENL_WARPS + warp; e < n_elem; e += (int64_t)gridDim.x * ENL_WARPS) {
    if (lane == 0) sn[warp] = 0;
    __syncwarp();
    bool over = false;
    for (int i = lane; i < nl; i += 32) {
      const int32_t d = ed[e * nl + i];
      const int64_t r0 = cons_ptr[d], r1 = cons_ptr[d + 1];
      const int k = atomicAdd(&sn[warp], 1 + (int)(r1 - r0));
      if (k + 1 + (r1 - r0) > ENL_CAP) { over = true; continue; }
      b[k] = d;
      for (int64_t r = r0; r < r1; ++r) b[k + 1 + (r - r0)] = cons_col[r];
    }
    __syncwarp();
    if (__any_sync(0xffffffffu, over)) {
      if (lane == 0) atomicOr(flag, 1);
      __syncwarp();
      continue;
    }
    const int n = sn[warp];
    int S = 1;
    while (S < n) S <<= 1;
    for (int t = n + lane; t < S; t += 32) b[t] = 0x7fffffff;
    __syncwarp();
    for (int k = 2; k <= S; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int t = lane; t < S; t += 32) {
          const int u = t ^ j;
          if (u > t) {
            const int32_t x = b[t], y = b[u];
            if ((x > y) == ((t & k) == 0)) { b[t] = y; b[u] = x; }
          }
        }
        __syncwarp();
      }
    int count = 0;
    bool chain = false;
    for (int t0 = 0; t0 < S; t0 += 32) {
      const int t = t0 + lane;
      const bool keep = t < S && b[t] != 0x7fffffff && (t == 0 || b[t] != b[t - 1]);
      if (keep && PASS == 0 && cons_ptr[b[t] + 1] > cons_ptr[b[t]]) {
        // a constrained dof in the list: it must be one of the element's own
        bool own = false;
        for (int i = 0; i < nl && !own; ++i) own = ed[e * nl + i] == b[t];
        chain |= !own;
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (PASS == 1 && keep) out[e * W + count + __popc(m & ((1u << lane) - 1u))] = b[t];
      count += __popc(m);
    }
    if (PASS == 0) {
      if (__any_sync(0xffffffffu, chain) && lane == 0) atomicOr(flag, 2);
      if (lane == 0) len[e] = count;
    } else {
      for (int t = count + lane; t < W; t += 32) out[e * W + t] = 0x7fffffff;
    }
    __syncwarp();
  }
}

__global__ void k_width(int64_t n, const int32_t *len, int *w) {
  int m = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    m = max(m, len[i]);
  atomicMax(w, m);
}

// Incidences of the padded lists (INT32_MAX entries skipped).
__global__ void k_count_padded(int64_t n, const int32_t *v, int32_t *cnt) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (v[i] != 0x7fffffff) atomicAdd(&cnt[v[i]], 1);
}
__global__ void k_fill_padded(int64_t n, const int32_t *v, const int32_t *ptr, int32_t *cur, int32_t *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    if (v[i] != 0x7fffffff) out[ptr[v[i]] + atomicAdd(&cur[v[i]], 1)] = (int32_t)i;
}

// Rows of the constrained graph: warp per dof, the lists of the elements whose
// enlarged list holds the dof, merged by a bitonic sort in a per-warp buffer of
// `cap` entries (dynamic shared memory); rows that need more raise `flag`.
template <int PASS>
__global__ void __launch_bounds__(ENL_WARPS * 32) k_row_graph(int64_t n_rows, int W, const int32_t *lists,
                                                             const int32_t *iptr, const int32_t *icon, int cap,
                                                             int32_t *deg, const int32_t *rptr, int32_t *col,
                                                             int *flag) {
  extern __shared__ int32_t rbuf[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t *b = rbuf + (size_t)warp * cap;
  for (int64_t P = (int64_t)blockIdx.x * ENL_WARPS + warp; P < n_rows; P += (int64_t)gridDim.x * ENL_WARPS) {
    const int32_t i0 = iptr[P], i1 = iptr[P + 1];
    const int n = (i1 - i0) * W;
    if (n > cap) {
      if (lane == 0) atomicOr(flag, 1);
      continue;
    }
    int S = 1;
    while (S < n) S <<= 1;
    for (int t = lane; t < S; t += 32) {
      int32_t v = 0x7fffffff;
      if (t < n) v = lists[(int64_t)(icon[i0 + t / W] / W) * W + t % W];
      b[t] = v;
    }
    __syncwarp();
    for (int k = 2; k <= S; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int t = lane; t < S; t += 32) {
          const int u = t ^ j;
          if (u > t) {
            const int32_t x = b[t], y = b[u];
            if ((x > y) == ((t & k) == 0)) { b[t] = y; b[u] = x; }
          }
        }
        __syncwarp();
      }
    int count = 0;
    for (int t0 = 0; t0 < S; t0 += 32) {
      const int t = t0 + lane;
      const bool keep = t < S && b[t] != 0x7fffffff && (t == 0 || b[t] != b[t - 1]);
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (PASS == 1 && keep) col[rptr[P] + count + __popc(m & ((1u << lane) - 1u))] = b[t];
      count += __popc(m);
    }
    if (PASS == 0 && lane == 0) deg[P] = count;
    __syncwarp();
  }
}

// Each segment is short (the elements sharing one block pair), so an
// insertion sort per thread puts contributions in element order.
__global__ void k_segsort(int64_t n_seg, const int32_t *ptr, int32_t *v) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_seg;
       s += (int64_t)gridDim.x * blockDim.x) {
    const int32_t b = ptr[s], e = ptr[s + 1];
    for (int32_t i = b + 1; i < e; ++i) {
      const int32_t x = v[i];
      int32_t j = i - 1;
      while (j >= b && v[j] > x) { v[j + 1] = v[j]; --j; }
      v[j + 1] = x;
    }
  }
}

// Last element contributing to block row P (contributions e*nb + a sorted
// ascending); -1 for a row no element touches.
__global__ void k_row_last(int64_t n_rows, int nb, const int32_t *ptr, const int32_t *contrib, int32_t *last) {
  for (int64_t P = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; P < n_rows;
       P += (int64_t)gridDim.x * blockDim.x)
    last[P] = ptr[P + 1] > ptr[P] ? contrib[ptr[P + 1] - 1] / nb : -1;
}

// Re-encodes every matrix contribution (e*nb + a)*nb + b of a slot into the
// symmetric element storage: diagonal pairs -> e*nb + a (Kdiag block), other
// pairs -> 2*(e*no + o) + t with o the strictly upper block of {a, b} and
// t = 1 for a > b (the slot reads the transpose).  Element order is kept.
__global__ void k_encode(int64_t n, int nb, int32_t *v) {
  const int no = nb * (nb - 1) / 2;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = v[i];
    const int64_t e = x / ((int64_t)nb * nb);
    const int ab = (int)(x - e * nb * nb);
    const int a = ab / nb, b = ab - a * nb;
    if (a == b) {
      v[i] = (int32_t)(e * nb + a);
    } else {
      const int lo = a < b ? a : b, hi = a < b ? b : a;
      const int o = lo * nb - lo * (lo + 1) / 2 + (hi - lo - 1);
      v[i] = (int32_t)(2 * (e * no + o) + (a > b ? 1 : 0));
    }
  }
}

// Whether block row P touches a constrained dof: one of its own or of its
// columns' bs dofs (thread per block row).
__global__ void k_rowcons(int64_t n_rows, int bs, const int64_t *brow_ptr, const int32_t *bcol, const uint8_t *cons,
                          uint8_t *out) {
  for (int64_t P = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; P < n_rows; P += (int64_t)gridDim.x * blockDim.x) {
    uint8_t v = 0;
    for (int64_t j = brow_ptr[P]; j < brow_ptr[P + 1] && !v; ++j)
      for (int k = 0; k < bs; ++k) v |= cons[(int64_t)bs * bcol[j] + k];
    out[P] = v ? 1 : 0;
  }
}

// Position of the diagonal slot in every block row (the insertion reads it
// with the row headers instead of searching the row's columns).
__global__ void k_bdiag(int64_t n_rows, const int64_t *brow_ptr, const int32_t *bcol, int32_t *bdiag) {
  for (int64_t P = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; P < n_rows; P += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = brow_ptr[P], hi = brow_ptr[P + 1];
    const int64_t b = lo;
    while (lo < hi) {
      const int64_t mid = (lo + hi) >> 1;
      if (bcol[mid] < P) lo = mid + 1; else hi = mid;
    }
    bdiag[P] = (lo < brow_ptr[P + 1] && bcol[lo] == (int32_t)P) ? (int32_t)(lo - b) : -1;
  }
}

// Nodal load split into double-float pairs (read by the affine element kernels).
__global__ void k_split(int64_t n, const double *x, float2 *y) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float hi = (float)x[i];
    y[i] = make_float2(hi, (float)(x[i] - (double)hi));
  }
}

// Exclusive scan helpers: block-local scan, then scan of block sums.
constexpr int SCAN_T = 1024;
__global__ void k_scan_local(int64_t n, const int32_t *in, int32_t *out, int32_t *bsum) {
  __shared__ int32_t ws[32];
  const int64_t i = (int64_t)blockIdx.x * SCAN_T + threadIdx.x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int32_t v = (i < n) ? in[i] : 0, x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    int32_t s = ws[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    ws[lane] = s;
  }
  __syncthreads();
  const int32_t off = w ? ws[w - 1] : 0;
  if (i < n) out[i] = x - v + off;
  if (threadIdx.x == SCAN_T - 1) bsum[blockIdx.x] = off + x;
}
__global__ void k_scan_add(int64_t n, int32_t *out, const int32_t *boff) {
  const int64_t i = (int64_t)blockIdx.x * SCAN_T + threadIdx.x;
  if (i < n) out[i] += boff[blockIdx.x];
}

}  // namespace

// DofMap::compute_sparsity on the device (block pattern of the block path):
// warp per block row P gathers the blocks of every element incident on P
// (the row's incidence list), sorts them in shared memory (bitonic) and keeps
// the distinct ones; pass 0 writes the degree, pass 1 the columns.  Rows with
// more than GRAPH_CAP candidates raise a flag and the host build takes over.
constexpr int GRAPH_CAP = 1024, GRAPH_WARPS = 4;
template <int PASS>
__global__ void __launch_bounds__(GRAPH_WARPS * 32) k_block_graph(int64_t n_rows, int nb, const int32_t *eb,
                                                                  const int32_t *iptr, const int32_t *icon,
                                                                  int32_t *deg, const int32_t *bptr, int32_t *bcol,
                                                                  int *overflow) {
  __shared__ int32_t buf[GRAPH_WARPS][GRAPH_CAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  int32_t *b = buf[warp];
  for (int64_t P = (int64_t)blockIdx.x * GRAPH_WARPS + warp; P < n_rows; P += (int64_t)gridDim.x * GRAPH_WARPS) {
    const int32_t i0 = iptr[P], i1 = iptr[P + 1];
    const int n = (i1 - i0) * nb;
    if (n > GRAPH_CAP) {
      if (lane == 0) *overflow = 1;
      continue;
    }
    int S = 1;
    while (S < n) S <<= 1;
    for (int t = lane; t < S; t += 32) {
      int32_t v = 0x7fffffff;
      if (t < n) {
        const int32_t entry = icon[i0 + t / nb];  // e * nb + a
        v = eb[(int64_t)(entry / nb) * nb + t % nb];
      }
      b[t] = v;
    }
    __syncwarp();
    for (int k = 2; k <= S; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int t = lane; t < S; t += 32) {
          const int u = t ^ j;
          if (u > t) {
            const int32_t x = b[t], y = b[u];
            const bool up = (t & k) == 0;
            if ((x > y) == up) {
              b[t] = y;
              b[u] = x;
            }
          }
        }
        __syncwarp();
      }
    int count = 0;
    for (int t0 = 0; t0 < S; t0 += 32) {
      const int t = t0 + lane;
      const bool keep = t < S && b[t] != 0x7fffffff && (t == 0 || b[t] != b[t - 1]);
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      if (PASS == 1 && keep) bcol[bptr[P] + count + __popc(m & ((1u << lane) - 1u))] = b[t];
      count += __popc(m);
    }
    if (PASS == 0 && lane == 0) deg[P] = count;
    __syncwarp();
  }
}

namespace {

int grid_for(lmg_ctx *c, int64_t items, int threads) {
  int64_t b = (items + threads - 1) / threads;
  const int64_t cap = (int64_t)c->n_sm * 16;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

// out[0..n] = exclusive scan of in[0..n); out[n] = total.
lmg_status scan_i32(lmg_ctx *c, const int32_t *in, int32_t *out, int64_t n) {
  const int64_t nblk = (n + SCAN_T - 1) / SCAN_T;
  int32_t *bsum = nullptr, *boff = nullptr;
  LMG_CUDA(c, dalloc(bsum, (size_t)nblk + 1));
  LMG_CUDA(c, dalloc(boff, (size_t)nblk + 1));
  if (n > 0) {
    k_scan_local<<<(unsigned)nblk, SCAN_T, 0, c->stream>>>(n, in, out, bsum);
    c->launches++;
    if (nblk > 1) {
      lmg_status st = scan_i32(c, bsum, boff, nblk);
      if (st != LMG_OK) { dfree(bsum); dfree(boff); return st; }
      k_scan_add<<<(unsigned)nblk, SCAN_T, 0, c->stream>>>(n, out, boff);
      c->launches++;
      LMG_CUDA(c, cudaMemcpyAsync(out + n, boff + nblk, sizeof(int32_t), cudaMemcpyDeviceToDevice,
                                  c->stream));
    } else {
      LMG_CUDA(c, cudaMemcpyAsync(out + n, bsum, sizeof(int32_t), cudaMemcpyDeviceToDevice, c->stream));
    }
  } else {
    LMG_CUDA(c, cudaMemsetAsync(out, 0, sizeof(int32_t), c->stream));
  }
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  dfree(bsum);
  dfree(boff);
  return LMG_OK;
}

// Constrained graph on the device (rows and columns into rp / cols, and into
// d_row_ptr / d_col); LMG_ERR_UNSUPPORTED when an element list or a row
// outgrows its buffer or a constraint row refers to a constrained dof (the
// caller then builds it on the host).
lmg_status constrained_graph_impl(lmg_ctx *c, std::vector<int64_t> &rp, std::vector<int32_t> &cols) {
  const int64_t E = c->n_elem, nd = c->n_dofs;
  const int nl = c->nl;
  std::vector<int64_t> cp = c->h_cons_ptr;
  if (cp.empty()) cp.assign((size_t)nd + 1, 0);
  int32_t *d_ed = nullptr, *d_ccol = nullptr, *len = nullptr, *lists = nullptr, *cnt = nullptr, *iptr = nullptr,
          *cur = nullptr, *icon = nullptr, *deg = nullptr, *rptr = nullptr, *colv = nullptr;
  int64_t *d_cp = nullptr;
  int *flag = nullptr;
  auto cleanup = [&]() {
    dfree(d_ed); dfree(d_ccol); dfree(len); dfree(lists); dfree(cnt); dfree(iptr); dfree(cur); dfree(icon);
    dfree(deg); dfree(d_cp); dfree(flag);
  };
  auto bad = [&](lmg_status st) { cleanup(); dfree(rptr); dfree(colv); return st; };
  if (dupload(c, d_ed, c->h_elem_dofs.data(), c->h_elem_dofs.size()) != cudaSuccess ||
      dupload(c, d_cp, cp.data(), cp.size()) != cudaSuccess ||
      dupload(c, d_ccol, c->h_cons_col.data(), c->h_cons_col.size()) != cudaSuccess ||
      dalloc(len, (size_t)E) != cudaSuccess || dalloc(flag, 2) != cudaSuccess)
    return bad(LMG_ERR_CUDA);
  cudaMemsetAsync(flag, 0, 2 * sizeof(int), c->stream);
  const int g = grid_for(c, E * 32, ENL_WARPS * 32);
  k_enlarge<0><<<g, ENL_WARPS * 32, 0, c->stream>>>(E, nl, d_ed, d_cp, d_ccol, 0, len, nullptr, flag);
  k_width<<<grid_for(c, E, 256), 256, 0, c->stream>>>(E, len, flag + 1);
  c->launches += 2;
  int hf[2] = {0, 0};
  if (cudaMemcpyAsync(hf, flag, sizeof(hf), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return bad(LMG_ERR_CUDA);
  if (hf[0]) return bad(LMG_ERR_UNSUPPORTED);
  const int W = std::max(hf[1], 1);
  if (dalloc(lists, (size_t)(E * W)) != cudaSuccess || dalloc(cnt, (size_t)nd) != cudaSuccess ||
      dalloc(cur, (size_t)nd) != cudaSuccess || dalloc(iptr, (size_t)nd + 1) != cudaSuccess ||
      dalloc(deg, (size_t)nd) != cudaSuccess || dalloc(rptr, (size_t)nd + 1) != cudaSuccess)
    return bad(LMG_ERR_OOM);
  k_enlarge<1><<<g, ENL_WARPS * 32, 0, c->stream>>>(E, nl, d_ed, d_cp, d_ccol, W, len, lists, flag);
  cudaMemsetAsync(cnt, 0, sizeof(int32_t) * nd, c->stream);
  k_count_padded<<<grid_for(c, E * W, 256), 256, 0, c->stream>>>(E * W, lists, cnt);
  c->launches += 2;
  lmg_status st = scan_i32(c, cnt, iptr, nd);
  if (st) return bad(st);
  int32_t n_inc = 0;
  if (cudaMemcpy(&n_inc, iptr + nd, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) return bad(LMG_ERR_CUDA);
  if (dalloc(icon, (size_t)std::max(n_inc, 1)) != cudaSuccess) return bad(LMG_ERR_OOM);
  cudaMemsetAsync(cur, 0, sizeof(int32_t) * nd, c->stream);
  k_fill_padded<<<grid_for(c, E * W, 256), 256, 0, c->stream>>>(E * W, lists, iptr, cur, icon);
  c->launches++;
  const int cap = 4096;
  const size_t smem = sizeof(int32_t) * cap * ENL_WARPS;
  cudaFuncSetAttribute(k_row_graph<0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  cudaFuncSetAttribute(k_row_graph<1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int gr = grid_for(c, nd * 32, ENL_WARPS * 32);
  k_row_graph<0><<<gr, ENL_WARPS * 32, smem, c->stream>>>(nd, W, lists, iptr, icon, cap, deg, nullptr, nullptr,
                                                          flag);
  c->launches++;
  if (cudaMemcpyAsync(hf, flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return bad(LMG_ERR_CUDA);
  if (hf[0]) return bad(LMG_ERR_UNSUPPORTED);
  if ((st = scan_i32(c, deg, rptr, nd))) return bad(st);
  int32_t nnz = 0;
  if (cudaMemcpy(&nnz, rptr + nd, sizeof(int32_t), cudaMemcpyDeviceToHost) != cudaSuccess) return bad(LMG_ERR_CUDA);
  if (nnz < 0) return bad(LMG_ERR_UNSUPPORTED);
  if (dalloc(colv, (size_t)std::max(nnz, 1)) != cudaSuccess) return bad(LMG_ERR_OOM);
  k_row_graph<1><<<gr, ENL_WARPS * 32, smem, c->stream>>>(nd, W, lists, iptr, icon, cap, nullptr, rptr, colv, flag);
  c->launches++;
  std::vector<int32_t> r32((size_t)nd + 1);
  cols.resize((size_t)nnz);
  if (cudaMemcpyAsync(r32.data(), rptr, sizeof(int32_t) * (nd + 1), cudaMemcpyDeviceToHost, c->stream) !=
          cudaSuccess ||
      cudaMemcpyAsync(cols.data(), colv, sizeof(int32_t) * nnz, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    return bad(LMG_ERR_CUDA);
  rp.assign(r32.begin(), r32.end());
  cleanup();
  dfree(c->d_row_ptr);
  dfree(c->d_col);
  c->d_row_ptr = rptr;
  c->d_col = colv;
  return LMG_OK;
}

// Block graph on the device; LMG_ERR_UNSUPPORTED when a row has too many
// candidates (the caller then builds it on the host).
lmg_status device_block_graph(lmg_ctx *c, std::vector<int64_t> &brow) {
  const int nb = c->nb;
  const int64_t nrow = c->n_elem * nb, nbk = c->n_blocks;
  int32_t *cnt = nullptr, *cur = nullptr, *iptr = nullptr, *icon = nullptr, *deg = nullptr, *bptr = nullptr,
          *dcol = nullptr;
  int *ovf = nullptr;
  auto cleanup = [&]() { dfree(cnt); dfree(cur); dfree(iptr); dfree(icon); dfree(deg); dfree(bptr); dfree(dcol); dfree(ovf); };
  LMG_CUDA(c, dalloc(cnt, (size_t)nbk));
  LMG_CUDA(c, dalloc(cur, (size_t)nbk));
  LMG_CUDA(c, dalloc(iptr, (size_t)nbk + 1));
  LMG_CUDA(c, dalloc(icon, (size_t)nrow));
  LMG_CUDA(c, dalloc(deg, (size_t)nbk));
  LMG_CUDA(c, dalloc(bptr, (size_t)nbk + 1));
  LMG_CUDA(c, dalloc(ovf, 1));
  LMG_CUDA(c, cudaMemsetAsync(ovf, 0, sizeof(int), c->stream));
  // incidence of every block row: (e*nb + a) entries in element order
  LMG_CUDA(c, cudaMemsetAsync(cnt, 0, sizeof(int32_t) * nbk, c->stream));
  k_count_rows<<<grid_for(c, nrow, 256), 256, 0, c->stream>>>(nrow, c->d_eb, cnt);
  lmg_status st = scan_i32(c, cnt, iptr, nbk);
  if (st) { cleanup(); return st; }
  LMG_CUDA(c, cudaMemsetAsync(cur, 0, sizeof(int32_t) * nbk, c->stream));
  k_fill<<<grid_for(c, nrow, 256), 256, 0, c->stream>>>(nrow, c->d_eb, iptr, cur, icon);
  const int g = grid_for(c, nbk * 32, GRAPH_WARPS * 32);
  k_block_graph<0><<<g, GRAPH_WARPS * 32, 0, c->stream>>>(nbk, nb, c->d_eb, iptr, icon, deg, nullptr, nullptr, ovf);
  c->launches += 3;
  int h_ovf = 0;
  LMG_CUDA(c, cudaMemcpyAsync(&h_ovf, ovf, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (h_ovf) { cleanup(); return LMG_ERR_UNSUPPORTED; }
  if ((st = scan_i32(c, deg, bptr, nbk))) { cleanup(); return st; }
  int32_t total = 0;
  LMG_CUDA(c, cudaMemcpyAsync(&total, bptr + nbk, sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  LMG_CUDA(c, dalloc(dcol, (size_t)total));
  k_block_graph<1><<<g, GRAPH_WARPS * 32, 0, c->stream>>>(nbk, nb, c->d_eb, iptr, icon, nullptr, bptr, dcol, ovf);
  c->launches++;
  std::vector<int32_t> hp((size_t)nbk + 1);
  LMG_CUDA(c, cudaMemcpyAsync(hp.data(), bptr, sizeof(int32_t) * (nbk + 1), cudaMemcpyDeviceToHost, c->stream));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  brow.assign(hp.begin(), hp.end());
  dfree(c->d_bcol);
  c->d_bcol = dcol;  // the columns stay on the device
  dcol = nullptr;
  cleanup();
  return LMG_OK;
}

lmg_status check_status(lmg_ctx *c, const char *what) {
  int st = 0;
  unsigned long long bad = ~0ull;
  LMG_CUDA(c, cudaMemcpyAsync(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  LMG_CUDA(c, cudaMemcpyAsync(&bad, c->d_bad, sizeof(bad), cudaMemcpyDeviceToHost, c->stream));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (st != 0) {
    const int64_t e = (bad == ~0ull) ? -1 : (int64_t)bad;
    std::string m = std::string(what) + ": ";
    if (st == LMG_ERR_DEGENERATE) m += "Jacobian at or under tolerance 0 (degenerate element)";
    else if (st == LMG_ERR_NEW_NONZERO) m += "element couples a dof pair outside the sparsity pattern";
    else m += "device error";
    return fail(c, st, m, e);
  }
  return LMG_OK;
}

lmg_status reset_status(lmg_ctx *c) {
  LMG_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(int), c->stream));
  LMG_CUDA(c, cudaMemsetAsync(c->d_bad, 0xff, sizeof(unsigned long long), c->stream));
  return LMG_OK;
}

// Element -> block map, and whether the variables sit node-interleaved
// (dof = bs * block + var), which lets the plan work on bs x bs blocks.
void detect_blocks(lmg_ctx *c) {
  block_structure(c->n_elem, c->npe, c->n_vars, c->h_elem_dofs.data(), c->bs, c->nb, c->h_eb);
  c->n_blocks = c->n_dofs / c->bs;
}

lmg_status build_plan(lmg_ctx *c) {
  const int nb = c->nb;
  const int64_t npair = c->n_elem * nb * nb, nrow = c->n_elem * nb;
  if (npair * c->bs * c->bs >= INT32_MAX) return fail(c, LMG_ERR_UNSUPPORTED, "mesh too large for 32-bit plan");
  if (!gather_built(c->bs)) return fail(c, LMG_ERR_UNSUPPORTED, "no insertion kernel for this block size");
  int32_t *slot = nullptr, *cnt = nullptr, *cur = nullptr;
  LMG_CUDA(c, dalloc(slot, (size_t)npair));
  LMG_CUDA(c, dalloc(cnt, (size_t)std::max(c->nnzb, c->n_blocks)));
  LMG_CUDA(c, dalloc(cur, (size_t)std::max(c->nnzb, c->n_blocks)));
  LMG_CUDA(c, dalloc(c->d_bptr, (size_t)c->nnzb + 1));
  LMG_CUDA(c, dalloc(c->d_bcontrib, (size_t)npair));
  LMG_CUDA(c, dalloc(c->d_fptr, (size_t)c->n_blocks + 1));
  LMG_CUDA(c, dalloc(c->d_fcontrib, (size_t)nrow));
  lmg_status st = reset_status(c);
  if (st) return st;
  // matrix plan
  LMG_CUDA(c, cudaMemsetAsync(cnt, 0, sizeof(int32_t) * c->nnzb, c->stream));
  k_slots<<<grid_for(c, npair, 256), 256, 0, c->stream>>>(c->n_elem, nb, c->d_eb, c->d_brow_ptr,
                                                          c->d_bcol, slot, cnt, c->d_status);
  c->launches++;
  if ((st = scan_i32(c, cnt, c->d_bptr, c->nnzb))) return st;
  LMG_CUDA(c, cudaMemsetAsync(cur, 0, sizeof(int32_t) * c->nnzb, c->stream));
  k_fill<<<grid_for(c, npair, 256), 256, 0, c->stream>>>(npair, slot, c->d_bptr, cur, c->d_bcontrib);
  k_segsort<<<grid_for(c, c->nnzb, 256), 256, 0, c->stream>>>(c->nnzb, c->d_bptr, c->d_bcontrib);
  k_encode<<<grid_for(c, npair, 256), 256, 0, c->stream>>>(npair, nb, c->d_bcontrib);
  c->launches += 3;
  dfree(c->d_relslot);
  dfree(c->d_rowcons);
  dfree(c->d_bdiag);
  LMG_CUDA(c, dalloc(c->d_bdiag, (size_t)std::max<int64_t>(c->n_blocks, 1)));
  k_bdiag<<<grid_for(c, c->n_blocks, 256), 256, 0, c->stream>>>(c->n_blocks, c->d_brow_ptr, c->d_bcol, c->d_bdiag);
  c->launches++;
  if (c->max_bdeg <= 255) {  // the fused mixed form addresses slots with one byte
    LMG_CUDA(c, dalloc(c->d_relslot, (size_t)npair));
    k_relslot<<<grid_for(c, npair, 256), 256, 0, c->stream>>>(npair, nb, c->d_eb, c->d_brow_ptr, slot,
                                                              c->d_relslot);
    c->launches++;
  }
  // vector plan
  LMG_CUDA(c, cudaMemsetAsync(cnt, 0, sizeof(int32_t) * c->n_blocks, c->stream));
  k_count_rows<<<grid_for(c, nrow, 256), 256, 0, c->stream>>>(nrow, c->d_eb, cnt);
  c->launches++;
  if ((st = scan_i32(c, cnt, c->d_fptr, c->n_blocks))) return st;
  LMG_CUDA(c, cudaMemsetAsync(cur, 0, sizeof(int32_t) * c->n_blocks, c->stream));
  k_fill<<<grid_for(c, nrow, 256), 256, 0, c->stream>>>(nrow, c->d_eb, c->d_fptr, cur, c->d_fcontrib);
  k_segsort<<<grid_for(c, c->n_blocks, 256), 256, 0, c->stream>>>(c->n_blocks, c->d_fptr,
                                                                  c->d_fcontrib);
  // last contributing element of every block row (the pipelined host output
  // inserts a row once every element before it has run)
  k_row_last<<<grid_for(c, c->n_blocks, 256), 256, 0, c->stream>>>(c->n_blocks, nb, c->d_fptr, c->d_fcontrib, cur);
  c->launches += 3;
  c->h_row_pmax.resize((size_t)c->n_blocks);
  LMG_CUDA(c, cudaMemcpyAsync(c->h_row_pmax.data(), cur, sizeof(int32_t) * c->n_blocks, cudaMemcpyDeviceToHost,
                              c->stream));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  for (size_t P = 1; P < c->h_row_pmax.size(); ++P)  // prefix maximum
    c->h_row_pmax[P] = std::max(c->h_row_pmax[P], c->h_row_pmax[P - 1]);
  dfree(slot);
  dfree(cnt);
  dfree(cur);
  return check_status(c, "sparsity plan");
}

// Host output of K pipelined with the assembly: the elements run in
// OUT_CHUNKS ranges of element ids; after range ch the block rows whose
// contributing elements all lie in ranges <= ch (a prefix of the rows, from
// the prefix maximum of each row's last element) are inserted on the context
// stream and copied on a second stream while the next range runs.
// launch_elems(E0, E1) enqueues the element work of elements [E0, E1);
// launch_rows(P0, P1) the insertion of block rows [P0, P1).
constexpr int OUT_CHUNKS = 32;
template <typename LaunchElems, typename LaunchRows>
lmg_status pipelined_copy(lmg_ctx *c, double *K, LaunchElems &&launch_elems, LaunchRows &&launch_rows) {
  if (!c->copy_stream) LMG_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  while ((int)c->chunk_ev.size() < OUT_CHUNKS) {
    cudaEvent_t e;
    LMG_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    c->chunk_ev.push_back(e);
  }
  const int64_t nb = c->n_blocks, E = c->n_elem;
  int64_t P0 = 0;
  for (int ch = 0; ch < OUT_CHUNKS; ++ch) {
    const int64_t E0 = E * ch / OUT_CHUNKS, E1 = E * (ch + 1) / OUT_CHUNKS;
    if (E1 > E0) launch_elems(E0, E1);
    const int64_t P1 = (ch == OUT_CHUNKS - 1)
                           ? nb
                           : (int64_t)(std::lower_bound(c->h_row_pmax.begin(), c->h_row_pmax.end(), (int32_t)E1) -
                                       c->h_row_pmax.begin());
    if (P1 <= P0) continue;
    launch_rows(P0, P1);
    LMG_CUDA(c, cudaEventRecord(c->chunk_ev[ch], c->stream));
    LMG_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->chunk_ev[ch], 0));
    const int64_t k0 = c->h_rowptr_blk[(size_t)(c->bs * P0)], k1 = c->h_rowptr_blk[(size_t)(c->bs * P1)];
    LMG_CUDA(c, cudaMemcpyAsync(K + k0, c->d_K + k0, sizeof(double) * (k1 - k0), cudaMemcpyDeviceToHost,
                                c->copy_stream));
    P0 = P1;
  }
  return LMG_OK;
}

// The slice of an ascending element list that falls in [E0, E1).
inline void list_slice(const std::vector<int32_t> &h, int64_t E0, int64_t E1, int64_t &off, int64_t &cnt) {
  const auto b = std::lower_bound(h.begin(), h.end(), (int32_t)E0), e = std::lower_bound(h.begin(), h.end(), (int32_t)E1);
  off = b - h.begin();
  cnt = e - b;
}

// Host outputs of a large system take the chunked path.
bool chunked_output(const lmg_ctx *c, const double *K, int32_t out_on_device) {
  return K && !out_on_device && c->nnz * (int64_t)sizeof(double) > ((int64_t)64 << 20) &&
         (int64_t)c->h_rowptr_blk.size() == c->n_dofs + 1 && (int64_t)c->h_row_pmax.size() == c->n_blocks;
}

void build_lists(lmg_ctx *c) {
  c->h_aff.clear();
  c->h_gen.clear();
  for (int64_t e = 0; e < c->n_elem; ++e) {
    double P[27 * 3];
    for (int a = 0; a < c->npe; ++a)
      for (int d = 0; d < 3; ++d)
        P[3 * a + d] = c->h_xyz[(size_t)(3 * (int64_t)c->h_conn[(size_t)(e * c->npe + a)] + d)];
    (elem_has_affine_map(c->elem_type, P) ? c->h_aff : c->h_gen).push_back((int32_t)e);
  }
}

lmg_status upload_cmask(lmg_ctx *c) {
  std::vector<uint64_t> m((size_t)c->n_elem, 0);
  if (!c->h_constrained.empty())
    for (int64_t e = 0; e < c->n_elem; ++e)
      for (int l = 0; l < c->nl; ++l)
        if (c->h_constrained[(size_t)c->h_elem_dofs[(size_t)(e * c->nl + l)]]) m[(size_t)e] |= 1ull << l;
  LMG_CUDA(c, dupload(c, c->d_cmask, m.data(), m.size()));
  std::vector<uint8_t> cons = c->h_constrained;
  cons.resize((size_t)c->n_dofs, 0);
  LMG_CUDA(c, dupload(c, c->d_cons, cons.data(), cons.size()));
  dfree(c->d_rowcons);  // re-derived on the next fused assembly
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  return LMG_OK;
}

}  // namespace

lmg_status lmg::device_constrained_graph(lmg_ctx *c, std::vector<int64_t> &rp, std::vector<int32_t> &cols) {
  return constrained_graph_impl(c, rp, cols);
}

extern "C" {

lmg_status lmg_context_create(lmg_ctx **out, int32_t device) {
  if (!out) return LMG_ERR_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return LMG_ERR_CUDA;
  if (device < 0 || device >= n) return LMG_ERR_ARG;
  lmg_ctx *c = new (std::nothrow) lmg_ctx;
  if (!c) return LMG_ERR_OOM;
  c->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return LMG_ERR_CUDA;
  }
  c->own_stream = true;
  cudaDeviceGetAttribute(&c->n_sm, cudaDevAttrMultiProcessorCount, device);
  if (cudaMalloc((void **)&c->d_status, sizeof(int)) != cudaSuccess ||
      cudaMalloc((void **)&c->d_bad, sizeof(unsigned long long)) != cudaSuccess) {
    cudaStreamDestroy(c->stream);
    delete c;
    return LMG_ERR_OOM;
  }
  *out = c;
  return LMG_OK;
}

lmg_status lmg_context_destroy(lmg_ctx *c) {
  if (!c) return LMG_OK;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  dfree(c->d_xyz); dfree(c->d_conn); dfree(c->d_aff); dfree(c->d_gen); dfree(c->d_eb);
  dfree(c->d_cmask); dfree(c->d_cons); dfree(c->d_rowcons); dfree(c->d_bdiag); dfree(c->d_brow_ptr); dfree(c->d_bcol); dfree(c->d_row_ptr); dfree(c->d_col);
  dfree(c->d_bptr); dfree(c->d_bcontrib); dfree(c->d_fptr); dfree(c->d_fcontrib); dfree(c->d_tab);
  dfree(c->d_coef); dfree(c->d_f); dfree(c->d_f2); dfree(c->d_Kdiag2); dfree(c->d_Koff2); dfree(c->d_Fe2); dfree(c->d_K);
  dfree(c->d_F); dfree(c->d_Koff32); dfree(c->d_status); dfree(c->d_bad);
  dfree(c->d_relslot); dfree(c->d_geo);
  general_free(c);
  hier3_free(c);
  dfree(c->d_D6); dfree(c->d_modes);
  dfree(c->d_Re2);
  for (cudaEvent_t e : c->chunk_ev) cudaEventDestroy(e);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return LMG_OK;
}

lmg_status lmg_context_set_stream(lmg_ctx *c, void *stream) {
  if (!c) return LMG_ERR_ARG;
  cudaSetDevice(c->device);
  if (c->stream) cudaStreamSynchronize(c->stream);
  if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
  c->stream = (cudaStream_t)stream;
  c->own_stream = false;
  return LMG_OK;
}

lmg_status lmg_mesh_upload(lmg_ctx *c, int64_t n_nodes, const double *xyz, int64_t n_elem,
                           int32_t elem_type, const int32_t *conn) {
  if (!c || !xyz || !conn || n_nodes <= 0 || n_elem <= 0) return fail(c, LMG_ERR_ARG, "mesh_upload: bad argument");
  const int npe = nodes_per_elem(elem_type);
  if (!npe) return fail(c, LMG_ERR_UNSUPPORTED, "mesh_upload: element type not built");
  if (n_elem * npe >= INT32_MAX || n_nodes >= INT32_MAX) return fail(c, LMG_ERR_UNSUPPORTED, "mesh too large");
  for (int64_t i = 0; i < n_elem * npe; ++i)
    if (conn[i] < 0 || conn[i] >= n_nodes) return fail(c, LMG_ERR_BOUNDS, "mesh_upload: node id out of range", i / npe);
  cudaSetDevice(c->device);
  c->elem_type = elem_type;
  c->npe = npe;
  c->n_nodes = n_nodes;
  c->n_elem = n_elem;
  c->h_xyz.assign(xyz, xyz + 3 * n_nodes);
  c->h_conn.assign(conn, conn + n_elem * npe);
  build_lists(c);
  LMG_CUDA(c, dupload(c, c->d_xyz, xyz, (size_t)(3 * n_nodes)));
  LMG_CUDA(c, dupload(c, c->d_conn, conn, (size_t)(n_elem * npe)));
  LMG_CUDA(c, dupload(c, c->d_aff, c->h_aff.data(), c->h_aff.size()));
  LMG_CUDA(c, dupload(c, c->d_gen, c->h_gen.data(), c->h_gen.size()));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_sparsity = false;
  c->n_vars = 0;
  return LMG_OK;
}

lmg_status lmg_dofmap_upload(lmg_ctx *c, int32_t n_vars, int64_t n_dofs, const int32_t *elem_dofs) {
  if (!c || !elem_dofs || n_vars <= 0 || n_dofs <= 0) return fail(c, LMG_ERR_ARG, "dofmap_upload: bad argument");
  if (!c->n_elem) return fail(c, LMG_ERR_STATE, "dofmap_upload: upload the mesh first");
  const int nl = n_vars * c->npe;
  if (nl > 64) return fail(c, LMG_ERR_UNSUPPORTED, "more than 64 dofs per element");
  for (int64_t i = 0; i < c->n_elem * nl; ++i)
    if (elem_dofs[i] < 0 || elem_dofs[i] >= n_dofs) return fail(c, LMG_ERR_BOUNDS, "dof id out of range", i / nl);
  cudaSetDevice(c->device);
  c->n_vars = n_vars;
  c->nl = nl;
  c->n_dofs = n_dofs;
  c->hier3 = false;
  c->h_elem_dofs.assign(elem_dofs, elem_dofs + c->n_elem * nl);
  detect_blocks(c);
  LMG_CUDA(c, dupload(c, c->d_eb, c->h_eb.data(), c->h_eb.size()));
  c->h_constrained.clear();
  c->h_cons_ptr.clear();
  c->h_cons_col.clear();
  c->h_cons_val.clear();
  c->has_rows = false;
  c->have_sparsity = false;
  c->gen_plan = false;
  return upload_cmask(c);
}

lmg_status lmg_dofmap_upload_fe(lmg_ctx *c, int32_t n_vars, int32_t fe_order, int64_t n_dofs,
                                const int32_t *elem_dofs) {
  const bool prism2 = c && fe_order == (2 | LMG_HIERARCHIC) && c->elem_type == LMG_PRISM18;
  if (fe_order != (3 | LMG_HIERARCHIC) && !prism2) return lmg_dofmap_upload(c, n_vars, n_dofs, elem_dofs);
  if (!c || !elem_dofs || n_vars != 1 || n_dofs <= 0) return fail(c, LMG_ERR_ARG, "dofmap_upload: bad argument");
  if (!c->n_elem) return fail(c, LMG_ERR_STATE, "dofmap_upload: upload the mesh first");
  const int nl = pattern_fe_dofs(c->elem_type, fe_order);
  if (!nl)
    return fail(c, LMG_ERR_UNSUPPORTED, "dofmap_upload: THIRD HIERARCHIC needs HEX27, TET14 or PRISM21");
  for (int64_t i = 0; i < c->n_elem * nl; ++i)
    if (elem_dofs[i] < 0 || elem_dofs[i] >= n_dofs) return fail(c, LMG_ERR_BOUNDS, "dof id out of range", i / nl);
  cudaSetDevice(c->device);
  c->n_vars = 1;
  c->nl = nl;
  c->n_dofs = n_dofs;
  c->hier3 = true;
  c->h_elem_dofs.assign(elem_dofs, elem_dofs + c->n_elem * nl);
  c->bs = 1;  // no block structure: the general path assembles these systems
  c->nb = nl;
  c->n_blocks = n_dofs;
  c->h_eb.clear();
  c->h_constrained.clear();
  c->h_cons_ptr.clear();
  c->h_cons_col.clear();
  c->h_cons_val.clear();
  c->has_rows = false;
  c->have_sparsity = false;
  c->have_form = false;
  c->gen_plan = false;
  return upload_cmask(c);
}

lmg_status lmg_constraints_upload(lmg_ctx *c, const uint8_t *constrained) {
  if (!c || !constrained) return fail(c, LMG_ERR_ARG, "constraints_upload: bad argument");
  if (!c->n_dofs) return fail(c, LMG_ERR_STATE, "constraints_upload: upload the dofmap first");
  cudaSetDevice(c->device);
  c->h_constrained.assign(constrained, constrained + c->n_dofs);
  if (c->has_rows) c->have_sparsity = false;  // the pattern loses the constraint couplings
  c->h_cons_ptr.clear();
  c->h_cons_col.clear();
  c->h_cons_val.clear();
  c->has_rows = false;
  c->gen_plan = false;
  return upload_cmask(c);
}

lmg_status lmg_sparsity_build(lmg_ctx *c, int64_t *nnz) {
  if (!c) return LMG_ERR_ARG;
  if (!c->n_dofs) return fail(c, LMG_ERR_STATE, "sparsity_build: upload the dofmap first");
  cudaSetDevice(c->device);
  c->gen_plan = false;
  c->h_row_ptr.clear();
  c->h_col.clear();
  c->general = c->has_rows || c->hier3 || (c->have_form && c->form == LMG_ADVDIFF);
  if (c->general) {  // constraint rows with coefficients: find_connected_dofs pattern
    lmg_status st = general_sparsity(c);
    if (st) return st;
    c->have_sparsity = true;
    if (nnz) *nnz = c->nnz;
    return LMG_OK;
  }
  std::vector<int64_t> brow;
  std::vector<int32_t> bcol;
  // the block pattern on the device; the host builds rows the device buffer cannot hold
  // (32-bit incidence and column offsets: every element adds at most nb^2 block pairs)
  lmg_status gs = c->n_elem * c->nb * c->nb < INT32_MAX ? device_block_graph(c, brow) : LMG_ERR_UNSUPPORTED;
  c->sparsity_on_device = gs == LMG_OK;
  if (gs == LMG_ERR_UNSUPPORTED) {
    const unsigned hw = std::thread::hardware_concurrency();
    build_block_graph(c->n_elem, c->nb, c->h_eb.data(), c->n_blocks, brow, bcol, hw ? (int)hw : 4);
    LMG_CUDA(c, dupload(c, c->d_bcol, bcol.data(), bcol.size()));
  } else if (gs) {
    return gs;
  }
  c->nnzb = brow.back();
  c->nnz = c->nnzb * c->bs * c->bs;
  c->max_bdeg = 0;
  for (size_t P = 0; P + 1 < brow.size(); ++P) c->max_bdeg = std::max(c->max_bdeg, (int)(brow[P + 1] - brow[P]));
  if (c->nnz >= INT32_MAX) return fail(c, LMG_ERR_UNSUPPORTED, "nnz exceeds 32-bit CSR");
  std::vector<int32_t> row_ptr((size_t)c->n_dofs + 1);
  row_ptr[0] = 0;
  for (int64_t r = 0; r < c->n_dofs; ++r) {
    const int64_t P = r / c->bs;
    row_ptr[(size_t)r + 1] = row_ptr[(size_t)r] + (int32_t)((brow[(size_t)P + 1] - brow[(size_t)P]) * c->bs);
  }
  LMG_CUDA(c, dupload(c, c->d_brow_ptr, brow.data(), brow.size()));
  LMG_CUDA(c, dupload(c, c->d_row_ptr, row_ptr.data(), row_ptr.size()));
  c->h_rowptr_blk = row_ptr;
  LMG_CUDA(c, dalloc(c->d_col, (size_t)c->nnz));
  k_expand_cols<<<grid_for(c, c->n_dofs * 32, 256), 256, 0, c->stream>>>(
      c->n_dofs, c->bs, c->d_brow_ptr, c->d_bcol, c->d_row_ptr, c->d_col);
  c->launches++;
  lmg_status st = build_plan(c);
  if (st) return st;
  LMG_CUDA(c, dalloc(c->d_K, (size_t)c->nnz));
  LMG_CUDA(c, dalloc(c->d_F, (size_t)c->n_dofs));
  // element-block buffers: allocated on the first assembly of each form
  dfree(c->d_Kdiag2);
  dfree(c->d_Koff2);
  dfree(c->d_Koff32);  // allocated on the first mixed assembly
  LMG_CUDA(c, dalloc(c->d_Fe2, (size_t)(c->n_elem * c->nl)));
  c->have_sparsity = true;
  if (nnz) *nnz = c->nnz;
  return LMG_OK;
}

lmg_status lmg_context_set_plan_on_device(lmg_ctx *c, int32_t on) {
  if (!c) return LMG_ERR_ARG;
  c->plan_on_device = on != 0;
  return LMG_OK;
}

lmg_status lmg_plan_on_device(lmg_ctx *c, int32_t *on_device) {
  if (!c || !on_device) return LMG_ERR_ARG;
  *on_device = c->plan_built_on_device ? 1 : 0;
  return LMG_OK;
}

lmg_status lmg_sparsity_on_device(lmg_ctx *c, int32_t *on_device) {
  if (!c || !on_device) return LMG_ERR_ARG;
  if (!c->have_sparsity) return fail(c, LMG_ERR_STATE, "sparsity_on_device: build the sparsity first");
  *on_device = c->sparsity_on_device ? 1 : 0;
  return LMG_OK;
}

lmg_status lmg_sparsity_copy(lmg_ctx *c, int32_t *row_ptr, int32_t *col_idx) {
  if (!c) return LMG_ERR_ARG;
  if (!c->have_sparsity) return fail(c, LMG_ERR_STATE, "sparsity_copy: build the sparsity first");
  cudaSetDevice(c->device);
  if (row_ptr)
    LMG_CUDA(c, cudaMemcpyAsync(row_ptr, c->d_row_ptr, sizeof(int32_t) * (c->n_dofs + 1),
                                cudaMemcpyDeviceToHost, c->stream));
  if (col_idx)
    LMG_CUDA(c, cudaMemcpyAsync(col_idx, c->d_col, sizeof(int32_t) * c->nnz, cudaMemcpyDeviceToHost,
                                c->stream));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  return LMG_OK;
}

}  // extern "C"

extern "C" {

lmg_status lmg_form_set(lmg_ctx *c, int32_t form, int32_t fe_order, int32_t q_order,
                        const double *params, int32_t n_params, const double *elem_coef,
                        const double *nodal_f) {
  if (!c) return LMG_ERR_ARG;
  if (!c->n_dofs) return fail(c, LMG_ERR_STATE, "form_set: upload the dofmap first");
  if (form != LMG_POISSON && form != LMG_ELASTICITY && form != LMG_ADVDIFF)
    return fail(c, LMG_ERR_ARG, "form_set: unknown form");
  if ((form != LMG_ELASTICITY && c->n_vars != 1) || (form == LMG_ELASTICITY && c->n_vars != 3))
    return fail(c, LMG_ERR_ARG, "form_set: variable count does not match the form");
  int n_modes = 0;
  if (form == LMG_ADVDIFF) {
    if (!params || n_params < 2) return fail(c, LMG_ERR_ARG, "form_set: ADVDIFF needs {kappa, n_modes, modes}");
    n_modes = (int)params[1];
    if (n_modes < 0 || n_modes > GEN_MAX_MODES || n_params != 2 + 7 * n_modes)
      return fail(c, LMG_ERR_ARG, "form_set: ADVDIFF parameter count does not match n_modes");
  }
  cudaSetDevice(c->device);
  if (c->hier3 != (pattern_fe_dofs(c->elem_type, fe_order) > 0))
    return fail(c, LMG_ERR_STATE, "form_set: the dof lists were uploaded for another FE type");
  if (c->hier3) return hier3_form_set(c, form, q_order, elem_coef, nodal_f);
  const int family = (fe_order & LMG_HIERARCHIC) ? 1 : 0;
  fe_order &= 0xff;
  // HIERARCHIC SECOND on HEX27: the shapes follow the elements' orientation
  // pattern (cube_indices' face swaps), built here for a mesh whose elements
  // all share one pattern (build_cube meshes)
  double X8[8][3];
  const double *xp = nullptr;
  if (family == 1 && fe_order == 2 && c->elem_type == LMG_HEX27 && c->n_elem > 0) {
    uint64_t pat0 = 0;
    for (int64_t e = 0; e < c->n_elem; ++e) {
      double X[8][3];
      for (int a = 0; a < 8; ++a)
        for (int d = 0; d < 3; ++d) X[a][d] = c->h_xyz[(size_t)(3 * (int64_t)c->h_conn[(size_t)(e * c->npe + a)] + d)];
      const uint64_t p = hex27_p2_pattern(X);
      if (e == 0) {
        pat0 = p;
        std::copy(&X[0][0], &X[0][0] + 24, &X8[0][0]);
      } else if (p != pat0) {
        return fail(c, LMG_ERR_UNSUPPORTED,
                    "form_set: HIERARCHIC SECOND on HEX27 needs one element orientation pattern per mesh", e);
      }
    }
    xp = &X8[0][0];
  }
  FETables t;
  std::string err = build_fe_tables(t, c->elem_type, fe_order, q_order, family, xp);
  if (!err.empty()) return fail(c, LMG_ERR_UNSUPPORTED, "form_set: " + err);
  if (t.n != c->npe || t.n_geo != c->npe)
    return fail(c, LMG_ERR_UNSUPPORTED, "form_set: only isoparametric LAGRANGE elements are built");
  if (t.q > 27) return fail(c, LMG_ERR_UNSUPPORTED, "form_set: more than 27 quadrature points");
  const bool general = c->has_rows || form == LMG_ADVDIFF;
  if (general) {
    if (!gen_elements_built(form, t.n, t.q))
      return fail(c, LMG_ERR_UNSUPPORTED, "form_set: no general-path kernel for this form / element / rule");
    if (!c->h_gen.empty())
      return fail(c, LMG_ERR_UNSUPPORTED, "form_set: the constrained / convection path takes affine elements only");
  } else {
    if (c->bs != c->n_vars)
      return fail(c, LMG_ERR_UNSUPPORTED, "form_set: variables must be node-interleaved (one VariableGroup)");
    if (!elements_built(form, t.n, c->n_vars))
      return fail(c, LMG_ERR_UNSUPPORTED, "form_set: no element kernel for this form / element");
  }
  if (c->n_vars == 1) {  // symmetrized reference tensors of the general path
    const int n = t.n;
    std::vector<double> D((size_t)6 * n * n);
    auto S = [&](int m, int k, int a, int b) { return t.S[(((size_t)(3 * m + k) * n) + a) * n + b]; };
    const int pm[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
    for (int k = 0; k < 6; ++k)
      for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) {
          const int m0 = pm[k][0], m1 = pm[k][1];
          D[((size_t)k * n + a) * n + b] = (m0 == m1) ? S(m0, m0, a, b) : S(m0, m1, a, b) + S(m1, m0, a, b);
        }
    // 1-D shapes at the 1-D Gauss points of a tensor hex rule: L1[i][q1]
    if (general && (c->elem_type == LMG_HEX8 || c->elem_type == LMG_HEX27)) {
      const int q1n = (t.q == 8) ? 2 : 3, n1 = (n == 8) ? 2 : 3;
      bool tensor = q1n * q1n * q1n == t.q;
      for (int q = 0; q < t.q && tensor; ++q) {
        const int id[3] = {q % q1n, (q / q1n) % q1n, q / (q1n * q1n)};
        for (int d = 0; d < 3; ++d) tensor = tensor && t.qp[3 * q + d] == t.qp[3 * id[d]];
      }
      // symmetric 1-D points: -g, +g (two) or -g, 0, +g (three)
      tensor = tensor && t.qp[0] == -t.qp[3 * (q1n - 1)] && t.qp[0] < 0.0 && (q1n == 2 || t.qp[3] == 0.0);
      if (!tensor) return fail(c, LMG_ERR_UNSUPPORTED, "form_set: the convection kernel needs a tensor Gauss rule");
      for (int i = 0; i < n1; ++i)
        for (int q1 = 0; q1 < q1n; ++q1) {
          const double x = t.qp[3 * q1];
          double v;
          if (n1 == 2) v = i == 0 ? .5 * (1. - x) : .5 * (1. + x);
          else if (family == 1) v = i == 0 ? .5 * (1. - x) : (i == 1 ? .5 * (1. + x) : (x * x - 1.) / 2.);
          else v = i == 0 ? .5 * x * (x - 1.) : (i == 1 ? .5 * x * (x + 1.) : (1. - x) * (1. + x));
          D.push_back(v);
        }
      D.push_back(t.qp[3 * (q1n - 1)]);  // outer 1-D Gauss point
    }
    LMG_CUDA(c, dupload(c, c->d_D6, D.data(), D.size()));
  }
  c->kappa = form == LMG_ADVDIFF ? params[0] : 0.0;
  c->n_modes = n_modes;
  dfree(c->d_modes);
  if (n_modes) LMG_CUDA(c, dupload(c, c->d_modes, params + 2, (size_t)(7 * n_modes)));
  if (general != c->general) c->gen_plan = false;
  c->general = general;
  c->tab = t;
  c->form = form;
  c->fe_order = fe_order;
  c->q_order = q_order;
  c->nu = (form == LMG_ELASTICITY && params && n_params > 0) ? params[0] : 0.3;
  std::vector<double> buf;
  auto put = [&](const std::vector<double> &v) { size_t o = buf.size(); buf.insert(buf.end(), v.begin(), v.end()); return o; };
  const size_t oqw = put(t.qw), ophi = put(t.phi), odphi = put(t.dphi), ogd = put(t.gdphi),
               oS = put(t.S), oM = put(t.M), ogp = put(t.gphi);
  LMG_CUDA(c, dupload(c, c->d_tab, buf.data(), buf.size()));
  c->dfe.n = t.n;
  c->dfe.q = t.q;
  c->dfe.n_geo = t.n_geo;
  c->dfe.qw = c->d_tab + oqw;
  c->dfe.phi = c->d_tab + ophi;
  c->dfe.dphi = c->d_tab + odphi;
  c->dfe.gdphi = c->d_tab + ogd;
  c->dfe.S = c->d_tab + oS;
  c->dfe.M = c->d_tab + oM;
  c->dfe.gphi = c->d_tab + ogp;
  dfree(c->d_coef);
  dfree(c->d_f);
  if (elem_coef) LMG_CUDA(c, dupload(c, c->d_coef, elem_coef, (size_t)c->n_elem));
  dfree(c->d_f2);
  if (nodal_f) {
    LMG_CUDA(c, dupload(c, c->d_f, nodal_f, (size_t)(c->n_nodes * c->n_vars)));
    LMG_CUDA(c, dalloc(c->d_f2, (size_t)(c->n_nodes * c->n_vars)));
    k_split<<<grid_for(c, c->n_nodes * c->n_vars, 256), 256, 0, c->stream>>>(c->n_nodes * c->n_vars, c->d_f, c->d_f2);
    c->launches++;
  }
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  c->have_form = true;
  return LMG_OK;
}

lmg_status lmg_inputs_update(lmg_ctx *c, const double *xyz, const double *elem_coef,
                             const double *nodal_f) {
  if (!c) return LMG_ERR_ARG;
  if (!c->have_form) return fail(c, LMG_ERR_STATE, "inputs_update: set the form first");
  cudaSetDevice(c->device);
  if (xyz) {
    c->h_xyz.assign(xyz, xyz + 3 * c->n_nodes);
    build_lists(c);
    LMG_CUDA(c, cudaMemcpyAsync(c->d_xyz, xyz, sizeof(double) * 3 * c->n_nodes, cudaMemcpyHostToDevice, c->stream));
    LMG_CUDA(c, dupload(c, c->d_aff, c->h_aff.data(), c->h_aff.size()));
    LMG_CUDA(c, dupload(c, c->d_gen, c->h_gen.data(), c->h_gen.size()));
  }
  if (elem_coef) {
    if (!c->d_coef) LMG_CUDA(c, dalloc(c->d_coef, (size_t)c->n_elem));
    LMG_CUDA(c, cudaMemcpyAsync(c->d_coef, elem_coef, sizeof(double) * c->n_elem, cudaMemcpyHostToDevice, c->stream));
  }
  if (nodal_f) {
    if (!c->d_f) LMG_CUDA(c, dalloc(c->d_f, (size_t)(c->n_nodes * c->n_vars)));
    if (!c->d_f2) LMG_CUDA(c, dalloc(c->d_f2, (size_t)(c->n_nodes * c->n_vars)));
    LMG_CUDA(c, cudaMemcpyAsync(c->d_f, nodal_f, sizeof(double) * c->n_nodes * c->n_vars, cudaMemcpyHostToDevice, c->stream));
    k_split<<<grid_for(c, c->n_nodes * c->n_vars, 256), 256, 0, c->stream>>>(c->n_nodes * c->n_vars, c->d_f, c->d_f2);
    c->launches++;
  }
  return LMG_OK;
}

lmg_status lmg_assemble(lmg_ctx *c, int32_t precision, double *K, double *F, int32_t out_on_device) {
  if (!c) return LMG_ERR_ARG;
  if (!c->have_sparsity) return fail(c, LMG_ERR_STATE, "assemble: build the sparsity first");
  if (!c->have_form) return fail(c, LMG_ERR_STATE, "assemble: set the form first");
  if (precision != LMG_FP64 && precision != LMG_MIXED) return fail(c, LMG_ERR_ARG, "assemble: unknown precision");
  cudaSetDevice(c->device);
  if (c->general) {
    const bool mixed = precision == LMG_MIXED;
    if (!c->gen_plan) {
      lmg_status st = general_plan(c);
      if (st) return st;
    }
    lmg_status st = reset_status(c);
    if (st) return st;
    cudaEvent_t e3[3] = {nullptr, nullptr, nullptr};
    if (c->perflog) {
      for (auto &e : e3) LMG_CUDA(c, cudaEventCreate(&e));
      for (auto &e : e3) c->ev.push_back(e);
      LMG_CUDA(c, cudaEventRecord(e3[0], c->stream));
    }
    general_assemble(c, mixed);
    if (c->perflog) LMG_CUDA(c, cudaEventRecord(e3[1], c->stream));
    // host output of a large system: the insertion in row ranges, each
    // range's copy overlapping the next range's insertion (a refined mesh's
    // rows complete only once nearly every element has run, so the element
    // stage itself is not split)
    const bool chunked = K && !out_on_device && c->nnz * (int64_t)sizeof(double) > ((int64_t)64 << 20) &&
                         (int64_t)c->h_row_ptr.size() == c->n_dofs + 1;
    if (chunked) {
      if (!c->copy_stream) LMG_CUDA(c, cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
      while ((int)c->chunk_ev.size() < OUT_CHUNKS) {
        cudaEvent_t e;
        LMG_CUDA(c, cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        c->chunk_ev.push_back(e);
      }
      for (int ch = 0; ch < OUT_CHUNKS; ++ch) {
        const int64_t P0 = c->n_dofs * ch / OUT_CHUNKS, P1 = c->n_dofs * (ch + 1) / OUT_CHUNKS;
        if (P1 <= P0) continue;
        general_gather(c, mixed, P0, P1);
        LMG_CUDA(c, cudaEventRecord(c->chunk_ev[ch], c->stream));
        LMG_CUDA(c, cudaStreamWaitEvent(c->copy_stream, c->chunk_ev[ch], 0));
        const int64_t k0 = c->h_row_ptr[(size_t)P0], k1 = c->h_row_ptr[(size_t)P1];
        LMG_CUDA(c, cudaMemcpyAsync(K + k0, c->d_K + k0, sizeof(double) * (k1 - k0), cudaMemcpyDeviceToHost,
                                    c->copy_stream));
      }
    } else {
      general_gather(c, mixed);
    }
    if (c->perflog) LMG_CUDA(c, cudaEventRecord(e3[2], c->stream));
    LMG_CUDA(c, cudaGetLastError());
    const cudaMemcpyKind kind = out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (K && !chunked) LMG_CUDA(c, cudaMemcpyAsync(K, c->d_K, sizeof(double) * c->nnz, kind, c->stream));
    if (F) LMG_CUDA(c, cudaMemcpyAsync(F, c->d_F, sizeof(double) * c->n_dofs, kind, c->stream));
    if (chunked) LMG_CUDA(c, cudaStreamSynchronize(c->copy_stream));
    if (out_on_device || (!K && !F)) return LMG_OK;
    return check_status(c, "assemble");
  }
  const bool mixed = precision == LMG_MIXED;
  const bool fused = mixed && c->h_gen.empty() && c->d_relslot && fused_built(c->form, c->tab.n, c->n_vars) &&
                     fused_fits(c->tab.n, c->n_vars, c->max_bdeg);
  if (mixed && !fused && !c->d_Koff32)
    LMG_CUDA(c, dalloc(c->d_Koff32, (size_t)c->n_elem * c->nb * (c->nb - 1) / 2 * c->bs * c->bs));
  if (fused && !c->d_geo)
    LMG_CUDA(c, dalloc(c->d_geo, (size_t)c->n_elem * (c->form == LMG_POISSON ? 9 : 11)));
  if (fused && !c->d_rowcons) {
    LMG_CUDA(c, dalloc(c->d_rowcons, (size_t)std::max<int64_t>(c->n_blocks, 1)));
    k_rowcons<<<grid_for(c, c->n_blocks, 256), 256, 0, c->stream>>>(c->n_blocks, c->bs, c->d_brow_ptr, c->d_bcol,
                                                                   c->d_cons, c->d_rowcons);
    c->launches++;
  }
  if (!mixed && !c->d_Kdiag2) {
    const size_t b2 = (size_t)c->bs * c->bs, no = (size_t)c->nb * (c->nb - 1) / 2;
    LMG_CUDA(c, dalloc(c->d_Kdiag2, (size_t)c->n_elem * c->nb * b2));
    LMG_CUDA(c, dalloc(c->d_Koff2, (size_t)c->n_elem * no * b2));
  }
  lmg_status st = reset_status(c);
  if (st) return st;
  ElemArgs a{};
  a.npe = c->npe;
  a.xyz = c->d_xyz;
  a.conn = c->d_conn;
  a.coef = c->d_coef;
  a.nodal_f = c->d_f;
  a.nodal_f2 = c->d_f2;
  a.cmask = c->d_cmask;
  a.nu = c->nu;
  a.Kdiag2 = c->d_Kdiag2;
  a.Koff2 = c->d_Koff2;
  a.Koff32 = c->d_Koff32;
  a.Fe2 = c->d_Fe2;
  a.status = c->d_status;
  a.bad_elem = c->d_bad;
  a.fe = c->dfe;
  const int grid = c->n_sm * c->ctas_per_sm;  // grid-stride over the element lists
  cudaEvent_t e3[3] = {nullptr, nullptr, nullptr};
  if (c->perflog) {
    for (auto &e : e3) LMG_CUDA(c, cudaEventCreate(&e));
    for (auto &e : e3) c->ev.push_back(e);
    LMG_CUDA(c, cudaEventRecord(e3[0], c->stream));
  }
  if (fused) {  // mixed form, one row kernel: no element-block buffer
    // the row kernel's grid-stride loop balances best at 48 CTAs per SM on
    // the 48^3 TET10 mesh (1.58 against 1.65 ms at 32, 2.06 ms with a CTA
    // per eight rows) unless the caller set the grid
    const int fgrid = c->grid_set ? grid : c->n_sm * 48;
    FusedArgs f{};
    f.el = a;
    f.el.n_list = (int64_t)c->h_aff.size();
    f.el.list = c->d_aff;
    f.geo = c->d_geo;
    f.n_brows = c->n_blocks;
    f.brow_ptr = c->d_brow_ptr;
    f.bcol = c->d_bcol;
    f.row_ptr = c->d_row_ptr;
    f.fptr = c->d_fptr;
    f.fcontrib = c->d_fcontrib;
    f.relslot = c->d_relslot;
    f.constrained = c->d_cons;
    f.rowcons = c->d_rowcons;
    f.max_deg = c->max_bdeg;
    f.K = c->d_K;
    f.F = c->d_F;
    const bool chunked = chunked_output(c, K, out_on_device);
    if (chunked) {
      lmg_status cs = pipelined_copy(
          c, K,
          [&](int64_t E0, int64_t E1) {
            int64_t off, cnt;
            list_slice(c->h_aff, E0, E1, off, cnt);
            if (cnt == 0) return;
            FusedArgs fg = f;
            fg.el.list = c->d_aff + off;
            fg.el.n_list = cnt;
            launch_fused_mixed(c->form, c->tab.n, c->n_vars, fg, fgrid, c->stream, true, false);
            c->launches++;
          },
          [&](int64_t P0, int64_t P1) {
            FusedArgs fc = f;
            fc.row_begin = P0;
            fc.n_brows = P1;
            launch_fused_mixed(c->form, c->tab.n, c->n_vars, fc, fgrid, c->stream, false, true);
            c->launches += 2;  // row kernel, load vector
          });
      if (cs) return cs;
    } else {
      launch_fused_mixed(c->form, c->tab.n, c->n_vars, f, fgrid, c->stream, true, true);
      c->launches += 3;  // operands, row kernel, load vector
    }
    if (c->perflog) {
      LMG_CUDA(c, cudaEventRecord(e3[1], c->stream));
      LMG_CUDA(c, cudaEventRecord(e3[2], c->stream));
    }
    LMG_CUDA(c, cudaGetLastError());
    const cudaMemcpyKind kind = out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    if (K && !chunked) LMG_CUDA(c, cudaMemcpyAsync(K, c->d_K, sizeof(double) * c->nnz, kind, c->stream));
    if (F) LMG_CUDA(c, cudaMemcpyAsync(F, c->d_F, sizeof(double) * c->n_dofs, kind, c->stream));
    if (chunked) LMG_CUDA(c, cudaStreamSynchronize(c->copy_stream));
    if (out_on_device || (!K && !F)) return LMG_OK;
    return check_status(c, "assemble");
  }
  // element kernels over the elements [E0, E1) of both lists
  auto run_elements = [&](int64_t E0, int64_t E1) {
    int64_t off, cnt;
    list_slice(c->h_aff, E0, E1, off, cnt);
    if (cnt) {
      ElemArgs aa = a;
      aa.n_list = cnt;
      aa.list = c->d_aff + off;
      launch_elements(c->form, c->tab.n, c->n_vars, true, mixed, aa, grid, c->stream);
      c->launches++;
    }
    list_slice(c->h_gen, E0, E1, off, cnt);
    if (cnt) {
      ElemArgs aa = a;
      aa.n_list = cnt;
      aa.list = c->d_gen + off;
      // mixed form: the per-point B^T D B products on the tensor cores where built
      const bool later_neg = std::any_of(c->tab.qw.begin() + 1, c->tab.qw.end(), [](double x) { return x < 0.0; });
      if (!(mixed && c->tensor_cores && !later_neg && tc_built(c->form, c->tab.n, c->n_vars, c->tab.q) &&
            launch_elements_tc(c->form, c->tab.n, c->n_vars, c->tab.q, c->tab.qw[0] < 0.0, aa, c->n_sm,
                               c->stream)))
        launch_elements(c->form, c->tab.n, c->n_vars, false, mixed, aa, grid, c->stream);
      c->launches++;
    }
  };
  const bool chunked = chunked_output(c, K, out_on_device);
  if (!chunked) run_elements(0, c->n_elem);
  if (c->perflog) LMG_CUDA(c, cudaEventRecord(e3[1], c->stream));
  GatherArgs g{};
  g.n_dofs = c->n_dofs;
  g.bs = c->bs;
  g.nb = c->nb;
  g.brow_ptr = c->d_brow_ptr;
  g.row_ptr = c->d_row_ptr;
  g.bcol = c->d_bcol;
  g.bptr = c->d_bptr;
  g.bdiag = c->d_bdiag;
  g.bcontrib = c->d_bcontrib;
  g.no = c->nb * (c->nb - 1) / 2;
  g.fptr = c->d_fptr;
  g.fcontrib = c->d_fcontrib;
  g.Kdiag2 = c->d_Kdiag2;
  g.Koff2 = c->d_Koff2;
  g.Koff32 = c->d_Koff32;
  g.Fe2 = c->d_Fe2;
  g.constrained = c->d_cons;
  g.K = c->d_K;
  g.F = c->d_F;
  if (chunked) {
    lmg_status cs = pipelined_copy(c, K, run_elements, [&](int64_t P0, int64_t P1) {
      GatherArgs gc = g;
      gc.row_begin = P0;
      gc.row_end = P1;
      launch_gather(gc, mixed, c->stream);
      c->launches += 2;  // insertion, load vector
    });
    if (cs) return cs;
  } else {
    launch_gather(g, mixed, c->stream);
    c->launches += 2;  // insertion, load vector
  }
  if (c->perflog) LMG_CUDA(c, cudaEventRecord(e3[2], c->stream));
  LMG_CUDA(c, cudaGetLastError());
  const cudaMemcpyKind kind = out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (K && !chunked) LMG_CUDA(c, cudaMemcpyAsync(K, c->d_K, sizeof(double) * c->nnz, kind, c->stream));
  if (F) LMG_CUDA(c, cudaMemcpyAsync(F, c->d_F, sizeof(double) * c->n_dofs, kind, c->stream));
  if (chunked) LMG_CUDA(c, cudaStreamSynchronize(c->copy_stream));
  // Device outputs stay asynchronous; lmg_synchronize reports their status.
  if (out_on_device || (!K && !F)) return LMG_OK;
  return check_status(c, "assemble");
}

lmg_status lmg_synchronize(lmg_ctx *c) {
  if (!c) return LMG_ERR_ARG;
  cudaSetDevice(c->device);
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  return check_status(c, "assemble");
}

lmg_status lmg_result_device(lmg_ctx *c, double **K, double **F) {
  if (!c) return LMG_ERR_ARG;
  if (K) *K = c->d_K;
  if (F) *F = c->d_F;
  return LMG_OK;
}

lmg_status lmg_result_copy(lmg_ctx *c, double *K, double *F) {
  if (!c) return LMG_ERR_ARG;
  if (!c->have_sparsity) return fail(c, LMG_ERR_STATE, "result_copy: nothing assembled");
  cudaSetDevice(c->device);
  if (K) LMG_CUDA(c, cudaMemcpyAsync(K, c->d_K, sizeof(double) * c->nnz, cudaMemcpyDeviceToHost, c->stream));
  if (F) LMG_CUDA(c, cudaMemcpyAsync(F, c->d_F, sizeof(double) * c->n_dofs, cudaMemcpyDeviceToHost, c->stream));
  return check_status(c, "result_copy");
}

lmg_status lmg_last_error(lmg_ctx *c, int64_t *elem_id, char *msg, int32_t msg_len) {
  if (!c) return LMG_ERR_ARG;
  if (elem_id) *elem_id = c->err_elem;
  if (msg && msg_len > 0) {
    std::strncpy(msg, c->err.c_str(), (size_t)msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  return LMG_OK;
}

namespace {
VjpArgs vjp_args(lmg_ctx *c) {
  VjpArgs v{};
  v.n_elem = c->n_elem;
  v.xyz = c->d_xyz;
  v.conn = c->d_conn;
  v.eb = c->d_eb;
  v.nu = c->nu;
  v.status = c->d_status;
  v.bad_elem = c->d_bad;
  v.cmask = c->d_cmask;
  v.fe = c->dfe;
  return v;
}
}  // namespace

lmg_status lmg_qoi_region_load(lmg_ctx *c, const uint8_t *in_region, double *q) {
  if (c && c->general)
    return fail(c, LMG_ERR_UNSUPPORTED, "adjoint sensitivities are built for the unconstrained symmetric forms");
  if (!c || !in_region || !q) return fail(c, LMG_ERR_ARG, "qoi_region_load: bad argument");
  if (!c->have_sparsity || !c->have_form) return fail(c, LMG_ERR_STATE, "qoi_region_load: set up the system first");
  cudaSetDevice(c->device);
  uint8_t *d_reg = nullptr;
  LMG_CUDA(c, dupload(c, d_reg, in_region, (size_t)c->n_elem));
  lmg_status st = reset_status(c);
  if (st) return st;
  VjpArgs v = vjp_args(c);
  v.region = d_reg;
  v.Fe2 = c->d_Fe2;
  launch_vjp(c->form, c->tab.n, c->n_vars, true, v, c->n_sm * 8, c->stream);
  GatherArgs g{};
  g.n_dofs = c->n_dofs;
  g.bs = c->bs;
  g.fptr = c->d_fptr;
  g.fcontrib = c->d_fcontrib;
  g.Fe2 = c->d_Fe2;
  double *d_q = nullptr;
  LMG_CUDA(c, dalloc(d_q, (size_t)c->n_dofs));
  g.F = d_q;
  launch_gather_f(g, c->stream);
  c->launches += 2;
  LMG_CUDA(c, cudaGetLastError());
  LMG_CUDA(c, cudaMemcpyAsync(q, d_q, sizeof(double) * c->n_dofs, cudaMemcpyDeviceToHost, c->stream));
  st = check_status(c, "qoi_region_load");
  dfree(d_reg);
  dfree(d_q);
  return st;
}

lmg_status lmg_vjp_coef(lmg_ctx *c, const double *u, const double *z, double *dq_dcoef) {
  if (c && c->general)
    return fail(c, LMG_ERR_UNSUPPORTED, "adjoint sensitivities are built for the unconstrained symmetric forms");
  if (!c || !u || !z || !dq_dcoef) return fail(c, LMG_ERR_ARG, "vjp_coef: bad argument");
  if (!c->have_sparsity || !c->have_form) return fail(c, LMG_ERR_STATE, "vjp_coef: set up the system first");
  cudaSetDevice(c->device);
  double *du = nullptr, *dz = nullptr, *dout = nullptr;
  LMG_CUDA(c, dupload(c, du, u, (size_t)c->n_dofs));
  LMG_CUDA(c, dupload(c, dz, z, (size_t)c->n_dofs));
  LMG_CUDA(c, dalloc(dout, (size_t)c->n_elem));
  lmg_status st = reset_status(c);
  if (st) return st;
  VjpArgs v = vjp_args(c);
  v.u = du;
  v.z = dz;
  v.out = dout;
  launch_vjp(c->form, c->tab.n, c->n_vars, false, v, c->n_sm * 8, c->stream);
  c->launches++;
  LMG_CUDA(c, cudaGetLastError());
  LMG_CUDA(c, cudaMemcpyAsync(dq_dcoef, dout, sizeof(double) * c->n_elem, cudaMemcpyDeviceToHost, c->stream));
  st = check_status(c, "vjp_coef");
  dfree(du);
  dfree(dz);
  dfree(dout);
  return st;
}

lmg_status lmg_residual(lmg_ctx *c, const double *u, double *R, int32_t on_device) {
  if (!c || !u || !R) return fail(c, LMG_ERR_ARG, "residual: bad argument");
  if (!c->have_sparsity || !c->have_form) return fail(c, LMG_ERR_STATE, "residual: set up the system first");
  if (c->general || !c->h_gen.empty())
    return fail(c, LMG_ERR_UNSUPPORTED, "residual: built for affine elements of the block path");
  cudaSetDevice(c->device);
  if (!c->d_Re2) LMG_CUDA(c, dalloc(c->d_Re2, (size_t)(c->n_elem * c->nl)));
  double *du = nullptr, *dR = nullptr;
  if (on_device) {
    du = const_cast<double *>(u);
    dR = R;
  } else {
    LMG_CUDA(c, dalloc(du, (size_t)c->n_dofs));
    LMG_CUDA(c, dalloc(dR, (size_t)c->n_dofs));
    LMG_CUDA(c, cudaMemcpyAsync(du, u, sizeof(double) * c->n_dofs, cudaMemcpyHostToDevice, c->stream));
  }
  lmg_status st = reset_status(c);
  if (st) return st;
  ElemArgs a{};
  a.n_list = (int64_t)c->h_aff.size();
  a.list = c->d_aff;
  a.npe = c->npe;
  a.xyz = c->d_xyz;
  a.conn = c->d_conn;
  a.coef = c->d_coef;
  a.nodal_f = c->d_f;
  a.nodal_f2 = c->d_f2;
  a.cmask = c->d_cmask;
  a.nu = c->nu;
  a.status = c->d_status;
  a.bad_elem = c->d_bad;
  a.fe = c->dfe;
  a.eb = c->d_eb;
  a.u = du;
  a.Re2 = c->d_Re2;
  if (!launch_residual(c->form, c->tab.n, c->n_vars, a, c->n_blocks, c->d_fptr, c->d_fcontrib, dR,
                       c->n_sm * c->ctas_per_sm, c->stream))
    return fail(c, LMG_ERR_UNSUPPORTED, "residual: no kernel for this form / element");
  c->launches += 2;
  LMG_CUDA(c, cudaGetLastError());
  if (on_device) return LMG_OK;
  LMG_CUDA(c, cudaMemcpyAsync(R, dR, sizeof(double) * c->n_dofs, cudaMemcpyDeviceToHost, c->stream));
  st = check_status(c, "residual");
  dfree(du);
  dfree(dR);
  return st;
}

lmg_status lmg_vjp_xyz(lmg_ctx *c, const double *u, const double *z, const uint8_t *in_region, double *dq_dxyz) {
  if (!c || !u || !z || !dq_dxyz) return fail(c, LMG_ERR_ARG, "vjp_xyz: bad argument");
  if (c->general || !((c->form == LMG_POISSON && c->n_vars == 1) || (c->form == LMG_ELASTICITY && c->n_vars == 3)) ||
      c->bs != c->n_vars)
    return fail(c, LMG_ERR_UNSUPPORTED, "vjp_xyz: built for the Poisson and elasticity forms");
  if (!c->have_sparsity || !c->have_form) return fail(c, LMG_ERR_STATE, "vjp_xyz: set up the system first");
  cudaSetDevice(c->device);
  double *du = nullptr, *dz = nullptr, *dx = nullptr, *drow = nullptr;
  uint8_t *dreg = nullptr;
  LMG_CUDA(c, dupload(c, du, u, (size_t)c->n_dofs));
  LMG_CUDA(c, dupload(c, dz, z, (size_t)c->n_dofs));
  if (in_region) LMG_CUDA(c, dupload(c, dreg, in_region, (size_t)c->n_elem));
  LMG_CUDA(c, dalloc(dx, (size_t)c->n_elem * c->npe * 3));
  LMG_CUDA(c, dalloc(drow, (size_t)c->n_blocks * 3));
  lmg_status st = reset_status(c);
  if (st) return st;
  VjpArgs v = vjp_args(c);
  v.u = du;
  v.z = dz;
  v.region = dreg;
  v.coef = c->d_coef;
  v.nodal_f = c->d_f;
  v.xout = dx;
  v.n_rows = c->n_blocks;
  v.fptr = c->d_fptr;
  v.fcontrib = c->d_fcontrib;
  v.row_out = drow;
  if (!launch_vjp_xyz(c->form, c->tab.n, v, c->n_sm * 8, c->stream))
    return fail(c, LMG_ERR_UNSUPPORTED, "vjp_xyz: element not built");
  c->launches += 2;
  LMG_CUDA(c, cudaGetLastError());
  std::vector<double> row((size_t)c->n_blocks * 3);
  LMG_CUDA(c, cudaMemcpyAsync(row.data(), drow, sizeof(double) * row.size(), cudaMemcpyDeviceToHost, c->stream));
  st = check_status(c, "vjp_xyz");
  dfree(du); dfree(dz); dfree(dreg); dfree(dx); dfree(drow);
  if (st) return st;
  std::fill(dq_dxyz, dq_dxyz + 3 * c->n_nodes, 0.0);
  for (int64_t e = 0; e < c->n_elem; ++e)  // node of every block row
    for (int a = 0; a < c->npe; ++a) {
      const int64_t node = c->h_conn[(size_t)(e * c->npe + a)], blk = c->h_eb[(size_t)(e * c->nb + a)];
      for (int d = 0; d < 3; ++d) dq_dxyz[3 * node + d] = row[(size_t)(3 * blk + d)];
    }
  return LMG_OK;
}

lmg_status lmg_cg_solve(lmg_ctx *c, const double *rhs, double *x, double rtol, int32_t maxit,
                        int32_t *iters, double *relres) {
  if (!c || !x || rtol <= 0 || maxit <= 0) return fail(c, LMG_ERR_ARG, "cg_solve: bad argument");
  if (!c->have_sparsity) return fail(c, LMG_ERR_STATE, "cg_solve: assemble first");
  cudaSetDevice(c->device);
  struct Bufs {  // the solution and right-hand side on the device, freed on every return path
    double *dx = nullptr, *db = nullptr;
    ~Bufs() { dfree(dx); dfree(db); }
  } w;
  double *b = c->d_F;
  LMG_CUDA(c, dalloc(w.dx, (size_t)c->n_dofs));
  if (rhs) {
    LMG_CUDA(c, dupload(c, w.db, rhs, (size_t)c->n_dofs));
    b = w.db;
  }
  int it = 0;
  double rr = 0.0;
  const int st = cg_solve(c->n_dofs, c->d_row_ptr, c->d_col, c->d_K, b, w.dx, rtol, maxit, c->stream, c->n_sm,
                          &it, &rr, &c->launches);
  if (st == 0)
    LMG_CUDA(c, cudaMemcpyAsync(x, w.dx, sizeof(double) * c->n_dofs, cudaMemcpyDeviceToHost, c->stream));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  if (st == 3) return fail(c, LMG_ERR_ARG, "cg_solve: the right-hand side is not finite");
  if (st) return fail(c, st == 7 ? LMG_ERR_OOM : LMG_ERR_CUDA, "cg_solve: device failure");
  if (iters) *iters = it;
  if (relres) *relres = rr;
  return LMG_OK;
}

lmg_status lmg_context_set_tensor_cores(lmg_ctx *c, int32_t on) {
  if (!c) return LMG_ERR_ARG;
  c->tensor_cores = on != 0;
  return LMG_OK;
}

lmg_status lmg_perflog_enable(lmg_ctx *c, int32_t on) {
  if (!c) return LMG_ERR_ARG;
  c->perflog = on != 0;
  return LMG_OK;
}

lmg_status lmg_perflog_read(lmg_ctx *c, double *elements_ms, double *gather_ms, int64_t *calls) {
  if (!c) return LMG_ERR_ARG;
  cudaSetDevice(c->device);
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  for (size_t i = 0; i + 2 < c->ev.size(); i += 3) {
    float a = 0, b = 0;
    LMG_CUDA(c, cudaEventElapsedTime(&a, c->ev[i], c->ev[i + 1]));
    LMG_CUDA(c, cudaEventElapsedTime(&b, c->ev[i + 1], c->ev[i + 2]));
    c->log_ms[0] += a;
    c->log_ms[1] += b;
    c->log_calls++;
  }
  for (auto e : c->ev) cudaEventDestroy(e);
  c->ev.clear();
  if (elements_ms) *elements_ms = c->log_ms[0];
  if (gather_ms) *gather_ms = c->log_ms[1];
  if (calls) *calls = c->log_calls;
  c->log_ms[0] = c->log_ms[1] = 0.0;
  c->log_calls = 0;
  return LMG_OK;
}

lmg_status lmg_context_set_grid(lmg_ctx *c, int32_t ctas_per_sm) {
  if (!c || ctas_per_sm < 0 || ctas_per_sm > 64) return fail(c, LMG_ERR_ARG, "set_grid: 0 (default) .. 64");
  c->ctas_per_sm = ctas_per_sm ? ctas_per_sm : 32;
  c->grid_set = ctas_per_sm != 0;
  return LMG_OK;
}

lmg_status lmg_launch_count(lmg_ctx *c, int64_t *count) {
  if (!c || !count) return LMG_ERR_ARG;
  *count = c->launches;
  return LMG_OK;
}

}  // extern "C"
