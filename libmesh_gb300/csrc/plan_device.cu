// The general path's insertion plan built on the device: the same arrays,
// bit for bit, as the host build in context_general.cu (general_plan).
//
// libMesh constrains each element's matrix through the element's constraint
// matrix (DofMap::build_constraint_matrix, src/base/dof_map_constraints.C:
// 3433-3540): the element's own dofs, then the dofs their constraint rows
// refer to that are not among them, ascending; column q of C holds, for each
// own dof i in ascending order, 1 when i = q is unconstrained and the
// coefficient of dofs[q] in the row of a constrained i (zeros skipped).  The
// constrained element matrices then add into the CSR in element order
// (PetscMatrix::add_matrix, src/numerics/petsc_matrix.C:735-755), which the
// slot plan records: per CSR slot the offsets of its element entries in
// element order.
//
// Steps: a warp per element sizes its dof list and its constraint matrix
// (pass 0), scans give every offset, a warp per element writes the lists and
// the columns of C (pass 1); the incidences of each dof are counted,
// scanned, filled and sorted into element order; a thread per dof row counts
// and then fills its slots' contributions by binary search in the row's
// columns; a thread per incidence gives the load vector's offsets.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>
#include <vector>

#include "context_internal.cuh"
#include "general.cuh"

namespace lmg {

namespace {

constexpr int PW = 4;       // warps per CTA of the element passes
constexpr int PCAP = 1024;  // candidate constraining dofs of one element
constexpr unsigned FULLM = 0xffffffffu;

struct PlanIn {
  int64_t E;
  int N;
  const int32_t *ed;     // [E][N] element dofs
  const uint8_t *cons;   // [n_dofs] constrained flags, or null (no element takes the constraint path)
  const int64_t *cp;     // [n_dofs + 1] constraint rows
  const int32_t *ccol;   // their columns (ascending per row)
  const double *cval;    // their coefficients
};

__device__ __forceinline__ bool is_cons(const PlanIn &in, int32_t d) { return in.cons && in.cons[d] != 0; }

// The element's dof list in `dofs` (own dofs, then the constraining dofs not
// among them, ascending) and whether any own dof is constrained; returns the
// list length, or -1 when the candidates outgrow the buffer.
__device__ int element_list(const PlanIn &in, int64_t e, int32_t *cand, int32_t *dofs, int lane, bool &any) {
  const int N = in.N;
  bool mine = false;
  for (int i = lane; i < N; i += 32) {
    const int32_t d = in.ed[e * N + i];
    dofs[i] = d;
    mine |= is_cons(in, d);
  }
  any = __any_sync(FULLM, mine);
  __syncwarp();
  if (!any) return N;
  // the columns of the constrained own dofs' rows
  int nc = 0;
  for (int i = 0; i < N; ++i) {
    const int32_t d = dofs[i];
    if (!is_cons(in, d)) continue;
    const int64_t r0 = in.cp[d], r1 = in.cp[d + 1];
    const int len = (int)(r1 - r0);
    if (nc + len > PCAP) return -1;
    for (int j = lane; j < len; j += 32) cand[nc + j] = in.ccol[r0 + j];
    nc += len;
  }
  __syncwarp();
  int S = 1;
  while (S < nc) S <<= 1;
  for (int t = nc + lane; t < S; t += 32) cand[t] = 0x7fffffff;
  __syncwarp();
  for (int k = 2; k <= S; k <<= 1)
    for (int j = k >> 1; j > 0; j >>= 1) {
      for (int t = lane; t < S; t += 32) {
        const int u = t ^ j;
        if (u > t) {
          const int32_t x = cand[t], y = cand[u];
          if ((x > y) == ((t & k) == 0)) {
            cand[t] = y;
            cand[u] = x;
          }
        }
      }
      __syncwarp();
    }
  // distinct candidates that are not own dofs, ascending, after the own dofs
  int ne = N;
  for (int t0 = 0; t0 < S; t0 += 32) {
    const int t = t0 + lane;
    bool keep = t < nc && (t == 0 || cand[t] != cand[t - 1]);
    if (keep)
      for (int i = 0; i < N; ++i)
        if (dofs[i] == cand[t]) keep = false;
    const unsigned m = __ballot_sync(FULLM, keep);
    const int pos = ne + __popc(m & ((1u << lane) - 1u));
    if (keep && pos < GEN_MAX_NE) dofs[pos] = cand[t];
    ne += __popc(m);
  }
  __syncwarp();
  return ne;
}

// Entries of column q of the element's constraint matrix: (own row i, value)
// for i ascending; calls put(i, v) for each and returns the count.
template <typename Put>
__device__ __forceinline__ int column_entries(const PlanIn &in, const int32_t *dofs, int q, Put &&put) {
  const int N = in.N;
  const int32_t dq = dofs[q];
  int n = 0;
  for (int i = 0; i < N; ++i) {
    const int32_t d = dofs[i];
    if (!is_cons(in, d)) {
      if (i == q) {
        put(i, 1.0);
        ++n;
      }
      continue;
    }
    for (int64_t k = in.cp[d]; k < in.cp[d + 1]; ++k)
      if (in.ccol[k] == dq) {
        const double v = in.cval[k];
        if (v != 0.0) {
          put(i, v);
          ++n;
        }
        break;
      }
  }
  return n;
}

// Pass 0: list length, constraint-matrix entries and whether constrained.
__global__ void __launch_bounds__(PW * 32) k_plan_sizes(PlanIn in, int32_t *ne_out, int32_t *nent_out,
                                                        int32_t *iscons, int *flag) {
  __shared__ int32_t s_cand[PW][PCAP];
  __shared__ int32_t s_dofs[PW][GEN_MAX_NE];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t e = (int64_t)blockIdx.x * PW + warp; e < in.E; e += (int64_t)gridDim.x * PW) {
    bool any = false;
    const int ne = element_list(in, e, s_cand[warp], s_dofs[warp], lane, any);
    int nent = 0;
    if (ne < 0 || ne > GEN_MAX_NE) {
      if (lane == 0) atomicOr(flag, 1);
    } else if (any) {
      for (int q = lane; q < ne; q += 32) nent += column_entries(in, s_dofs[warp], q, [](int, double) {});
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) nent += __shfl_xor_sync(FULLM, nent, o);
      if (nent > GEN_MAX_ENTRIES && lane == 0) atomicOr(flag, 2);
    }
    if (lane == 0) {
      ne_out[e] = ne < 0 ? in.N : ne;
      nent_out[e] = any ? nent : 0;
      iscons[e] = any ? 1 : 0;
    }
    __syncwarp();
  }
}

// The element regions: raw elements at e*N^2 / e*N, constrained ones after
// E*N^2 / E*N in element order; the constrained elements' records.
__global__ void k_plan_bases(PlanIn in, const int32_t *ne, const int32_t *nent, const int32_t *iscons,
                             const int64_t *ksc, const int64_t *fsc, const int64_t *psc, const int64_t *esc,
                             const int64_t *csc, int64_t *kbase, int64_t *fbase, int32_t *celem, int32_t *cne,
                             int64_t *ckout, int64_t *cfout, int64_t *cbase, int64_t *cebase) {
  const int64_t N = in.N;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < in.E; e += (int64_t)gridDim.x * blockDim.x) {
    if (!iscons[e]) {
      kbase[e] = e * N * N;
      fbase[e] = e * N;
      continue;
    }
    const int64_t k = in.E * N * N + ksc[e], f = in.E * N + fsc[e], c = csc[e];
    kbase[e] = k;
    fbase[e] = f;
    celem[c] = (int32_t)e;
    cne[c] = ne[e];
    ckout[c] = k;
    cfout[c] = f;
    cbase[c] = psc[e];
    cebase[c] = esc[e];
    (void)nent;
  }
}

// Pass 1: the dof lists and the columns of the constraint matrices.
__global__ void __launch_bounds__(PW * 32) k_plan_fill(PlanIn in, const int64_t *lptr, const int32_t *iscons,
                                                       const int64_t *csc, const int64_t *cbase,
                                                       const int64_t *cebase, int32_t *ldofs, int32_t *ccp,
                                                       uint8_t *cci, double *ccv, uint64_t *crow) {
  __shared__ int32_t s_cand[PW][PCAP];
  __shared__ int32_t s_dofs[PW][GEN_MAX_NE];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  for (int64_t e = (int64_t)blockIdx.x * PW + warp; e < in.E; e += (int64_t)gridDim.x * PW) {
    bool any = false;
    const int ne = element_list(in, e, s_cand[warp], s_dofs[warp], lane, any);
    const int32_t *dofs = s_dofs[warp];
    for (int q = lane; q < ne; q += 32) ldofs[lptr[e] + q] = dofs[q];
    if (iscons[e]) {
      const int64_t c = csc[e], pb = cbase[c], eb = cebase[c];
      // column starts: exclusive scan of the columns' entry counts, 32 columns at a time
      int carry = 0;
      for (int q0 = 0; q0 < ne; q0 += 32) {
        const int q = q0 + lane;
        const int n = q < ne ? column_entries(in, dofs, q, [](int, double) {}) : 0;
        int x = n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(FULLM, x, o);
          if (lane >= o) x += y;
        }
        const int start = carry + x - n;
        if (q < ne) {
          ccp[pb + q] = start;
          int w = 0;
          column_entries(in, dofs, q, [&](int i, double v) {
            cci[eb + start + w] = (uint8_t)i;
            ccv[eb + start + w] = v;
            ++w;
          });
        }
        carry += __shfl_sync(FULLM, x, 31);
      }
      if (lane == 0) ccp[pb + ne] = carry;
      uint64_t rows = 0;
      for (int i = 0; i < in.N; ++i)
        if (is_cons(in, dofs[i])) rows |= 1ull << i;
      if (lane == 0) crow[c] = rows;
    }
    __syncwarp();
  }
}

__global__ void k_inc_count(int64_t n, const int32_t *ldofs, int32_t *cnt) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    atomicAdd(&cnt[ldofs[t]], 1);
}

// (element, position) of every list entry, keyed e * 256 + position
__global__ void k_inc_fill(int64_t E, const int64_t *lptr, const int32_t *ldofs, const int64_t *iptr, int32_t *cur,
                           int32_t *key) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += (int64_t)gridDim.x * blockDim.x)
    for (int64_t k = lptr[e]; k < lptr[e + 1]; ++k) {
      const int32_t d = ldofs[k];
      key[iptr[d] + atomicAdd(&cur[d], 1)] = (int32_t)(e * 256 + (k - lptr[e]));
    }
}

__global__ void k_seg_sort64(int64_t n_seg, const int64_t *ptr, int32_t *v) {
  for (int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; s < n_seg; s += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = ptr[s], en = ptr[s + 1];
    for (int64_t i = b + 1; i < en; ++i) {
      const int32_t x = v[i];
      int64_t j = i - 1;
      while (j >= b && v[j] > x) {
        v[j + 1] = v[j];
        --j;
      }
      v[j + 1] = x;
    }
  }
}

__device__ __forceinline__ int64_t slot_of(const int32_t *col, int64_t b, int64_t en, int32_t c) {
  int64_t lo = b, hi = en;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (col[mid] < c) lo = mid + 1; else hi = mid;
  }
  return (lo < en && col[lo] == c) ? lo : -1;
}

// Thread per dof row: PASS 0 counts each slot's contributions, PASS 1 writes
// their element-matrix offsets in element order.
template <int PASS>
__global__ void k_slot_plan(int64_t nd, const int32_t *row_ptr, const int32_t *col, const int64_t *iptr,
                            const int32_t *key, const int64_t *lptr, const int32_t *ldofs, const int64_t *kbase,
                            int32_t *cnt, int64_t *cur, uint32_t *coff, int *flag) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < nd; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = row_ptr[r], en = row_ptr[r + 1];
    for (int64_t t = iptr[r]; t < iptr[r + 1]; ++t) {
      const int64_t e = key[t] >> 8, p = key[t] & 255;
      const int64_t l0 = lptr[e], ne = lptr[e + 1] - l0;
      for (int64_t k = 0; k < ne; ++k) {
        const int64_t s = slot_of(col, b, en, ldofs[l0 + k]);
        if (s < 0) {
          atomicOr(flag, 4);
          continue;
        }
        if (PASS == 0) ++cnt[s];
        else coff[cur[s]++] = (uint32_t)(kbase[e] + p * ne + k);
      }
    }
  }
}

__global__ void k_load_offsets(int64_t n, const int32_t *key, const int64_t *fbase, uint32_t *foff) {
  for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n; t += (int64_t)gridDim.x * blockDim.x)
    foff[t] = (uint32_t)(fbase[key[t] >> 8] + (key[t] & 255));
}

template <typename T>
__global__ void k_widen(int64_t n, const T *in, int64_t *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (int64_t)in[i];
}

// out[i] = sel ? v[i] : 0 (for the scans over the constrained elements)
__global__ void k_masked(int64_t n, const int32_t *sel, const int32_t *v, int kind, int64_t *out) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = v[i];
    const int64_t w = kind == 0 ? x : (kind == 1 ? x * x : (kind == 2 ? x + 1 : 1));
    out[i] = (sel == nullptr || sel[i]) ? w : 0;
  }
}

// exclusive scan of int64 values, out[n] = total
constexpr int ST = 1024;
__global__ void __launch_bounds__(ST) k_scan64_block(int64_t n, const int64_t *in, int64_t *out, int64_t *sums) {
  __shared__ int64_t s[ST];
  const int64_t i = (int64_t)blockIdx.x * ST + threadIdx.x;
  const int64_t x = i < n ? in[i] : 0;
  s[threadIdx.x] = x;
  __syncthreads();
  for (int off = 1; off < ST; off <<= 1) {
    const int64_t y = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += y;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - x;
  if (threadIdx.x == ST - 1) sums[blockIdx.x] = s[ST - 1];
}

__global__ void k_scan64_add(int64_t n, int64_t *out, const int64_t *offs) {
  const int64_t i = (int64_t)blockIdx.x * ST + threadIdx.x;
  if (i < n) out[i] += offs[blockIdx.x];
}

cudaError_t scan64(const int64_t *in, int64_t *out, int64_t n, cudaStream_t s) {
  const int64_t nb = std::max<int64_t>((n + ST - 1) / ST, 1);
  int64_t *sums = nullptr, *offs = nullptr;
  cudaError_t e = cudaMalloc((void **)&sums, sizeof(int64_t) * (size_t)(nb + 1));
  if (e == cudaSuccess) e = cudaMalloc((void **)&offs, sizeof(int64_t) * (size_t)(nb + 1));
  if (e == cudaSuccess) {
    if (n > 0) k_scan64_block<<<(unsigned)nb, ST, 0, s>>>(n, in, out, sums);
    else e = cudaMemsetAsync(sums, 0, sizeof(int64_t), s);
    if (e == cudaSuccess && nb > 1) {
      e = scan64(sums, offs, nb, s);
      if (e == cudaSuccess) k_scan64_add<<<(unsigned)nb, ST, 0, s>>>(n, out, offs);
      if (e == cudaSuccess) e = cudaMemcpyAsync(out + n, offs + nb, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
    } else if (e == cudaSuccess) {
      e = cudaMemcpyAsync(out + n, sums, sizeof(int64_t), cudaMemcpyDeviceToDevice, s);
    }
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (sums) cudaFree(sums);
  if (offs) cudaFree(offs);
  return e;
}

}  // namespace

// Builds the general path's plan on the device into the context's plan
// arrays.  Returns LMG_ERR_UNSUPPORTED (the caller builds it on the host)
// when an element's list or constraint matrix outgrows the limits, or when
// the element count does not fit the incidence keys.
lmg_status general_plan_device(lmg_ctx *c, bool use_cons, int64_t &kr, int64_t &fr, int &max_ne, int &max_ent,
                               int64_t &n_cons) {
  const int64_t E = c->n_elem, nd = c->n_dofs, nnz = c->nnz;
  const int N = c->nl;
  if (E >= ((int64_t)1 << 23) || N > 64) return LMG_ERR_UNSUPPORTED;
  cudaStream_t s = c->stream;
  std::vector<void *> tmp;
  auto alloc = [&](auto *&p, size_t n) {
    cudaError_t e = cudaMalloc((void **)&p, sizeof(*p) * std::max<size_t>(n, 1));
    if (e == cudaSuccess) tmp.push_back((void *)p);
    return e == cudaSuccess;
  };
  auto done = [&](lmg_status st) {
    cudaStreamSynchronize(s);
    for (void *p : tmp) cudaFree(p);
    return st;
  };
  auto grid = [&](int64_t n, int t) {
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + t - 1) / t, (int64_t)c->n_sm * 32));
  };
  const bool have_rows = !c->h_cons_ptr.empty();
  PlanIn in{};
  in.E = E;
  in.N = N;
  int32_t *ed = nullptr, *ccol = nullptr, *ne = nullptr, *nent = nullptr, *iscons = nullptr, *cnt = nullptr,
          *key = nullptr, *slot_cnt = nullptr, *cur32 = nullptr;
  int64_t *cp = nullptr, *v64 = nullptr, *lptr = nullptr, *ksc = nullptr, *fsc = nullptr, *psc = nullptr,
          *esc = nullptr, *csc = nullptr, *kbase = nullptr, *fbase = nullptr, *iptr = nullptr, *cur = nullptr;
  double *cval = nullptr;
  int *flag = nullptr;
  if (!alloc(ed, (size_t)(E * N)) || !alloc(ne, E) || !alloc(nent, E) || !alloc(iscons, E) || !alloc(flag, 1) ||
      !alloc(v64, E) || !alloc(lptr, E + 1) || !alloc(ksc, E + 1) || !alloc(fsc, E + 1) || !alloc(psc, E + 1) ||
      !alloc(esc, E + 1) || !alloc(csc, E + 1) || !alloc(kbase, E) || !alloc(fbase, E))
    return done(LMG_ERR_OOM);
  if (cudaMemcpyAsync(ed, c->h_elem_dofs.data(), sizeof(int32_t) * (size_t)(E * N), cudaMemcpyHostToDevice, s) ||
      cudaMemsetAsync(flag, 0, sizeof(int), s))
    return done(LMG_ERR_CUDA);
  in.ed = ed;
  if (use_cons && !c->h_constrained.empty()) {
    std::vector<uint8_t> hc = c->h_constrained;
    hc.resize((size_t)nd, 0);
    uint8_t *dc = nullptr;
    if (!alloc(dc, (size_t)nd)) return done(LMG_ERR_OOM);
    if (cudaMemcpyAsync(dc, hc.data(), (size_t)nd, cudaMemcpyHostToDevice, s) || cudaStreamSynchronize(s))
      return done(LMG_ERR_CUDA);
    in.cons = dc;
    if (have_rows) {
      if (!alloc(cp, (size_t)nd + 1) || !alloc(ccol, c->h_cons_col.size()) || !alloc(cval, c->h_cons_val.size()))
        return done(LMG_ERR_OOM);
      if (cudaMemcpyAsync(cp, c->h_cons_ptr.data(), sizeof(int64_t) * (size_t)(nd + 1), cudaMemcpyHostToDevice, s) ||
          cudaMemcpyAsync(ccol, c->h_cons_col.data(), sizeof(int32_t) * c->h_cons_col.size(), cudaMemcpyHostToDevice,
                          s) ||
          cudaMemcpyAsync(cval, c->h_cons_val.data(), sizeof(double) * c->h_cons_val.size(), cudaMemcpyHostToDevice,
                          s))
        return done(LMG_ERR_CUDA);
    } else {  // constrained flags without rows: every row is empty
      if (!alloc(cp, (size_t)nd + 1) || cudaMemsetAsync(cp, 0, sizeof(int64_t) * (size_t)(nd + 1), s))
        return done(LMG_ERR_OOM);
    }
    in.cp = cp;
    in.ccol = ccol;
    in.cval = cval;
  }
  const int ge = grid(E * 32, PW * 32);
  k_plan_sizes<<<ge, PW * 32, 0, s>>>(in, ne, nent, iscons, flag);
  int hf = 0;
  if (cudaMemcpyAsync(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s))
    return done(LMG_ERR_CUDA);
  if (hf) return done(LMG_ERR_UNSUPPORTED);
  // offsets: list (all elements), and per constrained element its matrix, vector,
  // column pointers, entries and record index
  const int gE = grid(E, 256);
  struct {
    int kind;
    const int32_t *sel;
    int64_t *out;
    const int32_t *val;
  } sc[] = {{0, nullptr, lptr, ne}, {1, iscons, ksc, ne}, {0, iscons, fsc, ne},
            {2, iscons, psc, ne}, {0, iscons, esc, nent}, {3, iscons, csc, ne}};
  for (auto &x : sc) {
    k_masked<<<gE, 256, 0, s>>>(E, x.sel, x.val, x.kind, v64);
    if (scan64(v64, x.out, E, s) != cudaSuccess) return done(LMG_ERR_CUDA);
  }
  int64_t tot[6] = {0, 0, 0, 0, 0, 0};
  for (int i = 0; i < 6; ++i)
    if (cudaMemcpyAsync(&tot[i], sc[i].out + E, sizeof(int64_t), cudaMemcpyDeviceToHost, s))
      return done(LMG_ERR_CUDA);
  if (cudaStreamSynchronize(s)) return done(LMG_ERR_CUDA);
  const int64_t n_list = tot[0];
  n_cons = tot[5];
  kr = E * (int64_t)N * N + tot[1];
  fr = E * (int64_t)N + tot[2];
  if (kr >= (int64_t)UINT32_MAX || fr >= (int64_t)UINT32_MAX || n_list >= INT32_MAX) return done(LMG_ERR_UNSUPPORTED);
  general_free(c);
  if (dalloc(c->d_celem, (size_t)n_cons) || dalloc(c->d_cne, (size_t)n_cons) || dalloc(c->d_ckout, (size_t)n_cons) ||
      dalloc(c->d_cfout, (size_t)n_cons) || dalloc(c->d_cbase, (size_t)n_cons) || dalloc(c->d_cebase, (size_t)n_cons) ||
      dalloc(c->d_ccp, (size_t)tot[3]) || dalloc(c->d_cci, (size_t)tot[4]) || dalloc(c->d_ccv, (size_t)tot[4]) ||
      dalloc(c->d_crow, (size_t)n_cons))
    return done(LMG_ERR_OOM);
  k_plan_bases<<<gE, 256, 0, s>>>(in, ne, nent, iscons, ksc, fsc, psc, esc, csc, kbase, fbase, c->d_celem, c->d_cne,
                                  c->d_ckout, c->d_cfout, c->d_cbase, c->d_cebase);
  int32_t *ldofs = nullptr;
  if (!alloc(ldofs, (size_t)n_list)) return done(LMG_ERR_OOM);
  k_plan_fill<<<ge, PW * 32, 0, s>>>(in, lptr, iscons, csc, c->d_cbase, c->d_cebase, ldofs, c->d_ccp, c->d_cci,
                                     c->d_ccv, c->d_crow);
  // incidences of every dof in element order
  if (!alloc(cnt, (size_t)nd) || !alloc(cur32, (size_t)nd) ||
      !alloc(key, (size_t)n_list) || dalloc(c->d_gfptr, (size_t)nd + 1) || dalloc(c->d_gfoff, (size_t)n_list))
    return done(LMG_ERR_OOM);
  cudaMemsetAsync(cnt, 0, sizeof(int32_t) * (size_t)nd, s);
  k_inc_count<<<grid(n_list, 256), 256, 0, s>>>(n_list, ldofs, cnt);
  int64_t *cnt64 = nullptr;
  if (!alloc(cnt64, (size_t)nd)) return done(LMG_ERR_OOM);
  k_widen<int32_t><<<grid(nd, 256), 256, 0, s>>>(nd, cnt, cnt64);
  if (scan64(cnt64, c->d_gfptr, nd, s) != cudaSuccess) return done(LMG_ERR_CUDA);
  iptr = c->d_gfptr;
  cudaMemsetAsync(cur32, 0, sizeof(int32_t) * (size_t)nd, s);
  k_inc_fill<<<gE, 256, 0, s>>>(E, lptr, ldofs, iptr, cur32, key);
  k_seg_sort64<<<grid(nd, 256), 256, 0, s>>>(nd, iptr, key);
  k_load_offsets<<<grid(n_list, 256), 256, 0, s>>>(n_list, key, fbase, c->d_gfoff);
  // slot counts, then the contributions' offsets in element order
  if (!alloc(slot_cnt, (size_t)nnz) || !alloc(cur, (size_t)nnz + 1) || dalloc(c->d_cptr, (size_t)nnz + 1))
    return done(LMG_ERR_OOM);
  cudaMemsetAsync(slot_cnt, 0, sizeof(int32_t) * (size_t)nnz, s);
  const int gd = grid(nd, 128);
  k_slot_plan<0><<<gd, 128, 0, s>>>(nd, c->d_row_ptr, c->d_col, iptr, key, lptr, ldofs, kbase, slot_cnt, nullptr,
                                    nullptr, flag);
  k_widen<int32_t><<<grid(nnz, 256), 256, 0, s>>>(nnz, slot_cnt, cur);
  if (scan64(cur, c->d_cptr, nnz, s) != cudaSuccess) return done(LMG_ERR_CUDA);
  int64_t n_contrib = 0;
  if (cudaMemcpyAsync(&n_contrib, c->d_cptr + nnz, sizeof(int64_t), cudaMemcpyDeviceToHost, s) ||
      cudaMemcpyAsync(&hf, flag, sizeof(int), cudaMemcpyDeviceToHost, s) || cudaStreamSynchronize(s))
    return done(LMG_ERR_CUDA);
  if (hf) return done(LMG_ERR_NEW_NONZERO);
  if (dalloc(c->d_coff, (size_t)n_contrib)) return done(LMG_ERR_OOM);
  cudaMemcpyAsync(cur, c->d_cptr, sizeof(int64_t) * (size_t)nnz, cudaMemcpyDeviceToDevice, s);
  k_slot_plan<1><<<gd, 128, 0, s>>>(nd, c->d_row_ptr, c->d_col, iptr, key, lptr, ldofs, kbase, nullptr, cur,
                                    c->d_coff, flag);
  // the largest constrained element (the constraint kernel's launch shape)
  std::vector<int32_t> hne((size_t)E), hent((size_t)E), hcons((size_t)E);
  if (cudaMemcpyAsync(hne.data(), ne, sizeof(int32_t) * E, cudaMemcpyDeviceToHost, s) ||
      cudaMemcpyAsync(hent.data(), nent, sizeof(int32_t) * E, cudaMemcpyDeviceToHost, s) ||
      cudaMemcpyAsync(hcons.data(), iscons, sizeof(int32_t) * E, cudaMemcpyDeviceToHost, s) ||
      cudaStreamSynchronize(s) || cudaGetLastError() != cudaSuccess)
    return done(LMG_ERR_CUDA);
  max_ne = 0;
  max_ent = 0;
  for (int64_t e = 0; e < E; ++e)
    if (hcons[(size_t)e]) {
      max_ne = std::max(max_ne, hne[(size_t)e]);
      max_ent = std::max(max_ent, hent[(size_t)e]);
    }
  return done(LMG_OK);
}

}  // namespace lmg
