// DofMap::distribute_dofs on the device (distribute_local_dofs_var_major,
// src/base/dof_map.C:1417-1537; dof_indices, :2198-2320).
//
// libMesh numbers the dofs in one sweep over the elements in id order: each
// node not yet numbered takes the next block of dofs (n_vars LAGRANGE dofs, or
// the HIERARCHIC count of its kind of node), then the element its own
// interior dofs; nodes no element touches come last.  That sequential sweep
// is an exclusive scan: position (e, a) carries the node's dof count when it
// is the node's first touch (the smallest e * npe + a among the node's
// positions, found with atomicMin), each element's extra position its
// interior count; the scan of those weights is every dof base.
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "lmg_internal.h"

namespace lmg {

namespace {

constexpr int DT = 1024;  // threads of the scan blocks

// Per-node dof counts of the numbering: LAGRANGE (n_vars per node) or the
// HIERARCHIC layouts of THIRD on HEX27 / TET14 / PRISM21.
struct Layout {
  int npe, nv_vertices, n_interior, kind;  // kind 0: n_vars per node; 1 HEX27 p3; 2 TET14 p3; 3 PRISM21 p3
  int n_vars;
  __host__ __device__ int node_dofs(int a) const {
    switch (kind) {
      case 1: return a < 8 ? 1 : (a < 20 ? 2 : (a < 26 ? 4 : 0));
      case 2: return a < 4 ? 1 : (a < 10 ? 2 : 1);
      case 3: return a < 6 ? 1 : (a < 15 ? 2 : (a < 18 ? 4 : (a < 20 ? 1 : 2)));
      default: return n_vars;
    }
  }
};

__global__ void k_first_touch(int64_t n_pos, Layout L, const int32_t *conn, unsigned long long *first) {
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_pos; p += (int64_t)gridDim.x * blockDim.x)
    if (L.node_dofs((int)(p % L.npe)) > 0) atomicMin(&first[conn[p]], (unsigned long long)p);
}

// weight of extended position q = e * (npe + 1) + a
__global__ void k_weights(int64_t n_elem, Layout L, const int32_t *conn, const unsigned long long *first,
                          int32_t *w) {
  const int64_t n = n_elem * (L.npe + 1);
  for (int64_t q = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = q / (L.npe + 1);
    const int a = (int)(q - e * (L.npe + 1));
    if (a == L.npe) {
      w[q] = L.n_interior;
    } else {
      const int64_t p = e * L.npe + a;
      w[q] = first[conn[p]] == (unsigned long long)p ? L.node_dofs(a) : 0;
    }
  }
}

// Block-local exclusive scan of 1024 entries per block; block totals to sums.
__global__ void __launch_bounds__(DT) k_scan_block(int64_t n, const int32_t *in, int32_t *out, int32_t *sums) {
  __shared__ int32_t s[DT];
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  const int32_t x = i < n ? in[i] : 0;
  s[threadIdx.x] = x;
  __syncthreads();
  for (int off = 1; off < DT; off <<= 1) {
    const int32_t y = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += y;
    __syncthreads();
  }
  if (i < n) out[i] = s[threadIdx.x] - x;
  if (threadIdx.x == DT - 1) sums[blockIdx.x] = s[DT - 1];
}

__global__ void k_scan_add(int64_t n, int32_t *out, const int32_t *offs) {
  const int64_t i = (int64_t)blockIdx.x * DT + threadIdx.x;
  if (i < n) out[i] += offs[blockIdx.x];
}

// exclusive scan of in[0..n) into out[0..n), total into *total (device)
cudaError_t scan(const int32_t *in, int32_t *out, int64_t n, int32_t *total) {
  const int64_t nb = (n + DT - 1) / DT;
  int32_t *sums = nullptr, *offs = nullptr;
  cudaError_t e = cudaMalloc((void **)&sums, sizeof(int32_t) * (size_t)(nb + 1));
  if (e == cudaSuccess) e = cudaMalloc((void **)&offs, sizeof(int32_t) * (size_t)(nb + 1));
  if (e == cudaSuccess && n > 0) {
    k_scan_block<<<(unsigned)nb, DT>>>(n, in, out, sums);
    if (nb > 1) {
      e = scan(sums, offs, nb, total);
      if (e == cudaSuccess) k_scan_add<<<(unsigned)nb, DT>>>(n, out, offs);
    } else {
      e = cudaMemcpy(total, sums, sizeof(int32_t), cudaMemcpyDeviceToDevice);
    }
  } else if (e == cudaSuccess) {
    e = cudaMemset(total, 0, sizeof(int32_t));
  }
  if (e == cudaSuccess) e = cudaGetLastError();
  if (sums) cudaFree(sums);
  if (offs) cudaFree(offs);
  return e;
}

__global__ void k_untouched(int64_t n_nodes, const unsigned long long *first, int32_t *u) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_nodes; i += (int64_t)gridDim.x * blockDim.x)
    u[i] = first[i] == ~0ull ? 1 : 0;
}

// dof_indices: variable-major LAGRANGE lists, or the HIERARCHIC node lists
// (non-vertex nodes' dofs last to first) and the element's interior dofs.
__global__ void k_elem_dofs(int64_t n_elem, Layout L, const int32_t *conn, const unsigned long long *first,
                            const int32_t *base, int32_t *ed, int nl) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < n_elem; e += (int64_t)gridDim.x * blockDim.x) {
    int32_t *d = ed + e * nl;
    if (L.kind == 0) {
      for (int a = 0; a < L.npe; ++a) {
        const unsigned long long p = first[conn[e * L.npe + a]];
        const int32_t b = base[(int64_t)(p / L.npe) * (L.npe + 1) + (int64_t)(p % L.npe)];
        for (int v = 0; v < L.n_vars; ++v) d[v * L.npe + a] = b + v;
      }
    } else {
      int k = 0;
      for (int a = 0; a < L.npe; ++a) {
        const int c = L.node_dofs(a);
        if (!c) continue;
        const unsigned long long p = first[conn[e * L.npe + a]];
        const int32_t b = base[(int64_t)(p / L.npe) * (L.npe + 1) + (int64_t)(p % L.npe)];
        for (int i = 0; i < c; ++i) d[k++] = b + (a < L.nv_vertices ? i : c - 1 - i);
      }
      const int32_t ib = base[e * (L.npe + 1) + L.npe];
      for (int i = 0; i < L.n_interior; ++i) d[k++] = ib + i;
    }
  }
}

}  // namespace

std::string distribute_dofs_device(int device, int64_t n_nodes, int64_t n_elem, int elem_type, const int32_t *conn,
                                   int n_vars, int fe_order, int64_t &n_dofs, int32_t *elem_dofs) {
  Layout L{};
  L.npe = nodes_per_elem(elem_type);
  L.nv_vertices = vertices_per_elem(elem_type);
  L.n_vars = n_vars;
  int nl = n_vars * L.npe;
  if (fe_order == (3 | LMG_HIERARCHIC)) {
    if (n_vars != 1) return "one variable";
    if (elem_type == LMG_HEX27) { L.kind = 1; L.n_interior = 8; nl = 64; }
    else if (elem_type == LMG_TET14) { L.kind = 2; nl = 20; }
    else if (elem_type == LMG_PRISM21) { L.kind = 3; nl = 40; }
    else return "THIRD HIERARCHIC needs HEX27, TET14 or PRISM21";
  }
  if (!L.npe) return "element type";
  const int64_t n_pos = n_elem * L.npe, n_ext = n_elem * (L.npe + 1);
  if (n_ext >= INT32_MAX || n_nodes >= INT32_MAX) return "too large";
  if (cudaSetDevice(device) != cudaSuccess) return "device";
  int32_t *d_conn = nullptr, *w = nullptr, *base = nullptr, *tot = nullptr, *u = nullptr, *ur = nullptr,
          *d_ed = nullptr;
  unsigned long long *first = nullptr;
  cudaError_t e = cudaSuccess;
  auto ok = [&](cudaError_t x) {
    if (e == cudaSuccess) e = x;
    return e == cudaSuccess;
  };
  int32_t h_tot[2] = {0, 0};
  const int threads = 256;
  auto blocks = [&](int64_t n) { return (int)std::max<int64_t>(1, std::min<int64_t>((n + threads - 1) / threads, 65536)); };
  if (ok(cudaMalloc((void **)&d_conn, sizeof(int32_t) * (size_t)std::max<int64_t>(n_pos, 1))) &&
      ok(cudaMemcpy(d_conn, conn, sizeof(int32_t) * (size_t)n_pos, cudaMemcpyHostToDevice)) &&
      ok(cudaMalloc((void **)&first, sizeof(unsigned long long) * (size_t)std::max<int64_t>(n_nodes, 1))) &&
      ok(cudaMemset(first, 0xff, sizeof(unsigned long long) * (size_t)n_nodes)) &&
      ok(cudaMalloc((void **)&w, sizeof(int32_t) * (size_t)std::max<int64_t>(n_ext, 1))) &&
      ok(cudaMalloc((void **)&base, sizeof(int32_t) * (size_t)std::max<int64_t>(n_ext, 1))) &&
      ok(cudaMalloc((void **)&tot, sizeof(int32_t) * 2))) {
    k_first_touch<<<blocks(n_pos), threads>>>(n_pos, L, d_conn, first);
    k_weights<<<blocks(n_ext), threads>>>(n_elem, L, d_conn, first, w);
    if (ok(cudaGetLastError()) && ok(scan(w, base, n_ext, tot)) &&
        ok(cudaMemcpy(&h_tot[0], tot, sizeof(int32_t), cudaMemcpyDeviceToHost))) {
      n_dofs = h_tot[0];
      if (L.kind == 0) {  // nodes no element touches: numbered after, in node order
        if (ok(cudaMalloc((void **)&u, sizeof(int32_t) * (size_t)std::max<int64_t>(n_nodes, 1))) &&
            ok(cudaMalloc((void **)&ur, sizeof(int32_t) * (size_t)std::max<int64_t>(n_nodes, 1)))) {
          k_untouched<<<blocks(n_nodes), threads>>>(n_nodes, first, u);
          if (ok(cudaGetLastError()) && ok(scan(u, ur, n_nodes, tot + 1)) &&
              ok(cudaMemcpy(&h_tot[1], tot + 1, sizeof(int32_t), cudaMemcpyDeviceToHost)))
            n_dofs += (int64_t)h_tot[1] * n_vars;
        }
      }
      if (e == cudaSuccess && elem_dofs &&
          ok(cudaMalloc((void **)&d_ed, sizeof(int32_t) * (size_t)std::max<int64_t>(n_elem * nl, 1)))) {
        k_elem_dofs<<<blocks(n_elem), threads>>>(n_elem, L, d_conn, first, base, d_ed, nl);
        if (ok(cudaGetLastError()))
          ok(cudaMemcpy(elem_dofs, d_ed, sizeof(int32_t) * (size_t)(n_elem * nl), cudaMemcpyDeviceToHost));
      }
    }
  }
  for (void *p : {(void *)d_conn, (void *)w, (void *)base, (void *)tot, (void *)u, (void *)ur, (void *)d_ed,
                  (void *)first})
    if (p) cudaFree(p);
  if (e != cudaSuccess) return std::string("device numbering: ") + cudaGetErrorString(e);
  return "";
}

}  // namespace lmg
