// Host mirror of libMesh's DofMap setup: dof numbering, dof_indices,
// Dirichlet constraint sets and the element-coupling sparsity graph.
#include <algorithm>
#include <atomic>
#include <new>
#include <thread>

#include "lmg_internal.h"

namespace lmg {

// Block graph: row P holds every block Q that shares an element with P,
// sorted ascending.  This is SparsityPattern::Build with DefaultCoupling(0)
// and full variable coupling (src/base/sparsity_pattern.C:279-363): every row
// of an element couples every column of the same element.
void build_block_graph(int64_t n_elem, int nb, const int32_t *eb, int64_t n_blocks,
                       std::vector<int64_t> &row_ptr, std::vector<int32_t> &cols, int n_threads) {
  // block -> elements (CSR), elements listed once per block they touch
  std::vector<int64_t> bptr((size_t)n_blocks + 1, 0);
  for (int64_t i = 0; i < n_elem * nb; ++i) bptr[(size_t)eb[i] + 1]++;
  for (int64_t b = 0; b < n_blocks; ++b) bptr[(size_t)b + 1] += bptr[(size_t)b];
  std::vector<int32_t> belem((size_t)bptr[(size_t)n_blocks]);
  {
    std::vector<int64_t> cur(bptr.begin(), bptr.end() - 1);
    for (int64_t e = 0; e < n_elem; ++e)
      for (int a = 0; a < nb; ++a) belem[(size_t)cur[(size_t)eb[e * nb + a]]++] = (int32_t)e;
  }
  if (n_threads < 1) n_threads = 1;
  std::vector<int64_t> deg((size_t)n_blocks, 0);
  // pass 1: degrees; pass 2: fill.  Each pass sorts the candidate list of a row.
  auto row_cols = [&](int64_t P, std::vector<int32_t> &buf) {
    buf.clear();
    for (int64_t k = bptr[(size_t)P]; k < bptr[(size_t)P + 1]; ++k) {
      const int32_t *b = eb + (int64_t)belem[(size_t)k] * nb;
      buf.insert(buf.end(), b, b + nb);
    }
    std::sort(buf.begin(), buf.end());
    buf.erase(std::unique(buf.begin(), buf.end()), buf.end());
  };
  auto run = [&](auto &&fn) {
    std::atomic<int64_t> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t)
      th.emplace_back([&]() {
        std::vector<int32_t> buf;
        const int64_t chunk = 4096;
        for (;;) {
          int64_t s = next.fetch_add(chunk);
          if (s >= n_blocks) break;
          int64_t e = std::min(n_blocks, s + chunk);
          for (int64_t P = s; P < e; ++P) fn(P, buf);
        }
      });
    for (auto &t : th) t.join();
  };
  run([&](int64_t P, std::vector<int32_t> &buf) {
    row_cols(P, buf);
    deg[(size_t)P] = (int64_t)buf.size();
  });
  row_ptr.assign((size_t)n_blocks + 1, 0);
  for (int64_t P = 0; P < n_blocks; ++P) row_ptr[(size_t)P + 1] = row_ptr[(size_t)P] + deg[(size_t)P];
  cols.resize((size_t)row_ptr[(size_t)n_blocks]);
  run([&](int64_t P, std::vector<int32_t> &buf) {
    row_cols(P, buf);
    std::copy(buf.begin(), buf.end(), cols.begin() + row_ptr[(size_t)P]);
  });
}

// Element lists of varying length (eptr [n_elem+1], elist): the same row-wise
// union as build_block_graph.
static void build_var_graph(int64_t n_elem, const std::vector<int64_t> &eptr, const std::vector<int32_t> &elist,
                            int64_t n_rows, std::vector<int64_t> &row_ptr, std::vector<int32_t> &cols,
                            int n_threads) {
  std::vector<int64_t> rptr((size_t)n_rows + 1, 0);
  for (int32_t r : elist) rptr[(size_t)r + 1]++;
  for (int64_t r = 0; r < n_rows; ++r) rptr[(size_t)r + 1] += rptr[(size_t)r];
  std::vector<int32_t> relem((size_t)rptr[(size_t)n_rows]);
  {
    std::vector<int64_t> cur(rptr.begin(), rptr.end() - 1);
    for (int64_t e = 0; e < n_elem; ++e)
      for (int64_t k = eptr[(size_t)e]; k < eptr[(size_t)e + 1]; ++k)
        relem[(size_t)cur[(size_t)elist[(size_t)k]]++] = (int32_t)e;
  }
  if (n_threads < 1) n_threads = 1;
  std::vector<int64_t> deg((size_t)n_rows, 0);
  // columns of row r: the union of its elements' dof lists, deduplicated with
  // a per-thread stamp array (last row that saw each dof), then sorted
  auto row_cols = [&](int64_t r, std::vector<int32_t> &buf, std::vector<int64_t> &stamp) {
    buf.clear();
    for (int64_t k = rptr[(size_t)r]; k < rptr[(size_t)r + 1]; ++k) {
      const int64_t e = relem[(size_t)k];
      for (int64_t j = eptr[(size_t)e]; j < eptr[(size_t)e + 1]; ++j) {
        const int32_t d = elist[(size_t)j];
        if (stamp[(size_t)d] != r) {
          stamp[(size_t)d] = r;
          buf.push_back(d);
        }
      }
    }
    std::sort(buf.begin(), buf.end());
  };
  // rows in chunks; each thread keeps its chunks' columns until the row
  // pointer is known, then copies them into place
  const int64_t CH = 4096, n_ch = (n_rows + CH - 1) / CH;
  std::vector<std::vector<int32_t>> chunk_cols((size_t)n_ch);
  {
    std::atomic<int64_t> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t)
      th.emplace_back([&]() {
        std::vector<int32_t> buf;
        std::vector<int64_t> stamp((size_t)n_rows, -1);
        for (;;) {
          const int64_t c = next.fetch_add(1);
          if (c >= n_ch) break;
          std::vector<int32_t> &out = chunk_cols[(size_t)c];
          for (int64_t r = c * CH; r < std::min(n_rows, (c + 1) * CH); ++r) {
            row_cols(r, buf, stamp);
            deg[(size_t)r] = (int64_t)buf.size();
            out.insert(out.end(), buf.begin(), buf.end());
          }
        }
      });
    for (auto &t : th) t.join();
  }
  row_ptr.assign((size_t)n_rows + 1, 0);
  for (int64_t r = 0; r < n_rows; ++r) row_ptr[(size_t)r + 1] = row_ptr[(size_t)r] + deg[(size_t)r];
  cols.resize((size_t)row_ptr[(size_t)n_rows]);
  {
    std::atomic<int64_t> next{0};
    std::vector<std::thread> th;
    for (int t = 0; t < n_threads; ++t)
      th.emplace_back([&]() {
        for (;;) {
          const int64_t c = next.fetch_add(1);
          if (c >= n_ch) break;
          std::vector<int32_t> &v = chunk_cols[(size_t)c];
          std::copy(v.begin(), v.end(), cols.begin() + row_ptr[(size_t)(c * CH)]);
          std::vector<int32_t>().swap(v);
        }
      });
    for (auto &t : th) t.join();
  }
}

void build_constrained_graph(int64_t n_elem, int nl, const int32_t *ed, int64_t n_dofs, const int64_t *cons_ptr,
                             const int32_t *cons_col, std::vector<int64_t> &row_ptr, std::vector<int32_t> &cols,
                             int n_threads) {
  // find_connected_dofs: close each element's dof set under "constrained by"
  // (elements in contiguous ranges per thread, lists concatenated in order)
  const int T = std::max(1, std::min<int>(n_threads, (int)std::max<int64_t>(1, n_elem / 1024)));
  std::vector<std::vector<int32_t>> part((size_t)T);
  std::vector<std::vector<int64_t>> plen((size_t)T);
  std::vector<std::thread> th;
  for (int tid = 0; tid < T; ++tid)
    th.emplace_back([&, tid]() {
      const int64_t e0 = n_elem * tid / T, e1 = n_elem * (tid + 1) / T;
      std::vector<int32_t> &out = part[(size_t)tid];
      std::vector<int64_t> &len = plen[(size_t)tid];
      out.reserve((size_t)((e1 - e0) * nl));
      std::vector<int32_t> set, add;
      for (int64_t e = e0; e < e1; ++e) {
        set.assign(ed + e * nl, ed + (e + 1) * nl);
        std::sort(set.begin(), set.end());
        set.erase(std::unique(set.begin(), set.end()), set.end());
        for (bool done = false; !done;) {
          add.clear();
          for (int32_t d : set)
            for (int64_t k = cons_ptr[d]; k < cons_ptr[d + 1]; ++k)
              if (!std::binary_search(set.begin(), set.end(), cons_col[k])) add.push_back(cons_col[k]);
          done = add.empty();
          if (!done) {
            set.insert(set.end(), add.begin(), add.end());
            std::sort(set.begin(), set.end());
            set.erase(std::unique(set.begin(), set.end()), set.end());
          }
        }
        out.insert(out.end(), set.begin(), set.end());
        len.push_back((int64_t)set.size());
      }
    });
  for (auto &t : th) t.join();
  std::vector<int64_t> eptr((size_t)n_elem + 1, 0);
  std::vector<int32_t> elist;
  size_t total = 0;
  for (auto &p : part) total += p.size();
  elist.reserve(total);
  int64_t e = 0;
  for (int tid = 0; tid < T; ++tid) {
    elist.insert(elist.end(), part[(size_t)tid].begin(), part[(size_t)tid].end());
    for (int64_t l : plen[(size_t)tid]) {
      eptr[(size_t)e + 1] = eptr[(size_t)e] + l;
      ++e;
    }
    std::vector<int32_t>().swap(part[(size_t)tid]);
  }
  build_var_graph(n_elem, eptr, elist, n_dofs, row_ptr, cols, n_threads);
}

void block_structure(int64_t n_elem, int npe, int nv, const int32_t *ed, int &bs, int &nb,
                     std::vector<int32_t> &eb) {
  const int nl = nv * npe;
  bool ok = nv > 1;
  for (int64_t e = 0; ok && e < n_elem; ++e) {
    const int32_t *d = ed + e * nl;
    for (int a = 0; ok && a < npe; ++a) {
      if (d[a] % nv != 0) ok = false;
      for (int v = 1; ok && v < nv; ++v) ok = (d[v * npe + a] == d[a] + v);
    }
  }
  bs = ok ? nv : 1;
  nb = ok ? npe : nl;
  eb.resize((size_t)(n_elem * nb));
  for (int64_t e = 0; e < n_elem; ++e)
    for (int a = 0; a < nb; ++a) eb[(size_t)(e * nb + a)] = ed[e * nl + a] / bs;
}

}  // namespace lmg

extern "C" {

lmg_status lmg_host_sparsity_constrained(int64_t n_elem, int32_t dofs_per_elem, int64_t n_dofs,
                                         const int32_t *elem_dofs, const int64_t *cons_ptr,
                                         const int32_t *cons_col, int64_t *nnz, int32_t *row_ptr,
                                         int32_t *col_idx) {
  if (!elem_dofs || !nnz || !cons_ptr || n_elem <= 0 || dofs_per_elem <= 0 || n_dofs <= 0) return LMG_ERR_ARG;
  for (int64_t i = 0; i < n_elem * dofs_per_elem; ++i)
    if (elem_dofs[i] < 0 || elem_dofs[i] >= n_dofs) return LMG_ERR_BOUNDS;
  for (int64_t k = 0; k < cons_ptr[n_dofs]; ++k)
    if (!cons_col || cons_col[k] < 0 || cons_col[k] >= n_dofs) return LMG_ERR_BOUNDS;
  try {
    std::vector<int64_t> rp;
    std::vector<int32_t> cols;
    const unsigned hw = std::thread::hardware_concurrency();
    lmg::build_constrained_graph(n_elem, dofs_per_elem, elem_dofs, n_dofs, cons_ptr, cons_col, rp, cols,
                                 hw ? (int)hw : 4);
    if ((int64_t)cols.size() >= INT32_MAX) return LMG_ERR_UNSUPPORTED;
    *nnz = (int64_t)cols.size();
    if (row_ptr && col_idx) {
      for (int64_t r = 0; r <= n_dofs; ++r) row_ptr[r] = (int32_t)rp[(size_t)r];
      std::copy(cols.begin(), cols.end(), col_idx);
    }
  } catch (const std::bad_alloc &) {
    return LMG_ERR_OOM;
  }
  return LMG_OK;
}

lmg_status lmg_host_sparsity(int64_t n_elem, int32_t npe, int32_t n_vars, int64_t n_dofs,
                             const int32_t *elem_dofs, int64_t *nnz, int32_t *row_ptr, int32_t *col_idx) {
  if (!elem_dofs || !nnz || n_elem <= 0 || npe <= 0 || n_vars <= 0 || n_dofs <= 0) return LMG_ERR_ARG;
  try {
    int bs = 1, nb = 0;
    std::vector<int32_t> eb;
    lmg::block_structure(n_elem, npe, n_vars, elem_dofs, bs, nb, eb);
    std::vector<int64_t> brow;
    std::vector<int32_t> bcol;
    const unsigned hw = std::thread::hardware_concurrency();
    lmg::build_block_graph(n_elem, nb, eb.data(), n_dofs / bs, brow, bcol, hw ? (int)hw : 4);
    const int64_t total = (int64_t)bcol.size() * bs * bs;
    if (total >= INT32_MAX) return LMG_ERR_UNSUPPORTED;
    *nnz = total;
    if (row_ptr && col_idx) {
      int64_t o = 0;
      for (int64_t r = 0; r < n_dofs; ++r) {
        row_ptr[r] = (int32_t)o;
        const int64_t P = r / bs;
        for (int64_t j = brow[(size_t)P]; j < brow[(size_t)P + 1]; ++j)
          for (int k = 0; k < bs; ++k) col_idx[o++] = bs * bcol[(size_t)j] + k;
      }
      row_ptr[n_dofs] = (int32_t)o;
    }
  } catch (const std::bad_alloc &) {
    return LMG_ERR_OOM;
  }
  return LMG_OK;
}

lmg_status lmg_dofmap_distribute(int64_t n_nodes, int64_t n_elem, int32_t npe, const int32_t *conn,
                                 int32_t n_vars, int64_t *n_dofs, int32_t *elem_dofs) {
  if (!conn || !n_dofs || n_nodes < 0 || n_elem < 0 || npe <= 0 || n_vars <= 0) return LMG_ERR_ARG;
  try {
    // distribute_local_dofs_var_major (dof_map.C:1417-1537): one VariableGroup
    // of n_vars LAGRANGE variables, one component per node; a node's dofs are
    // vg_dof_base + var (DofObject::dof_number, include/base/dof_object.h:1029-1056).
    std::vector<int64_t> base((size_t)n_nodes, -1);
    int64_t next = 0;
    for (int64_t e = 0; e < n_elem; ++e)
      for (int a = 0; a < npe; ++a) {
        const int32_t n = conn[e * npe + a];
        if (n < 0 || n >= n_nodes) return LMG_ERR_BOUNDS;
        if (base[(size_t)n] < 0) {
          base[(size_t)n] = next;
          next += n_vars;
        }
      }
    // Nodes no element touches get numbered afterwards (dof_map.C:1515-1527).
    for (int64_t n = 0; n < n_nodes; ++n)
      if (base[(size_t)n] < 0) {
        base[(size_t)n] = next;
        next += n_vars;
      }
    if (next > INT32_MAX) return LMG_ERR_UNSUPPORTED;
    *n_dofs = next;
    if (elem_dofs) {
      const int64_t nl = (int64_t)n_vars * npe;
      for (int64_t e = 0; e < n_elem; ++e)
        for (int v = 0; v < n_vars; ++v)
          for (int a = 0; a < npe; ++a)
            elem_dofs[e * nl + v * npe + a] = (int32_t)(base[(size_t)conn[e * npe + a]] + v);
    }
  } catch (const std::bad_alloc &) {
    return LMG_ERR_OOM;
  }
  return LMG_OK;
}

// FEType{THIRD, HIERARCHIC} on HEX27 (HIERARCHIC_n_dofs_at_node,
// fe_hierarchic.C:236-290): a vertex carries 1 dof, an edge node 2, a face
// node 4, the centre node none; the 8 interior dofs belong to the element.
// distribute_local_dofs_var_major numbers, per element, the nodes not yet
// numbered and then the element's dofs; dof_indices lists a non-vertex node's
// dofs last to first (extra_hanging_dofs, dof_map.h:2685-2712).
// On TET14 (HIERARCHIC_n_dofs_at_node, fe_hierarchic.C:440-470) a vertex
// carries 1 dof, an edge node 2, a face node 1, and no dof is the element's.
// On PRISM21 (HIERARCHIC_n_dofs_at_node, fe_hierarchic.C:289-340) a vertex
// carries 1 dof, an edge node 2, a quadrilateral-face node 4, a triangle-face
// node 1 and the interior node 20 the element's 2; no dof is the element's.
struct P3Layout {
  int npe, nl, n_interior, nsides;
  int node_dofs(int a) const {
    if (npe == 27) return a < 8 ? 1 : (a < 20 ? 2 : (a < 26 ? 4 : 0));
    if (npe == 21) return a < 6 ? 1 : (a < 15 ? 2 : (a < 18 ? 4 : (a < 20 ? 1 : 2)));
    return a < 4 ? 1 : (a < 10 ? 2 : 1);
  }
};
static bool p3_layout(int32_t elem_type, P3Layout &l) {
  if (elem_type == LMG_HEX27) l = {27, 64, 8, 6};
  else if (elem_type == LMG_TET14) l = {14, 20, 0, 4};
  else if (elem_type == LMG_PRISM21) l = {21, 40, 0, 5};
  else return false;
  return true;
}

lmg_status lmg_fe_dofs_per_elem(int32_t elem_type, int32_t fe_order, int32_t n_vars, int32_t *n) {
  if (!n || n_vars <= 0) return LMG_ERR_ARG;
  if (fe_order == (3 | LMG_HIERARCHIC)) {
    P3Layout l;
    if (!p3_layout(elem_type, l) || n_vars != 1) return LMG_ERR_UNSUPPORTED;
    *n = l.nl;
    return LMG_OK;
  }
  const int npe = lmg::nodes_per_elem(elem_type);
  if (!npe) return LMG_ERR_UNSUPPORTED;
  *n = n_vars * npe;
  return LMG_OK;
}

lmg_status lmg_dofmap_distribute_fe(int64_t n_nodes, int64_t n_elem, int32_t elem_type, const int32_t *conn,
                                    int32_t n_vars, int32_t fe_order, int64_t *n_dofs, int32_t *elem_dofs) {
  if (fe_order != (3 | LMG_HIERARCHIC))
    return lmg_dofmap_distribute(n_nodes, n_elem, lmg::nodes_per_elem(elem_type), conn, n_vars, n_dofs, elem_dofs);
  if (!conn || !n_dofs || n_nodes < 0 || n_elem < 0) return LMG_ERR_ARG;
  P3Layout l;
  if (!p3_layout(elem_type, l) || n_vars != 1) return LMG_ERR_UNSUPPORTED;
  const int npe = l.npe, nv = lmg::vertices_per_elem(elem_type);
  try {
    std::vector<int64_t> base((size_t)n_nodes, -1), ebase((size_t)n_elem);
    int64_t next = 0;
    for (int64_t e = 0; e < n_elem; ++e) {
      for (int a = 0; a < npe; ++a) {
        const int32_t n = conn[e * npe + a];
        if (n < 0 || n >= n_nodes) return LMG_ERR_BOUNDS;
        if (l.node_dofs(a) && base[(size_t)n] < 0) {
          base[(size_t)n] = next;
          next += l.node_dofs(a);
        }
      }
      ebase[(size_t)e] = next;
      next += l.n_interior;
    }
    if (next > INT32_MAX) return LMG_ERR_UNSUPPORTED;
    *n_dofs = next;
    if (elem_dofs)
      for (int64_t e = 0; e < n_elem; ++e) {
        int32_t *d = elem_dofs + e * l.nl;
        for (int a = 0; a < npe; ++a) {
          const int c = l.node_dofs(a);
          const int64_t b = base[(size_t)conn[e * npe + a]];
          for (int i = 0; i < c; ++i) *d++ = (int32_t)(b + (a < nv ? i : c - 1 - i));
        }
        for (int i = 0; i < l.n_interior; ++i) *d++ = (int32_t)(ebase[(size_t)e] + i);
      }
  } catch (const std::bad_alloc &) {
    return LMG_ERR_OOM;
  }
  return LMG_OK;
}

lmg_status lmg_dofmap_distribute_device(int32_t device, int64_t n_nodes, int64_t n_elem, int32_t elem_type,
                                        const int32_t *conn, int32_t n_vars, int32_t fe_order, int64_t *n_dofs,
                                        int32_t *elem_dofs) {
  if (!conn || !n_dofs || n_nodes < 0 || n_elem < 0 || n_vars <= 0 || device < 0) return LMG_ERR_ARG;
  const int npe = lmg::nodes_per_elem(elem_type);
  if (!npe) return LMG_ERR_UNSUPPORTED;
  for (int64_t i = 0; i < n_elem * npe; ++i)
    if (conn[i] < 0 || conn[i] >= n_nodes) return LMG_ERR_BOUNDS;
  try {
    int64_t nd = 0;
    const std::string err =
        lmg::distribute_dofs_device(device, n_nodes, n_elem, elem_type, conn, n_vars, fe_order, nd, elem_dofs);
    if (!err.empty()) return err.rfind("device", 0) == 0 ? LMG_ERR_CUDA : LMG_ERR_UNSUPPORTED;
    *n_dofs = nd;
  } catch (const std::bad_alloc &) {
    return LMG_ERR_OOM;
  }
  return LMG_OK;
}

lmg_status lmg_dirichlet_dofs_fe(int64_t n_elem, int32_t elem_type, int32_t fe_order, int32_t n_vars,
                                 const int32_t *elem_dofs, const int8_t *side_bid, const int32_t *bids,
                                 int32_t n_bids, const int32_t *vars, int32_t n_vars_bc, int64_t n_dofs,
                                 uint8_t *constrained) {
  if (fe_order != (3 | LMG_HIERARCHIC))
    return lmg_dirichlet_dofs(n_elem, elem_type, n_vars, elem_dofs, side_bid, bids, n_bids, vars, n_vars_bc,
                              n_dofs, constrained);
  if (!elem_dofs || !side_bid || !constrained || (n_bids > 0 && !bids)) return LMG_ERR_ARG;
  P3Layout l;
  if (!p3_layout(elem_type, l) || n_vars != 1) return LMG_ERR_UNSUPPORTED;
  std::fill(constrained, constrained + n_dofs, (uint8_t)0);
  if (n_vars_bc == 0) return LMG_OK;
  int first[27];
  for (int a = 0, k = 0; a < l.npe; ++a) {
    first[a] = k;
    k += l.node_dofs(a);
  }
  int sn[9];
  for (int64_t e = 0; e < n_elem; ++e)
    for (int s = 0; s < l.nsides; ++s) {
      const int b = side_bid[e * l.nsides + s];
      if (b < 0) continue;
      bool hit = false;
      for (int i = 0; i < n_bids; ++i) hit |= (bids[i] == b);
      if (!hit) continue;
      const int k = lmg::side_nodes(elem_type, s, sn);
      for (int j = 0; j < k; ++j)
        for (int i = 0; i < l.node_dofs(sn[j]); ++i) {
          const int32_t d = elem_dofs[e * l.nl + first[sn[j]] + i];
          if (d < 0 || d >= n_dofs) return LMG_ERR_BOUNDS;
          constrained[d] = 1;
        }
    }
  return LMG_OK;
}

lmg_status lmg_dirichlet_dofs(int64_t n_elem, int32_t elem_type, int32_t n_vars,
                              const int32_t *elem_dofs, const int8_t *side_bid, const int32_t *bids,
                              int32_t n_bids, const int32_t *vars, int32_t n_vars_bc,
                              int64_t n_dofs, uint8_t *constrained) {
  if (!elem_dofs || !side_bid || !constrained || (n_bids > 0 && !bids) ||
      (n_vars_bc > 0 && !vars) || n_vars <= 0)
    return LMG_ERR_ARG;
  const int npe = lmg::nodes_per_elem(elem_type), ns = lmg::sides_per_elem(elem_type);
  if (!npe) return LMG_ERR_UNSUPPORTED;
  for (int i = 0; i < n_vars_bc; ++i)
    if (vars[i] < 0 || vars[i] >= n_vars) return LMG_ERR_ARG;
  std::fill(constrained, constrained + n_dofs, (uint8_t)0);
  const int64_t nl = (int64_t)n_vars * npe;
  int sn[9];
  for (int64_t e = 0; e < n_elem; ++e)
    for (int s = 0; s < ns; ++s) {
      const int b = side_bid[e * ns + s];
      if (b < 0) continue;
      bool hit = false;
      for (int i = 0; i < n_bids; ++i) hit |= (bids[i] == b);
      if (!hit) continue;
      const int k = lmg::side_nodes(elem_type, s, sn);
      for (int i = 0; i < n_vars_bc; ++i)
        for (int j = 0; j < k; ++j) {
          const int32_t d = elem_dofs[e * nl + (int64_t)vars[i] * npe + sn[j]];
          if (d < 0 || d >= n_dofs) return LMG_ERR_BOUNDS;
          constrained[d] = 1;
        }
    }
  return LMG_OK;
}

}  // extern "C"
