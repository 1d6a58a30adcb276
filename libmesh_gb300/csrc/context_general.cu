// Host side of the general assembly path (general.cu): the CSR pattern with
// constraint couplings, the per-element constraint matrices, the slot plan of
// the gather, and the launch sequence.
//
//   DofMap::compute_sparsity + find_connected_dofs   src/base/dof_map.C:1960-1977, 2915-2970
//   DofMap::build_constraint_matrix                  src/base/dof_map_constraints.C:3433-3540
//     (the element's dofs, then its constraining dofs in ascending order)
//   SparseMatrix::add_matrix in element order         src/numerics/petsc_matrix.C:735-755
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <thread>
#include <vector>

#include "context_internal.cuh"
#include "general.cuh"

namespace lmg {

namespace {

int host_threads() {
  const unsigned hw = std::thread::hardware_concurrency();
  return hw ? (int)hw : 4;
}

template <typename Fn>
void parallel_rows(int64_t n, Fn &&fn) {
  std::atomic<int64_t> next{0};
  std::vector<std::thread> th;
  for (int t = 0; t < host_threads(); ++t)
    th.emplace_back([&]() {
      for (;;) {
        const int64_t s0 = next.fetch_add(2048);
        if (s0 >= n) break;
        const int64_t s1 = std::min(n, s0 + 2048);
        for (int64_t r = s0; r < s1; ++r) fn(r);
      }
    });
  for (auto &t : th) t.join();
}

}  // namespace

void general_free(lmg_ctx *c) {
  dfree(c->d_Ebuf); dfree(c->d_Fbuf); dfree(c->d_cptr); dfree(c->d_gfptr);
  dfree(c->d_coff); dfree(c->d_gfoff); dfree(c->d_celem); dfree(c->d_cne); dfree(c->d_ccp); dfree(c->d_ckout);
  dfree(c->d_cfout); dfree(c->d_cbase); dfree(c->d_cebase); dfree(c->d_cci); dfree(c->d_ccv); dfree(c->d_crow);
  c->gen_plan = false;
}

lmg_status general_sparsity(lmg_ctx *c) {
  std::vector<int64_t> rp;
  std::vector<int32_t> cols;
  // on the device; the host build where an element list or a row outgrows
  // the device buffers, or a constraint row refers to a constrained dof
  const bool on_device = c->n_dofs < INT32_MAX && c->n_elem * (int64_t)c->nl < INT32_MAX &&
                         device_constrained_graph(c, rp, cols) == LMG_OK;
  c->sparsity_on_device = on_device;
  if (!on_device) {
    std::vector<int64_t> cp = c->h_cons_ptr;
    if (cp.empty()) cp.assign((size_t)c->n_dofs + 1, 0);
    build_constrained_graph(c->n_elem, c->nl, c->h_elem_dofs.data(), c->n_dofs, cp.data(), c->h_cons_col.data(), rp,
                            cols, host_threads());
  }
  if ((int64_t)cols.size() >= INT32_MAX) return fail(c, LMG_ERR_UNSUPPORTED, "nnz exceeds 32-bit CSR");
  c->nnz = (int64_t)cols.size();
  c->h_row_ptr.resize((size_t)c->n_dofs + 1);
  for (size_t r = 0; r < rp.size(); ++r) c->h_row_ptr[r] = (int32_t)rp[r];
  c->h_col.swap(cols);
  if (!on_device) {
    LMG_CUDA(c, dupload(c, c->d_row_ptr, c->h_row_ptr.data(), c->h_row_ptr.size()));
    LMG_CUDA(c, dupload(c, c->d_col, c->h_col.data(), c->h_col.size()));
  }
  LMG_CUDA(c, dalloc(c->d_K, (size_t)c->nnz));
  LMG_CUDA(c, dalloc(c->d_F, (size_t)c->n_dofs));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  return LMG_OK;
}

lmg_status general_plan(lmg_ctx *c) {
  const int N = c->nl;
  const int64_t E = c->n_elem;
  if (c->n_vars != 1 || (N > GEN_MAX_N && !(c->hier3 && N <= 64)))
    return fail(c, LMG_ERR_UNSUPPORTED, "general path: one variable and at most 27 dofs per element");
  // the cubic hex kernel masks homogeneous Dirichlet rows itself
  const bool use_cons = !(c->h_constrained.empty() || hier3_masks(c) || c->persist_pattern);
  c->plan_built_on_device = false;
  if (c->plan_on_device && c->n_dofs < INT32_MAX && E * (int64_t)N < INT32_MAX) {
    // on the device; the host build below where a list or a constraint
    // matrix outgrows the device buffers
    int64_t kr = 0, fr = 0, n_cons = 0;
    int max_ne = 0, max_ent = 0;
    const lmg_status st = general_plan_device(c, use_cons, kr, fr, max_ne, max_ent, n_cons);
    if (st == LMG_ERR_NEW_NONZERO)
      return fail(c, st, "an element couples a pair outside the sparsity pattern");
    if (st == LMG_ERR_OOM) return fail(c, st, "general plan: device memory");
    if (st == LMG_ERR_CUDA) return fail(c, st, "general plan: CUDA error");
    if (st == LMG_OK) {
      c->n_cons_elem = n_cons;
      c->cons_max_ne = max_ne;
      c->cons_max_ent = max_ent;
      LMG_CUDA(c, dalloc(c->d_Ebuf, (size_t)kr));
      LMG_CUDA(c, dalloc(c->d_Fbuf, (size_t)fr));
      LMG_CUDA(c, cudaStreamSynchronize(c->stream));
      c->plan_built_on_device = true;
      c->gen_plan = true;
      return LMG_OK;
    }
  }
  if (c->h_row_ptr.empty()) {  // pattern built by the block path: bring it to the host
    c->h_row_ptr.resize((size_t)c->n_dofs + 1);
    c->h_col.resize((size_t)c->nnz);
    LMG_CUDA(c, cudaMemcpyAsync(c->h_row_ptr.data(), c->d_row_ptr, sizeof(int32_t) * (c->n_dofs + 1),
                                cudaMemcpyDeviceToHost, c->stream));
    LMG_CUDA(c, cudaMemcpyAsync(c->h_col.data(), c->d_col, sizeof(int32_t) * c->nnz, cudaMemcpyDeviceToHost,
                                c->stream));
    LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  }
  const bool have_rows = !c->h_cons_ptr.empty();
  auto row_of = [&](int32_t d, int64_t &b, int64_t &e) {
    b = have_rows ? c->h_cons_ptr[(size_t)d] : 0;
    e = have_rows ? c->h_cons_ptr[(size_t)d + 1] : 0;
  };
  const uint8_t *cons = use_cons ? c->h_constrained.data() : nullptr;
  // per element: output dof list, its length and where its matrix / vector sit
  std::vector<int64_t> lptr((size_t)E + 1, 0);
  std::vector<int32_t> ldofs;
  ldofs.reserve((size_t)(E * N));
  std::vector<int64_t> kbase((size_t)E), fbase((size_t)E);
  std::vector<int32_t> celem, cne, ccp;
  std::vector<int64_t> ckout, cfout, cbase, cebase;
  std::vector<uint8_t> cci;
  std::vector<double> ccv;
  std::vector<uint64_t> crow;
  int64_t kr = E * (int64_t)N * N, fr = E * (int64_t)N;  // enlarged regions start after the raw ones
  std::vector<int32_t> dofs;
  std::vector<std::vector<std::pair<int, double>>> col;
  int max_ne = 0, max_ent = 0;
  for (int64_t e = 0; e < E; ++e) {
    const int32_t *ed = &c->h_elem_dofs[(size_t)(e * N)];
    bool any = false;
    for (int i = 0; i < N && cons; ++i) any |= cons[ed[i]] != 0;
    if (!any) {
      ldofs.insert(ldofs.end(), ed, ed + N);
      kbase[(size_t)e] = e * (int64_t)N * N;
      fbase[(size_t)e] = e * (int64_t)N;
    } else {
      // build_constraint_matrix: own dofs, then the constraining dofs not among them (ascending)
      dofs.assign(ed, ed + N);
      std::vector<int32_t> extra;
      for (int i = 0; i < N; ++i)
        if (cons[ed[i]]) {
          int64_t b, en;
          row_of(ed[i], b, en);
          for (int64_t k = b; k < en; ++k) extra.push_back(c->h_cons_col[(size_t)k]);
        }
      std::sort(extra.begin(), extra.end());
      extra.erase(std::unique(extra.begin(), extra.end()), extra.end());
      for (int32_t x : extra)
        if (std::find(ed, ed + N, x) == ed + N) dofs.push_back(x);
      const int ne = (int)dofs.size();
      if (ne > GEN_MAX_NE) return fail(c, LMG_ERR_UNSUPPORTED, "constrained element with too many dofs", e);
      col.assign((size_t)ne, {});
      uint64_t rows = 0;
      for (int i = 0; i < N; ++i) {
        if (!cons[ed[i]]) {
          col[(size_t)i].emplace_back(i, 1.0);
          continue;
        }
        rows |= 1ull << i;
        int64_t b, en;
        row_of(ed[i], b, en);
        for (int64_t k = b; k < en; ++k) {
          const double v = c->h_cons_val[(size_t)k];
          if (v == 0.0) continue;  // the reference's dense products skip zero entries
          const int j = (int)(std::find(dofs.begin(), dofs.end(), c->h_cons_col[(size_t)k]) - dofs.begin());
          col[(size_t)j].emplace_back(i, v);
        }
      }
      int n_ent = 0;
      for (auto &cl : col) n_ent += (int)cl.size();
      if (n_ent > GEN_MAX_ENTRIES) return fail(c, LMG_ERR_UNSUPPORTED, "constraint matrix too large", e);
      max_ne = std::max(max_ne, ne);
      max_ent = std::max(max_ent, n_ent);
      celem.push_back((int32_t)e);
      cne.push_back(ne);
      ckout.push_back(kr);
      cfout.push_back(fr);
      cbase.push_back((int64_t)ccp.size());
      cebase.push_back((int64_t)cci.size());
      crow.push_back(rows);
      int acc = 0;
      for (int q = 0; q < ne; ++q) {
        ccp.push_back(acc);
        for (auto &it : col[(size_t)q]) {  // ascending row index by construction
          cci.push_back((uint8_t)it.first);
          ccv.push_back(it.second);
        }
        acc += (int)col[(size_t)q].size();
      }
      ccp.push_back(acc);
      ldofs.insert(ldofs.end(), dofs.begin(), dofs.end());
      kbase[(size_t)e] = kr;
      fbase[(size_t)e] = fr;
      kr += (int64_t)ne * ne;
      fr += ne;
    }
    lptr[(size_t)e + 1] = (int64_t)ldofs.size();
  }
  if (kr >= (int64_t)UINT32_MAX || fr >= (int64_t)UINT32_MAX)
    return fail(c, LMG_ERR_UNSUPPORTED, "element matrices exceed 32-bit offsets");
  // incidence of each row: (element, position) in element order
  const int64_t nd = c->n_dofs;
  std::vector<int64_t> iptr((size_t)nd + 1, 0);
  for (int32_t d : ldofs) iptr[(size_t)d + 1]++;
  for (int64_t d = 0; d < nd; ++d) iptr[(size_t)d + 1] += iptr[(size_t)d];
  std::vector<int32_t> ie(ldofs.size()), ip(ldofs.size());
  {
    std::vector<int64_t> cur(iptr.begin(), iptr.end() - 1);
    for (int64_t e = 0; e < E; ++e)
      for (int64_t k = lptr[(size_t)e]; k < lptr[(size_t)e + 1]; ++k) {
        const int64_t o = cur[(size_t)ldofs[(size_t)k]]++;
        ie[(size_t)o] = (int32_t)e;
        ip[(size_t)o] = (int32_t)(k - lptr[(size_t)e]);
      }
  }
  // slot counts, then the contribution offsets in element order
  const int64_t nnz = c->nnz;
  std::vector<int64_t> cptr((size_t)nnz + 1, 0);
  std::atomic<int> missing{0};
  parallel_rows(nd, [&](int64_t r) {
    const int32_t *b = c->h_col.data() + c->h_row_ptr[(size_t)r], *en = c->h_col.data() + c->h_row_ptr[(size_t)r + 1];
    for (int64_t t = iptr[(size_t)r]; t < iptr[(size_t)r + 1]; ++t) {
      const int64_t e = ie[(size_t)t];
      for (int64_t k = lptr[(size_t)e]; k < lptr[(size_t)e + 1]; ++k) {
        const int32_t *it = std::lower_bound(b, en, ldofs[(size_t)k]);
        if (it == en || *it != ldofs[(size_t)k]) {
          missing = 1;
          continue;
        }
        cptr[(size_t)(it - c->h_col.data()) + 1]++;
      }
    }
  });
  if (missing) return fail(c, LMG_ERR_NEW_NONZERO, "an element couples a pair outside the sparsity pattern");
  for (int64_t s = 0; s < nnz; ++s) cptr[(size_t)s + 1] += cptr[(size_t)s];
  std::vector<uint32_t> coff((size_t)cptr[(size_t)nnz]);
  parallel_rows(nd, [&](int64_t r) {
    const int32_t *b = c->h_col.data() + c->h_row_ptr[(size_t)r], *en = c->h_col.data() + c->h_row_ptr[(size_t)r + 1];
    std::vector<int64_t> cur((size_t)(en - b));
    for (size_t j = 0; j < cur.size(); ++j) cur[j] = cptr[(size_t)(b - c->h_col.data()) + j];
    for (int64_t t = iptr[(size_t)r]; t < iptr[(size_t)r + 1]; ++t) {
      const int64_t e = ie[(size_t)t], p = ip[(size_t)t];
      const int64_t ne = lptr[(size_t)e + 1] - lptr[(size_t)e];
      for (int64_t k = lptr[(size_t)e]; k < lptr[(size_t)e + 1]; ++k) {
        const int32_t *it = std::lower_bound(b, en, ldofs[(size_t)k]);
        coff[(size_t)cur[(size_t)(it - b)]++] = (uint32_t)(kbase[(size_t)e] + p * ne + (k - lptr[(size_t)e]));
      }
    }
  });
  std::vector<uint32_t> foff(ldofs.size());
  for (int64_t d = 0; d < nd; ++d)
    for (int64_t t = iptr[(size_t)d]; t < iptr[(size_t)d + 1]; ++t)
      foff[(size_t)t] = (uint32_t)(fbase[(size_t)ie[(size_t)t]] + ip[(size_t)t]);
  general_free(c);
  c->n_cons_elem = (int64_t)celem.size();
  c->cons_max_ne = max_ne;
  c->cons_max_ent = max_ent;
  LMG_CUDA(c, dupload(c, c->d_cptr, cptr.data(), cptr.size()));
  LMG_CUDA(c, dupload(c, c->d_coff, coff.data(), coff.size()));
  LMG_CUDA(c, dupload(c, c->d_gfptr, iptr.data(), iptr.size()));
  LMG_CUDA(c, dupload(c, c->d_gfoff, foff.data(), foff.size()));
  LMG_CUDA(c, dupload(c, c->d_celem, celem.data(), celem.size()));
  LMG_CUDA(c, dupload(c, c->d_cne, cne.data(), cne.size()));
  LMG_CUDA(c, dupload(c, c->d_ckout, ckout.data(), ckout.size()));
  LMG_CUDA(c, dupload(c, c->d_cfout, cfout.data(), cfout.size()));
  LMG_CUDA(c, dupload(c, c->d_cbase, cbase.data(), cbase.size()));
  LMG_CUDA(c, dupload(c, c->d_cebase, cebase.data(), cebase.size()));
  LMG_CUDA(c, dupload(c, c->d_ccp, ccp.data(), ccp.size()));
  LMG_CUDA(c, dupload(c, c->d_cci, cci.data(), cci.size()));
  LMG_CUDA(c, dupload(c, c->d_ccv, ccv.data(), ccv.size()));
  LMG_CUDA(c, dupload(c, c->d_crow, crow.data(), crow.size()));
  LMG_CUDA(c, dalloc(c->d_Ebuf, (size_t)kr));
  LMG_CUDA(c, dalloc(c->d_Fbuf, (size_t)fr));
  LMG_CUDA(c, cudaStreamSynchronize(c->stream));
  c->gen_plan = true;
  return LMG_OK;
}

lmg_status general_assemble(lmg_ctx *c, bool mixed) {
  GenElemArgs a{};
  a.n_elem = c->n_elem;
  a.xyz = c->d_xyz;
  a.conn = c->d_conn;
  a.coef = c->d_coef;
  a.nodal_f = c->d_f;
  a.D6 = c->d_D6;
  a.kappa = c->kappa;
  a.n_modes = c->n_modes;
  a.modes = c->d_modes;
  a.Kraw = c->d_Ebuf;
  a.Fraw = c->d_Fbuf;
  a.status = c->d_status;
  a.bad_elem = c->d_bad;
  a.fe = c->dfe;
  if (c->hier3) launch_hier3(c, mixed);
  else launch_gen_elements(c->form, c->tab.n, c->tab.q, mixed, a, c->n_sm * c->ctas_per_sm / 4, c->stream);
  c->launches++;
  if (c->n_cons_elem) {
    ConsArgs k{};
    k.n_cons = c->n_cons_elem;
    k.N = c->nl;
    k.max_ne = c->cons_max_ne;
    k.max_ent = c->cons_max_ent;
    k.elem = c->d_celem;
    k.ne = c->d_cne;
    k.kout = c->d_ckout;
    k.fout = c->d_cfout;
    k.cbase = c->d_cbase;
    k.ccp = c->d_ccp;
    k.ebase = c->d_cebase;
    k.ci = c->d_cci;
    k.cv = c->d_ccv;
    k.rowmask = c->d_crow;
    k.Kraw = c->d_Ebuf;
    k.Fraw = c->d_Fbuf;
    k.Ebuf = c->d_Ebuf;
    k.Fbuf = c->d_Fbuf;
    launch_constrain(k, mixed, c->n_sm, c->stream);
    c->launches++;
  }
  return LMG_OK;
}

void general_gather(lmg_ctx *c, bool mixed, int64_t P0, int64_t P1) {
  // element matrices are double (FP64 drop-in) or float (mixed form)
  int64_t s0 = 0, s1 = c->nnz;
  if (P1 < 0) {
    P1 = c->n_dofs;
  } else {
    s0 = c->h_row_ptr[(size_t)P0];
    s1 = c->h_row_ptr[(size_t)P1];
  }
  launch_gather_full(c->nnz, c->d_cptr, c->d_coff, c->d_Ebuf, mixed, c->d_K, c->n_dofs, c->d_gfptr, c->d_gfoff,
                     c->d_Fbuf, c->d_F, c->n_sm, c->stream, s0, s1, P0, P1);
  c->launches++;
}

}  // namespace lmg

extern "C" lmg_status lmg_constraint_rows_upload(lmg_ctx *c, const uint8_t *constrained, const int64_t *cons_ptr,
                                                 const int32_t *cons_col, const double *cons_val) {
  using namespace lmg;
  if (!c || !constrained || !cons_ptr) return fail(c, LMG_ERR_ARG, "constraint_rows_upload: bad argument");
  if (!c->n_dofs) return fail(c, LMG_ERR_STATE, "constraint_rows_upload: upload the dofmap first");
  const int64_t nent = cons_ptr[c->n_dofs];
  if (cons_ptr[0] != 0 || nent < 0 || (nent > 0 && (!cons_col || !cons_val)))
    return fail(c, LMG_ERR_ARG, "constraint_rows_upload: bad row pointers");
  for (int64_t d = 0; d < c->n_dofs; ++d) {
    if (cons_ptr[d + 1] < cons_ptr[d]) return fail(c, LMG_ERR_ARG, "constraint_rows_upload: bad row pointers");
    if (cons_ptr[d + 1] > cons_ptr[d] && !constrained[d])
      return fail(c, LMG_ERR_ARG, "constraint_rows_upload: a row for an unconstrained dof");
    for (int64_t k = cons_ptr[d]; k < cons_ptr[d + 1]; ++k)
      if (cons_col[k] < 0 || cons_col[k] >= c->n_dofs || constrained[cons_col[k]])
        return fail(c, LMG_ERR_BOUNDS, "constraint_rows_upload: rows must refer to free dofs only");
  }
  const lmg_status st = lmg_constraints_upload(c, constrained);
  if (st) return st;
  c->h_cons_ptr.assign(cons_ptr, cons_ptr + c->n_dofs + 1);
  c->h_cons_col.assign(cons_col, cons_col + nent);
  c->h_cons_val.assign(cons_val, cons_val + nent);
  c->has_rows = nent > 0;
  c->have_sparsity = false;
  return LMG_OK;
}
