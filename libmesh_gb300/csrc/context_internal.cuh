// Internal state of the device context (shared by context.cu and
// context_general.cu).  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "assemble.cuh"
#include "lmg_internal.h"

struct lmg_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int n_sm = 152;
  int ctas_per_sm = 32;  // element-kernel grid (grid-stride), set by the batch autotuner
  bool grid_set = false;  // ctas_per_sm chosen by the caller (lmg_context_set_grid)
  bool tensor_cores = true;  // mixed form: per-point Gram products on the tensor cores where built
  int64_t launches = 0;
  std::string err;
  int64_t err_elem = -1;
  // mesh
  int elem_type = 0, npe = 0;
  int64_t n_nodes = 0, n_elem = 0;
  std::vector<double> h_xyz;
  std::vector<int32_t> h_conn;
  double *d_xyz = nullptr;
  int32_t *d_conn = nullptr;
  std::vector<int32_t> h_aff, h_gen;  // affine / general element lists
  int32_t *d_aff = nullptr, *d_gen = nullptr;
  // dofmap
  int n_vars = 0, nl = 0, bs = 1, nb = 0;
  int64_t n_dofs = 0, n_blocks = 0;
  std::vector<int32_t> h_elem_dofs, h_eb;
  int32_t *d_eb = nullptr;
  // constraints
  std::vector<uint8_t> h_constrained;
  uint64_t *d_cmask = nullptr;
  uint8_t *d_cons = nullptr;
  // sparsity and plan
  bool have_sparsity = false;
  int64_t nnz = 0, nnzb = 0;
  int64_t *d_brow_ptr = nullptr;
  int32_t *d_bcol = nullptr, *d_row_ptr = nullptr, *d_col = nullptr;
  int32_t *d_bptr = nullptr, *d_bcontrib = nullptr, *d_fptr = nullptr, *d_fcontrib = nullptr;
  std::vector<int32_t> h_rowptr_blk;      // host copy of row_ptr (block path), for chunked output copies
  std::vector<int32_t> h_row_pmax;        // prefix maximum of each block row's last contributing element
  cudaStream_t copy_stream = nullptr;     // device-to-host copies overlapped with the insertion
  std::vector<cudaEvent_t> chunk_ev;
  uint8_t *d_relslot = nullptr;  // [E][nb][nb] slot of block (a, b) in block row of a (fused mixed form)
  uint8_t *d_rowcons = nullptr;  // [n_blocks] block row touches a constrained dof (fused mixed form)
  int32_t *d_bdiag = nullptr;    // [n_blocks] position of the diagonal slot in each block row
  int max_bdeg = 0;              // largest block-row degree
  float *d_geo = nullptr;        // [E][NG] per-element operands (fused mixed form)
  // form
  bool have_form = false;
  int form = 0, fe_order = 0, q_order = 0;
  double nu = 0.3;
  lmg::FETables tab;
  double *d_tab = nullptr;
  lmg::DevFE dfe{};
  double *d_coef = nullptr, *d_f = nullptr;
  float2 *d_f2 = nullptr;  // nodal load as double-float pairs
  // work and result buffers
  float2 *d_Kdiag2 = nullptr, *d_Koff2 = nullptr;
  float2 *d_Fe2 = nullptr;
  float2 *d_Re2 = nullptr;  // per-element residuals of lmg_residual
  double *d_K = nullptr, *d_F = nullptr;
  float *d_Koff32 = nullptr;
  int *d_status = nullptr;
  unsigned long long *d_bad = nullptr;
  // general path (general.cu): constraint rows with coefficients or a
  // nonsymmetric form; full element matrices, C^T K C, slot gather
  std::vector<int64_t> h_cons_ptr;   // [n_dofs+1] constraint rows (empty: none uploaded)
  std::vector<int32_t> h_cons_col;
  std::vector<double> h_cons_val;
  bool has_rows = false;             // some row has coefficients
  bool general = false;              // assembly runs through general.cu
  bool gen_plan = false;
  std::vector<int32_t> h_row_ptr, h_col;  // host copy of the CSR pattern
  double kappa = 0.0;
  int n_modes = 0;
  double *d_D6 = nullptr, *d_modes = nullptr, *d_Ebuf = nullptr, *d_Fbuf = nullptr;
  int64_t *d_cptr = nullptr, *d_gfptr = nullptr;
  uint32_t *d_coff = nullptr, *d_gfoff = nullptr;
  int64_t n_cons_elem = 0;
  int cons_max_ne = 0, cons_max_ent = 0;
  int32_t *d_celem = nullptr, *d_cne = nullptr, *d_ccp = nullptr;
  int64_t *d_ckout = nullptr, *d_cfout = nullptr, *d_cbase = nullptr, *d_cebase = nullptr;
  uint8_t *d_cci = nullptr;
  double *d_ccv = nullptr;
  uint64_t *d_crow = nullptr;
  // per-pattern HIERARCHIC elements (hier3.cu): cubic hexes, tets and prisms,
  // quadratic prisms; general path
  bool hier3 = false;
  bool plan_on_device = true;         // general_plan tries the device build first
  bool plan_built_on_device = false;  // the last general plan came from the device
  bool sparsity_on_device = false;  // the general path's graph came from device_constrained_graph
  bool persist_pattern = false;     // block-path system also held in per-pattern form (persistent batch)
  int32_t *d_h3batch = nullptr, *d_h3order = nullptr;  // element batches of one orientation pattern
  float2 *d_h3D = nullptr;           // per-pattern reference tensors, double-float pairs
  float *d_h3Df = nullptr;           // the same rounded to FP32 (mixed form)
  double *d_h3M = nullptr, *d_h3gd = nullptr;
  int64_t h3_nbatch = 0;
  int h3_patterns = 0;
  int h3_tile = 8;                    // elements per CTA tile (4, 8, 16 or 32; the batch tuner picks it)
  std::vector<int32_t> h3_order, h3_pid;  // host copies: elements sorted by pattern, pattern of each
  // PerfLog-style stage timing (CUDA events on the context stream)
  bool perflog = false;
  std::vector<cudaEvent_t> ev;       // 3 per logged assemble call
  double log_ms[2] = {0.0, 0.0};     // element kernels, gather
  int64_t log_calls = 0;
};

namespace lmg {


template <typename T>
inline void dfree(T *&p) {
  if (p) cudaFree((void *)p);
  p = nullptr;
}

inline lmg_status fail(lmg_ctx *c, lmg_status code, const std::string &msg, int64_t elem = -1) {
  if (c) {
    c->err = msg;
    c->err_elem = elem;
  }
  return code;
}

#define LMG_CUDA(ctx, call)                                                        \
  do {                                                                             \
    cudaError_t e_ = (call);                                                       \
    if (e_ != cudaSuccess)                                                         \
      return fail(ctx, e_ == cudaErrorMemoryAllocation ? LMG_ERR_OOM : LMG_ERR_CUDA, \
                  std::string(#call) + ": " + cudaGetErrorString(e_));             \
  } while (0)

template <typename T>
inline cudaError_t dalloc(T *&p, size_t n) {
  dfree(p);
  if (n == 0) n = 1;
  return cudaMalloc((void **)&p, n * sizeof(T));
}

template <typename T>
inline cudaError_t dupload(lmg_ctx *c, T *&p, const T *h, size_t n) {
  cudaError_t e = dalloc(p, n);
  if (e != cudaSuccess) return e;
  if (n) e = cudaMemcpyAsync(p, h, n * sizeof(T), cudaMemcpyHostToDevice, c->stream);
  return e;
}

// general.cu path (context_general.cu)
lmg_status general_sparsity(lmg_ctx *c);   // CSR with the constraint couplings
// find_connected_dofs on the device: rows into rp / cols and d_row_ptr /
// d_col; LMG_ERR_UNSUPPORTED when the host build must take over.
lmg_status device_constrained_graph(lmg_ctx *c, std::vector<int64_t> &rp, std::vector<int32_t> &cols);
lmg_status general_plan(lmg_ctx *c);       // constraint columns, slot plan, buffers
// general_plan's arrays built on the device (plan_device.cu); kr / fr are the
// element-matrix and element-vector buffer sizes.  LMG_ERR_UNSUPPORTED when
// the host build must take over.
lmg_status general_plan_device(lmg_ctx *c, bool use_cons, int64_t &kr, int64_t &fr, int &max_ne, int &max_ent,
                               int64_t &n_cons);
// element and constraint kernels; mixed: FP32 contraction, FP64 map and sums
lmg_status general_assemble(lmg_ctx *c, bool mixed);
// slot gather into the K rows and F entries [P0, P1) (P1 < 0: all)
void general_gather(lmg_ctx *c, bool mixed, int64_t P0 = 0, int64_t P1 = -1);
// hier3.cu
// FE types whose shapes follow each element's orientation pattern and that
// take the per-pattern tables of hier3.cu: HIERARCHIC THIRD on HEX27, TET14
// and PRISM21, HIERARCHIC SECOND on PRISM18; their dofs per element (0 for
// any other type).
int pattern_fe_dofs(int elem_type, int fe_order);
void hier3_free(lmg_ctx *c);
lmg_status hier3_form_set(lmg_ctx *c, int32_t form, int32_t q_order, const double *elem_coef,
                          const double *nodal_f);
void launch_hier3(lmg_ctx *c, bool mixed);
// Regroups the per-pattern elements into CTA tiles of `tile` elements (4, 8,
// 16 or 32); the element matrices do not depend on the grouping.
lmg_status hier3_set_tile(lmg_ctx *c, int tile);
// Per-pattern tables on the device (hier3.cu), and a block-path Poisson
// system converted to that form for the persistent batch.
lmg_status pattern_upload(lmg_ctx *c, const Hier3Tables &h);
lmg_status pattern_from_block(lmg_ctx *c);
bool hier3_masks(const lmg_ctx *c);  // Dirichlet rows applied by the element kernel
void general_free(lmg_ctx *c);             // plan and work buffers

}  // namespace lmg
