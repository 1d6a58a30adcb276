// Batched assembly: many independent systems (meshes, forms, element types)
// assembled as one CUDA graph.  libMesh assembles each system
// through its own System::assemble call (src/systems/system.C:554-561); a
// batch replays the kernels of all of them with one graph launch, after an
// autotuner has picked each system's element-kernel grid.
//
// Life cycle: lmg_batch_add registers a fully set-up context (sparsity,
// form); lmg_batch_tune times a few grid sizes per context, and for the
// per-pattern HIERARCHIC members the number of elements each CTA takes per
// tile (4 to 32: more elements share one read of the pattern's tables, fewer
// spread a small system over more SMs); lmg_batch_assemble
// warms every context up once (lazy plans, buffers), then captures their
// assemblies into a graph per precision and replays it.  The capture forks
// from the batch stream into every context's own stream and joins back, so
// the graph holds one independent branch per system and small systems run
// side by side.
#include <cuda_runtime.h>

#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include "batch_persistent.cuh"
#include "context_internal.cuh"

// Device state of the persistent mode: members, work items, queue head,
// per-member tile counters and a status word.
struct PersistentState {
  lmg::PMember *mem = nullptr;
  lmg::PItem *items = nullptr;
  int64_t n_items = 0;
  unsigned long long *head = nullptr;
  unsigned int *done = nullptr;
  int *status = nullptr;
  int tile = 0, grid = 0;   // the settings the members and items were prepared for
  bool mixed = false;
  cudaGraphExec_t exec = nullptr;
  cudaGraph_t graph = nullptr;
};

struct lmg_batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<lmg_ctx *> ctx;
  std::vector<cudaEvent_t> join;                  // one per context, capture-time joins
  cudaEvent_t fork = nullptr;
  cudaGraphExec_t exec[2] = {nullptr, nullptr};  // per precision
  cudaGraph_t graph[2] = {nullptr, nullptr};
  bool warm[2] = {false, false};
  int64_t launches = 0;    // kernels in one replay
  std::string err;
  bool persistent = false;     // one persistent launch per replay (lmg_batch_set_persistent)
  bool p_hybrid = false;       // ... over the per-pattern members only, the others' own kernels beside it
  int p_tile = 8, p_ctas = 0;  // its tile (elements per CTA) and CTAs per SM (0: occupancy)
  PersistentState ps;
};

namespace {

void drop_persistent(lmg_batch *b) {
  PersistentState &ps = b->ps;
  if (ps.exec) cudaGraphExecDestroy(ps.exec);
  if (ps.graph) cudaGraphDestroy(ps.graph);
  for (void *p : {(void *)ps.mem, (void *)ps.items, (void *)ps.head, (void *)ps.done, (void *)ps.status})
    if (p) cudaFree(p);
  ps = PersistentState();
}

void drop_graphs(lmg_batch *b) {
  for (int p = 0; p < 2; ++p) {
    if (b->exec[p]) cudaGraphExecDestroy(b->exec[p]);
    if (b->graph[p]) cudaGraphDestroy(b->graph[p]);
    b->exec[p] = nullptr;
    b->graph[p] = nullptr;
  }
  drop_persistent(b);
}

lmg_status bfail(lmg_batch *b, lmg_status code, const std::string &msg) {
  if (b) b->err = msg;
  return code;
}

// Assemble every context once on its own stream with outputs kept on the
// device, then check each context's status.
lmg_status run_all(lmg_batch *b, int precision) {
  for (lmg_ctx *c : b->ctx) {
    const lmg_status st = lmg_assemble(c, precision, nullptr, nullptr, 1);
    if (st) return bfail(b, st, "batch: assemble failed: " + c->err);
  }
  for (lmg_ctx *c : b->ctx) {
    const lmg_status st = lmg_synchronize(c);
    if (st) return bfail(b, st, "batch: " + c->err);
  }
  return LMG_OK;
}

// Members in per-pattern form with their insertion plans, the work list
// (every member's element tiles, then every member's insertion ranges) and
// the graph of one replay: the queue head and tile counters cleared, then the
// persistent kernel.
lmg_status prepare_persistent(lmg_batch *b, int precision) {
  const bool mixed = precision == LMG_MIXED;
  PersistentState &ps = b->ps;
  const int tile = b->p_tile;
  int n_sm = 0;
  cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, b->device);
  const int per_sm = b->p_ctas > 0 ? b->p_ctas : lmg::persistent_ctas_per_sm(mixed, tile);
  const int grid = n_sm * per_sm;
  if (ps.exec && ps.tile == tile && ps.grid == grid && ps.mixed == mixed) return LMG_OK;
  drop_persistent(b);
  std::vector<lmg::PMember> mem;
  std::vector<lmg::PItem> items;
  std::vector<size_t> own;  // hybrid: members that keep their own kernels
  for (size_t i = 0; i < b->ctx.size(); ++i) {
    lmg_ctx *c = b->ctx[i];
    if (b->p_hybrid && !c->hier3) {
      own.push_back(i);
      continue;
    }
    lmg_status st = c->hier3 ? lmg::hier3_set_tile(c, tile) : lmg::pattern_from_block(c);
    if (!st && !c->hier3) st = lmg::hier3_set_tile(c, tile);
    if (!st && !c->gen_plan) st = lmg::general_plan(c);
    if (st) return bfail(b, st, "batch: member " + std::to_string(i) + ": " + c->err);
    lmg::PMember m{};
    m.el.n_batch = c->h3_nbatch;
    m.el.batch = c->d_h3batch;
    m.el.order = c->d_h3order;
    m.el.xyz = c->d_xyz;
    m.el.conn = c->d_conn;
    m.el.npe = c->npe;
    m.el.coef = c->d_coef;
    m.el.nodal_f = c->d_f;
    m.el.cmask = c->d_cmask;
    m.el.D = c->d_h3D;
    m.el.Df = c->d_h3Df;
    m.el.M = c->d_h3M;
    m.el.gd0 = c->d_h3gd;
    m.el.Kraw = c->d_Ebuf;
    m.el.Fraw = c->d_Fbuf;
    m.el.status = c->d_status;
    m.el.bad_elem = c->d_bad;
    m.N = c->nl;
    m.G = c->hier3 ? c->tab.n_geo : c->npe;
    if (!lmg::persistent_kind_built(m.N, m.G))
      return bfail(b, LMG_ERR_UNSUPPORTED, "batch: no persistent kernel for member " + std::to_string(i));
    m.n_tiles = c->h3_nbatch;
    m.nnz = c->nnz;
    m.n_dofs = c->n_dofs;
    m.cptr = c->d_cptr;
    m.coff = c->d_coff;
    m.fptr = c->d_gfptr;
    m.foff = c->d_gfoff;
    m.K = c->d_K;
    m.F = c->d_F;
    mem.push_back(m);
  }
  for (size_t i = 0; i < mem.size(); ++i)
    for (int64_t t = 0; t < mem[i].n_tiles; ++t) items.push_back({(int32_t)i, 0, t});
  for (size_t i = 0; i < mem.size(); ++i) {
    const int64_t n = (mem[i].nnz + mem[i].n_dofs + lmg::PB_SLOTS - 1) / lmg::PB_SLOTS;
    for (int64_t t = 0; t < n; ++t) items.push_back({(int32_t)i, 1, t});
  }
  auto up = [&](auto *&d, const auto *h, size_t n) {
    return cudaMalloc((void **)&d, sizeof(*h) * (n ? n : 1)) == cudaSuccess &&
           (n == 0 || cudaMemcpy(d, h, sizeof(*h) * n, cudaMemcpyHostToDevice) == cudaSuccess);
  };
  if (!up(ps.mem, mem.data(), mem.size()) || !up(ps.items, items.data(), items.size()) ||
      cudaMalloc((void **)&ps.head, sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc((void **)&ps.done, sizeof(unsigned int) * (mem.size() ? mem.size() : 1)) != cudaSuccess ||
      cudaMalloc((void **)&ps.status, sizeof(int)) != cudaSuccess ||
      cudaMemset(ps.status, 0, sizeof(int)) != cudaSuccess) {
    drop_persistent(b);
    return bfail(b, LMG_ERR_OOM, "batch: persistent state allocation failed");
  }
  ps.n_items = (int64_t)items.size();
  ps.tile = tile;
  ps.grid = grid;
  ps.mixed = mixed;
  if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
    return bfail(b, LMG_ERR_CUDA, "batch: capture failed to start");
  cudaError_t fe = cudaEventRecord(b->fork, b->stream);
  int64_t l0 = 0, l1 = 0;
  for (size_t i : own) l0 += b->ctx[i]->launches;
  lmg_status ast = LMG_OK;
  // hybrid: the members with their own kernels join as branches beside the persistent launch
  for (size_t k = 0; k < own.size() && fe == cudaSuccess && !ast; ++k) {
    lmg_ctx *c = b->ctx[own[k]];
    fe = cudaStreamWaitEvent(c->stream, b->fork, 0);
    if (fe != cudaSuccess) break;
    ast = lmg_assemble(c, precision, nullptr, nullptr, 1);
    if (ast) break;
    fe = cudaEventRecord(b->join[own[k]], c->stream);
    if (fe == cudaSuccess) fe = cudaStreamWaitEvent(b->stream, b->join[own[k]], 0);
  }
  for (size_t i : own) l1 += b->ctx[i]->launches;
  if (!mem.empty()) {
    cudaMemsetAsync(ps.head, 0, sizeof(unsigned long long), b->stream);
    cudaMemsetAsync(ps.done, 0, sizeof(unsigned int) * mem.size(), b->stream);
    lmg::launch_batch_persistent(ps.mem, ps.items, ps.n_items, ps.head, ps.done, ps.status, mixed, tile, grid,
                                 b->stream);
  }
  const cudaError_t le = cudaGetLastError();
  const cudaError_t ce = cudaStreamEndCapture(b->stream, &ps.graph);
  if (ast || fe != cudaSuccess || le != cudaSuccess || ce != cudaSuccess || !ps.graph ||
      cudaGraphInstantiate(&ps.exec, ps.graph, 0) != cudaSuccess) {
    drop_persistent(b);
    return bfail(b, ast ? ast : LMG_ERR_CUDA, "batch: persistent graph failed");
  }
  b->launches = (mem.empty() ? 0 : 1) + (l1 - l0);
  return LMG_OK;
}

}  // namespace

extern "C" {

lmg_status lmg_batch_create(lmg_batch **out, int32_t device) {
  if (!out) return LMG_ERR_ARG;
  *out = nullptr;
  lmg_batch *b = new (std::nothrow) lmg_batch;
  if (!b) return LMG_ERR_OOM;
  b->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete b;
    return LMG_ERR_CUDA;
  }
  if (cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
    cudaStreamDestroy(b->stream);
    delete b;
    return LMG_ERR_CUDA;
  }
  *out = b;
  return LMG_OK;
}

lmg_status lmg_batch_destroy(lmg_batch *b) {
  if (!b) return LMG_OK;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  for (lmg_ctx *c : b->ctx) cudaStreamSynchronize(c->stream);
  drop_graphs(b);
  for (cudaEvent_t e : b->join) cudaEventDestroy(e);
  cudaEventDestroy(b->fork);
  cudaStreamDestroy(b->stream);
  delete b;
  return LMG_OK;
}

lmg_status lmg_batch_add(lmg_batch *b, lmg_ctx *c) {
  if (!b || !c) return bfail(b, LMG_ERR_ARG, "batch_add: bad argument");
  if (c->device != b->device) return bfail(b, LMG_ERR_ARG, "batch_add: context on another device");
  if (!c->have_sparsity || !c->have_form) return bfail(b, LMG_ERR_STATE, "batch_add: build sparsity and form first");
  if (std::find(b->ctx.begin(), b->ctx.end(), c) != b->ctx.end()) return LMG_OK;
  cudaSetDevice(b->device);
  cudaEvent_t e = nullptr;
  if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess)
    return bfail(b, LMG_ERR_CUDA, "batch_add: event creation failed");
  c->perflog = false;
  b->ctx.push_back(c);
  b->join.push_back(e);
  drop_graphs(b);
  b->warm[0] = b->warm[1] = false;
  return LMG_OK;
}

lmg_status lmg_batch_tune(lmg_batch *b, int32_t precision, int32_t reps) {
  if (!b || (precision != LMG_FP64 && precision != LMG_MIXED)) return bfail(b, LMG_ERR_ARG, "batch_tune: bad argument");
  cudaSetDevice(b->device);
  if (reps <= 0) reps = 3;
  if (b->persistent) {  // the tile (elements per CTA) and CTAs per SM of the one launch, by timing replays
    static const int tiles[] = {8, 16, 32}, ctas[] = {1, 2, 4, 0};
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
      return bfail(b, LMG_ERR_CUDA, "batch_tune: event creation failed");
    float best = 1e30f;
    int bt = b->p_tile, bc = b->p_ctas;
    lmg_status st = LMG_OK;
    for (int tl : tiles)
      for (int k : ctas) {
        b->p_tile = tl;
        b->p_ctas = k;
        if ((st = lmg_batch_assemble(b, precision))) break;
        cudaEventRecord(e0, b->stream);
        for (int r = 0; r < reps && !st; ++r) st = lmg_batch_assemble(b, precision);
        cudaEventRecord(e1, b->stream);
        if (st || cudaEventSynchronize(e1) != cudaSuccess) break;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (ms < best) {
          best = ms;
          bt = tl;
          bc = k;
        }
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    b->p_tile = bt;
    b->p_ctas = bc;
    if (st) return st;
    return lmg_batch_synchronize(b, nullptr);
  }
  lmg_status st = run_all(b, precision);  // lazy plans and buffers before any timing
  if (st) return st;
  static const int cand[] = {2, 4, 8, 16, 32};
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return bfail(b, LMG_ERR_CUDA, "batch_tune: event creation failed");
  // one timed measurement of a context's assembly under its current settings
  auto time_one = [&](lmg_ctx *c, float &ms) -> lmg_status {
    lmg_status s = lmg_assemble(c, precision, nullptr, nullptr, 1);
    if (s) return s;
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < reps && !s; ++r) s = lmg_assemble(c, precision, nullptr, nullptr, 1);
    cudaEventRecord(e1, c->stream);
    if (s) return s;
    if (cudaEventSynchronize(e1) != cudaSuccess) return LMG_ERR_CUDA;
    cudaEventElapsedTime(&ms, e0, e1);
    return LMG_OK;
  };
  static const int tiles[] = {4, 8, 16, 32};
  for (lmg_ctx *c : b->ctx) {
    // CTAs per SM of the element kernels
    float best = 1e30f;
    int best_c = c->ctas_per_sm;
    for (int k : cand) {
      c->ctas_per_sm = k;
      float ms = 0.f;
      if ((st = time_one(c, ms))) break;
      if (ms < best) {
        best = ms;
        best_c = k;
      }
    }
    c->ctas_per_sm = best_c;
    if (st) break;
    // elements per CTA tile of the per-pattern HIERARCHIC kernels
    if (c->hier3) {
      best = 1e30f;
      int best_t = c->h3_tile;
      for (int tl : tiles) {
        float ms = 0.f;
        if ((st = lmg::hier3_set_tile(c, tl)) || (st = time_one(c, ms))) break;
        if (ms < best) {
          best = ms;
          best_t = tl;
        }
      }
      if (!st) st = lmg::hier3_set_tile(c, best_t);
      if (st) break;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return bfail(b, st, "batch_tune: assemble failed");
  drop_graphs(b);
  return LMG_OK;
}

lmg_status lmg_batch_assemble(lmg_batch *b, int32_t precision) {
  if (!b || (precision != LMG_FP64 && precision != LMG_MIXED)) return bfail(b, LMG_ERR_ARG, "batch_assemble: bad argument");
  if (b->ctx.empty()) return bfail(b, LMG_ERR_STATE, "batch_assemble: no contexts");
  cudaSetDevice(b->device);
  if (b->persistent) {
    if (!b->warm[precision == LMG_MIXED ? 1 : 0]) {  // lazy plans and buffers of every member
      const lmg_status st = run_all(b, precision);
      if (st) return st;
      b->warm[precision == LMG_MIXED ? 1 : 0] = true;
    }
    const lmg_status st = prepare_persistent(b, precision);
    if (st) return st;
    if (cudaGraphLaunch(b->ps.exec, b->stream) != cudaSuccess)
      return bfail(b, LMG_ERR_CUDA, "batch_assemble: graph launch failed");
    for (lmg_ctx *c : b->ctx) c->launches += 1;
    return LMG_OK;
  }
  const int p = precision == LMG_MIXED ? 1 : 0;
  if (!b->exec[p]) {
    if (!b->warm[p]) {
      const lmg_status st = run_all(b, precision);
      if (st) return st;
      b->warm[p] = true;
    }
    int64_t l0 = 0, l1 = 0;
    for (lmg_ctx *c : b->ctx) l0 += c->launches;
    if (cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return bfail(b, LMG_ERR_CUDA, "batch_assemble: stream capture failed to start");
    lmg_status st = LMG_OK;
    cudaError_t fe = cudaEventRecord(b->fork, b->stream);
    for (size_t i = 0; i < b->ctx.size() && !st && fe == cudaSuccess; ++i) {
      lmg_ctx *c = b->ctx[i];
      fe = cudaStreamWaitEvent(c->stream, b->fork, 0);   // the context's stream joins the capture
      if (fe != cudaSuccess) break;
      st = lmg_assemble(c, precision, nullptr, nullptr, 1);
      if (st) break;
      fe = cudaEventRecord(b->join[i], c->stream);
      if (fe == cudaSuccess) fe = cudaStreamWaitEvent(b->stream, b->join[i], 0);
    }
    if (fe != cudaSuccess && !st) st = LMG_ERR_CUDA;
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(b->stream, &g);
    if (st || ce != cudaSuccess || !g) {
      if (g) cudaGraphDestroy(g);
      return bfail(b, st ? st : LMG_ERR_CUDA, "batch_assemble: capture failed");
    }
    for (lmg_ctx *c : b->ctx) l1 += c->launches;
    b->launches = l1 - l0;
    b->graph[p] = g;
    if (cudaGraphInstantiate(&b->exec[p], g, 0) != cudaSuccess) {
      drop_graphs(b);
      return bfail(b, LMG_ERR_CUDA, "batch_assemble: graph instantiation failed");
    }
  }
  if (cudaGraphLaunch(b->exec[p], b->stream) != cudaSuccess)
    return bfail(b, LMG_ERR_CUDA, "batch_assemble: graph launch failed");
  for (lmg_ctx *c : b->ctx) c->launches += b->launches / (int64_t)b->ctx.size();
  return LMG_OK;
}

lmg_status lmg_batch_synchronize(lmg_batch *b, int64_t *first_failed) {
  if (!b) return LMG_ERR_ARG;
  if (first_failed) *first_failed = -1;
  cudaSetDevice(b->device);
  if (cudaStreamSynchronize(b->stream) != cudaSuccess) return bfail(b, LMG_ERR_CUDA, "batch: device failure");
  if (b->persistent && b->ps.status) {
    int st = 0;
    if (cudaMemcpy(&st, b->ps.status, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess || st)
      return bfail(b, st ? (lmg_status)st : LMG_ERR_CUDA, "batch: a persistent wait gave up");
  }
  for (size_t i = 0; i < b->ctx.size(); ++i) {
    const lmg_status st = lmg_synchronize(b->ctx[i]);
    if (st) {
      if (first_failed) *first_failed = (int64_t)i;
      return bfail(b, st, "batch: context " + std::to_string(i) + ": " + b->ctx[i]->err);
    }
  }
  return LMG_OK;
}

lmg_status lmg_batch_last_error(lmg_batch *b, char *msg, int32_t cap) {
  if (!b || !msg || cap <= 0) return LMG_ERR_ARG;
  const size_t n = std::min((size_t)(cap - 1), b->err.size());
  std::copy(b->err.begin(), b->err.begin() + n, msg);
  msg[n] = 0;
  return LMG_OK;
}

lmg_status lmg_batch_set_persistent(lmg_batch *b, int32_t on) {
  if (!b) return LMG_ERR_ARG;
  cudaSetDevice(b->device);
  cudaStreamSynchronize(b->stream);
  b->persistent = on != 0;
  b->p_hybrid = on == 2;
  drop_graphs(b);
  b->warm[0] = b->warm[1] = false;
  return LMG_OK;
}

lmg_status lmg_batch_persistent_info(lmg_batch *b, int32_t *tile, int32_t *ctas_per_sm, int64_t *items) {
  if (!b) return LMG_ERR_ARG;
  if (tile) *tile = b->p_tile;
  if (ctas_per_sm) *ctas_per_sm = b->p_ctas;
  if (items) *items = b->ps.n_items;
  return LMG_OK;
}

lmg_status lmg_batch_info(lmg_batch *b, void **stream, int64_t *launches_per_replay, int32_t *ctas_per_sm,
                          int32_t n) {
  if (!b) return LMG_ERR_ARG;
  if (stream) *stream = (void *)b->stream;
  if (launches_per_replay) *launches_per_replay = b->launches;
  if (ctas_per_sm)
    for (int32_t i = 0; i < n && i < (int32_t)b->ctx.size(); ++i) ctas_per_sm[i] = b->ctx[(size_t)i]->ctas_per_sm;
  return LMG_OK;
}

}  // extern "C"
