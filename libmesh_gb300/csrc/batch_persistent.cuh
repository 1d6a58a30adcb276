// Persistent batched assembly: the members and work items of one launch
// (batch_persistent.cu, driven by batch.cu).
#pragma once

#include <cstdint>

#include "pattern.cuh"

namespace lmg {

// One system of the batch in per-pattern form: its element tiles and its
// slot-ordered insertion (the general path's plan).
struct PMember {
  H3Args el;                 // per-pattern tables, tiles, element buffers
  int N, G;                  // dofs and map nodes per element (kernel dispatch)
  int64_t n_tiles;           // element tiles (el.n_batch)
  int64_t nnz, n_dofs;       // CSR slots and dofs
  const int64_t *cptr;       // [nnz+1] contributions of each slot
  const uint32_t *coff;      // element-matrix offsets, element order per slot
  const int64_t *fptr;       // [n_dofs+1]
  const uint32_t *foff;      // element-vector offsets
  double *K, *F;
};

// Work item: an element tile (kind 0) or a range of PB_SLOTS slots / dofs of
// the insertion (kind 1) of a member.
struct PItem {
  int32_t member, kind;
  int64_t local;
};
constexpr int PB_SLOTS = 2048;

// (N, G) pairs the persistent kernel is built for.
bool persistent_kind_built(int N, int G);

void launch_batch_persistent(const PMember *mem, const PItem *items, int64_t n_items, unsigned long long *head,
                             unsigned int *done, int *status, bool mixed, int tile, int grid, cudaStream_t s);
int persistent_ctas_per_sm(bool mixed, int tile);

}  // namespace lmg
