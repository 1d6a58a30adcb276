// Declarations of the general scalar assembly path (general.cu).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "assemble.cuh"

namespace lmg {

constexpr int GEN_MAX_N = 27;          // dofs per element
constexpr int GEN_MAX_NE = 128;        // dofs of a constrained element incl. constraining dofs
constexpr int GEN_MAX_ENTRIES = 2048;  // nonzeros of one element's constraint matrix
constexpr int GEN_MAX_MODES = 64;      // transport-velocity modes

struct GenElemArgs {
  int64_t n_elem;
  const double *xyz;          // [n_nodes][3]
  const int32_t *conn;        // [n_elem][N]
  const double *coef;         // [n_elem] or null (=1)
  const double *nodal_f;      // [n_nodes] or null (=0)
  const double *D6;           // [6][N][N]: S00, S11, S22, S01+S10, S02+S20, S12+S21
  double kappa;               // convection-diffusion diffusivity
  int n_modes;
  const double *modes;        // [n_modes][7]: a[3], k[3], phase
  void *Kraw;                 // [n_elem][N][N] element matrices: double (FP64 drop-in) or float (mixed)
  double *Fraw;               // [n_elem][N]
  int *status;
  unsigned long long *bad_elem;
  DevFE fe;
};

// Constrained elements: column lists of each element's constraint matrix.
struct ConsArgs {
  int64_t n_cons;
  int N;
  int max_ne;                 // largest ne over the constrained elements
  int max_ent;                // largest entry count over the constrained elements
  const int32_t *elem;        // [n_cons] element id
  const int32_t *ne;          // [n_cons] dofs after enlargement
  const int64_t *kout;        // [n_cons] offset of the ne x ne result in Ebuf
  const int64_t *fout;        // [n_cons] offset of the ne result in Fbuf
  const int64_t *cbase;       // [n_cons] start of the element's ne+1 column pointers in ccp
  const int32_t *ccp;         // column pointers, relative to the element's entries
  const int64_t *ebase;       // [n_cons] start of the element's entries in ci / cv
  const uint8_t *ci;          // row index of each entry
  const double *cv;           // coefficient of each entry
  const uint64_t *rowmask;    // [n_cons] constrained local rows
  const void *Kraw;           // element matrices, double or float
  const double *Fraw;
  void *Ebuf;                 // enlarged element matrices, same type
  double *Fbuf;
};

bool gen_elements_built(int form, int n, int q);
// mixed: FP32 element contraction (the map stays FP64); max_ctas: grid cap of
// the grid-stride element loop
void launch_gen_elements(int form, int n, int q, bool mixed, const GenElemArgs &a, int max_ctas, cudaStream_t s);
void launch_constrain(const ConsArgs &c, bool mixed, int n_sm, cudaStream_t s);
// slot gather (FP64 sums) over element matrices stored as double, or float when mixed
// over the slots [s0, s1) and the dofs [d0, d1)
void launch_gather_full(int64_t nnz, const int64_t *cptr, const uint32_t *coff, const void *E, bool mixed, double *K,
                        int64_t n_dofs, const int64_t *fptr, const uint32_t *foff, const double *Fb, double *F,
                        int n_sm, cudaStream_t s, int64_t s0, int64_t s1, int64_t d0, int64_t d1);

}  // namespace lmg
