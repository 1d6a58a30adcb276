// Device-side declarations for the assembly kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace lmg {

// Reference-element tables in device memory (one set per context).
struct DevFE {
  int n, q, n_geo;
  const double *qw;     // [q]
  const double *phi;    // [q][n]
  const double *dphi;   // [q][n][3]
  const double *gdphi;  // [q][n_geo][3]
  const double *gphi;   // [q][n_geo] mapping shapes
  const double *S;      // [9][n][n]
  const double *M;      // [n][n]
};

// Everything an element kernel reads or writes.
struct ElemArgs {
  int64_t n_list;             // elements in `list`
  const int32_t *list;        // element ids to process
  int npe;                    // nodes per element (geometry)
  const double *xyz;          // [n_nodes][3]
  const int32_t *conn;        // [n_elem][npe]
  const double *coef;         // [n_elem] or null (=1)
  const double *nodal_f;      // [n_nodes][nv] or null (=0)
  const float2 *nodal_f2;     // the same as double-float pairs, or null
  const uint64_t *cmask;      // [n_elem] constrained local dofs, bit v*n + a
  double nu;                  // Poisson ratio (elasticity)
  // Symmetric element matrices are stored as nv x nv blocks: the n diagonal
  // blocks and the n(n-1)/2 strictly upper blocks (a < b, row-major over a
  // then b).  The FP64 drop-in stores every entry as a double-float pair
  // (hi + lo, 48-bit significand); the mixed form stores only the off-diagonal
  // blocks, in FP32.
  float2 *Kdiag2;             // [n_elem][n][nv][nv]          (FP64 drop-in)
  float2 *Koff2;              // [n_elem][n(n-1)/2][nv][nv]   (FP64 drop-in)
  float *Koff32;              // [n_elem][n(n-1)/2][nv][nv]   (mixed)
  float2 *Fe2;                // [n_elem][n][nv] load vector, double-float pairs
  int *status;                // [0] error code
  unsigned long long *bad_elem;  // first failing element id
  DevFE fe;
  // matrix-free residual (k_residual_affine): element block ids, the vector
  // u [n_dofs] and the per-element residual R_e = K_e u_e - F_e [n_elem][N][nv]
  const int32_t *eb;
  const double *u;
  float2 *Re2;
};

// Fused mixed assembly (element contraction and insertion in one row kernel).
struct FusedArgs {
  ElemArgs el;                // geometry, coefficients, loads, mask, status; list = elements
  float *geo;                 // [n_elem][NG] per-element FP32 operands of the contraction
  int64_t n_brows;            // block rows [row_begin, n_brows) are assembled
  int64_t row_begin;
  const int64_t *brow_ptr;    // [n_brows+1]
  const int32_t *bcol;        // [nnzb]
  const int32_t *row_ptr;     // [n_dofs+1]
  const int32_t *fptr;        // [n_brows+1] incidences of each block row
  const int32_t *fcontrib;    // e*N + a, ascending (element order)
  const uint8_t *relslot;     // [n_elem][N][N] slot of block (a, b) inside block row of a
  const uint8_t *constrained; // [n_dofs]
  const uint8_t *rowcons;     // [n_brows] 1 when the block row or one of its columns holds a constrained dof
  int max_deg;                // largest block-row degree
  double *K;
  double *F;
};

// Scatter plan: gather-by-slot segmented reduction into CSR values.
struct GatherArgs {
  int64_t n_dofs;
  int64_t row_begin, row_end; // block rows to insert (row_end 0 = all)
  int bs;                     // dofs per block (node-interleaved variables)
  int nb;                     // blocks per element
  const int64_t *brow_ptr;    // [n_blocks+1]
  const int32_t *row_ptr;     // [n_dofs+1]
  const int32_t *bcol;        // [nnzb]
  const int32_t *bptr;        // [nnzb+1] contributions per block slot
  const int32_t *bdiag;       // [n_blocks] position of the diagonal slot in each block row (or null)
  // Per slot, ascending in element: diagonal slots hold e*nb + a (a Kdiag
  // block); off-diagonal slots hold 2*(e*no + o) + t, o the strictly upper
  // block of the element pair and t = 1 when the slot takes its transpose.
  const int32_t *bcontrib;
  int no;                     // strictly upper blocks per element
  const int32_t *fptr;        // [n_blocks+1]
  const int32_t *fcontrib;    // e*nb + a, ascending per block row
  const float2 *Kdiag2;
  const float2 *Koff2;
  const float *Koff32;
  const float2 *Fe2;
  const uint8_t *constrained; // [n_dofs] (mixed form applies the Dirichlet rows here)
  double *K;
  double *F;
};

// Adjoint sensitivity and QoI load arguments.
struct VjpArgs {
  int64_t n_elem;
  const double *xyz;
  const int32_t *conn;        // [n_elem][n]
  const int32_t *eb;          // [n_elem][n] block (node) of each local node
  const double *u, *z;        // [n_dofs] primal and adjoint solutions
  const uint8_t *region;      // [n_elem] QoI element set
  const uint64_t *cmask;      // [n_elem] constrained local dofs (their QoI load is zero)
  double nu;
  double *out;                // [n_elem] dq/dp_e
  const double *coef;         // [n_elem] or null (=1): element coefficients (coordinate sensitivities)
  const double *nodal_f;      // [n_nodes][nv] or null: nodal load (coordinate sensitivities)
  double *xout;               // [n_elem][n][3] d q / d X of each element's nodes
  int64_t n_rows;             // rows of the per-dof gather
  const int32_t *fptr;        // [n_rows+1] incidences (e*n + a) of each dof row
  const int32_t *fcontrib;
  double *row_out;            // [n_rows][3]
  float2 *Fe2;                // [n_elem][n][nv] load of the QoI set
  int *status;
  unsigned long long *bad_elem;
  DevFE fe;
};
bool launch_vjp(int form, int n, int nv, bool region, const VjpArgs &v, int grid, cudaStream_t s);
// Coordinate sensitivities (Poisson and elasticity): element pass then per-node gather.
bool launch_vjp_xyz(int form, int n, const VjpArgs &v, int grid, cudaStream_t s);
void launch_gather_f(const GatherArgs &g, cudaStream_t s);

// Whether an element kernel is instantiated for (form, shapes per variable, variables).
bool fused_built(int form, int n, int nv);
// Whether the fused row kernel's shared-memory rows fit for rows of max_deg slots.
bool fused_fits(int n, int nv, int max_deg);
// k_geo (when geo) then k_rows_mixed over f's rows (when rows); false if no kernel is built.
bool launch_fused_mixed(int form, int n, int nv, const FusedArgs &f, int grid, cudaStream_t s, bool geo = true,
                        bool rows = true);
bool elements_built(int form, int n, int nv);
// R = K u - F without K (affine elements): residual kernel, then the per-dof
// sums over the load-vector plan; false when no kernel is built for the form.
bool launch_residual(int form, int n, int nv, const ElemArgs &a, int64_t n_brows, const int32_t *fptr,
                     const int32_t *fcontrib, double *R, int grid, cudaStream_t s);
void launch_elements(int form, int n, int nv, bool affine, bool mixed, const ElemArgs &a, int grid,
                     cudaStream_t s);
// Mixed-form element matrices of any (affine or not) elements as per-point
// Gram products E^T E on the tensor cores (tc.cu): built for (form, shapes per
// variable, variables, quadrature points) when tc_built says so; writes the
// strictly upper blocks to Koff32 and the FP64 path's load vector to Fe2.
bool tc_built(int form, int n, int nv, int q);
// neg_weights: the rule's first point has a negative weight (Keast's 11-point
// rule); a rule with a negative weight elsewhere is not built
bool launch_elements_tc(int form, int n, int nv, int q, bool neg_weights, const ElemArgs &a, int n_sm,
                        cudaStream_t s);
bool gather_built(int bs);
// PCG (Jacobi) on a CSR matrix; returns 0 on success, 7 out of memory, 2 CUDA error.
int cg_solve(int64_t n, const int32_t *rp, const int32_t *col, const double *val, const double *b, double *x,
             double rtol, int maxit, cudaStream_t s, int n_sm, int *iters, double *relres, int64_t *launches);
void launch_gather(const GatherArgs &g, bool mixed, cudaStream_t s);
// The load vector of block rows [r0, r1): per dof the element entries in
// element order (thread per block row; every insertion's F).
void launch_load_vec(int bs, int64_t r0, int64_t r1, const int32_t *fptr, const int32_t *fcontrib,
                     const float2 *Fe2, double *F, cudaStream_t s);

}  // namespace lmg
