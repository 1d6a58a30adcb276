/*
 * libmesh_gb300 — GB300-native finite-element assembly behind a C ABI.
 *
 * This header is the whole drop-in boundary.  It replaces libMesh's per-element
 * assembly loop (the user callback run by System::assemble) with one device
 * pass over the mesh, and it mirrors the host-side libMesh setup that feeds
 * that loop (mesh generation, DofMap numbering, Dirichlet constraint sets,
 * sparsity).  Plain C types only: pointers, sizes, int status codes.
 * Nothing here throws; every call returns an lmg_status.
 *
 * Reference interfaces replaced (paths inside the libMesh source tree):
 *   System::assemble / attach_assemble_function / attach_assemble_object
 *       src/systems/system.C:554-561, 1959-1986; include/systems/system.h:157-171
 *   FEBase::reinit + get_phi/get_dphi/get_JxW over QGauss
 *       src/fe/fe.C:197-368; src/fe/fe_base.C:762-793; src/fe/fe_map.C:1167-1374
 *   DofMap::distribute_dofs / dof_indices
 *       src/base/dof_map.C:949-1116, 1417-1537, 2201-2314; include/base/dof_map.h:2619-2760
 *   DofMap::compute_sparsity (SparsityPattern::Build)
 *       src/base/dof_map.C:1960-1977; src/base/sparsity_pattern.C:96-363
 *   DofMap::(heterogenously_)constrain_element_matrix_and_vector
 *       src/base/dof_map_constraints.C:2439-2616, 3433-3540
 *   SparseMatrix::add_matrix / NumericVector::add_vector (PETSc AIJ layout)
 *       src/numerics/petsc_matrix.C:735-755; src/numerics/petsc_vector.C:174-195
 *   MeshTools::Generation::build_cube, MeshTools::Modification::all_tri,
 *   MeshBase::all_second_order, ReplicatedMesh::renumber_nodes_and_elements
 *       src/mesh/mesh_generation.C:317-1937; src/mesh/mesh_modification.C:449-1180;
 *       src/mesh/unstructured_mesh.C:60-640; src/mesh/replicated_mesh.C:700-860
 */
#ifndef LIBMESH_GB300_H
#define LIBMESH_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t lmg_status;

/* Status codes.  libMesh raises C++ exceptions for the same conditions
 * (libmesh_error_msg, DegenerateMap: include/base/libmesh_exceptions.h:65-207). */
enum {
  LMG_OK = 0,
  LMG_ERR_ARG = 1,          /* bad argument (null pointer, size, unknown enum)          */
  LMG_ERR_CUDA = 2,         /* a CUDA runtime call failed                               */
  LMG_ERR_STATE = 3,        /* call order violated (e.g. assemble before sparsity)     */
  LMG_ERR_DEGENERATE = 4,   /* detJ <= 0 at a quadrature point (fe_map.C:466-500)       */
  LMG_ERR_BOUNDS = 5,       /* connectivity or dof index outside its range              */
  LMG_ERR_NEW_NONZERO = 6,  /* element couples a pair not in the sparsity (petsc_matrix.C:330-336) */
  LMG_ERR_OOM = 7,          /* device or host allocation failed                         */
  LMG_ERR_UNSUPPORTED = 8   /* element type / order / form combination not built       */
};

/* Element types: the numeric values of libMesh's ElemType (include/enums/enum_elem_type.h). */
enum {
  LMG_TET4 = 8, LMG_TET10 = 9, LMG_HEX8 = 10, LMG_HEX27 = 12, LMG_PRISM6 = 13, LMG_PRISM18 = 15,
  LMG_TET14 = 34, LMG_PRISM21 = 36
};

/* Weak forms registered with the element kernels (examples the forms follow):
 *   LMG_POISSON    Ke += k_e JxW dphi_i.dphi_j, Fe += JxW f phi_i
 *                  (examples/introduction/introduction_ex4/introduction_ex4.C:467,536)
 *   LMG_ELASTICITY Ke_var[i][k] += JxW C_ijkl(E_e, nu) dphi_b(l) dphi_a(j), Fe_var[i] += JxW f_i phi_a
 *                  (examples/systems_of_equations/systems_of_equations_ex6/systems_of_equations_ex6.C:136-230)
 *   LMG_ADVDIFF    Ke += JxW [(b . dphi_j) phi_i + kappa k_e dphi_i.dphi_j], Fe += JxW f phi_i, the
 *                  steady Galerkin convection-diffusion of examples/adaptivity/adaptivity_ex2/adaptivity_ex2.C:660-690
 *                  with b = curl of psi = sum_m a_m sin(k_m . x + phase_m) */
enum { LMG_POISSON = 0, LMG_ELASTICITY = 1, LMG_ADVDIFF = 2 };

/* Arithmetic of the element contraction.  LMG_FP64 is the drop-in (matches
 * libMesh to 1e-13 per entry).  LMG_MIXED keeps Jacobians, the global
 * accumulation and the outputs in FP64 and contracts in FP32. */
enum { LMG_FP64 = 0, LMG_MIXED = 1 };

/* ------------------------------------------------------------------------- */
/* Host mirror of libMesh's setup: mesh generation and DofMap.               */
/* ------------------------------------------------------------------------- */

typedef struct lmg_mesh lmg_mesh;

/* MeshTools::Generation::build_cube(nx,ny,nz, 0..1 x3, type) followed by
 * prepare_for_use (first-touch node renumbering), src/mesh/mesh_generation.C:317-1937.
 * elem_type LMG_HEX8 or LMG_HEX27 gives the hex mesh; LMG_TET4 / LMG_TET10 gives
 * build_cube(HEX8) -> jitter -> MeshTools::Modification::all_tri (6 tets per hex,
 * src/mesh/mesh_modification.C:449-1180) [-> all_second_order for TET10,
 * -> all_complete_order for TET14: edge nodes and face nodes at the face
 * centroids, src/mesh/unstructured_mesh.C:60-170, 1800-1860].
 * jitter > 0 moves every interior vertex of the HEX8 grid by an independent
 * uniform offset in [-jitter*h, +jitter*h] per coordinate, drawn from a
 * splitmix64 stream seeded with `seed`, before the tet split (so TET10 / TET14
 * edge and face nodes sit at midpoints and centroids and every tet stays affine). */
lmg_status lmg_mesh_cube(int32_t nx, int32_t ny, int32_t nz, int32_t elem_type,
                         double jitter, uint64_t seed, lmg_mesh **out);
lmg_status lmg_mesh_info(const lmg_mesh *m, int64_t *n_nodes, int64_t *n_elem,
                         int32_t *elem_type, int32_t *nodes_per_elem, int32_t *sides_per_elem);
/* xyz [n_nodes][3]; conn [n_elem][nodes_per_elem] (libMesh local node order);
 * side_bid [n_elem][sides_per_elem] boundary id of each side or -1. Any may be NULL. */
lmg_status lmg_mesh_copy(const lmg_mesh *m, double *xyz, int32_t *conn, int8_t *side_bid);
lmg_status lmg_mesh_free(lmg_mesh *m);

/* DofMap::distribute_dofs (var-major, first touch over active elements,
 * src/base/dof_map.C:1417-1537) for n_vars LAGRANGE variables of one
 * VariableGroup with one dof per node, then DofMap::dof_indices for every
 * element (include/base/dof_map.h:2619-2760): elem_dofs[e][v*npe + a].
 * elem_dofs has n_elem * n_vars * npe entries. */
lmg_status lmg_dofmap_distribute(int64_t n_nodes, int64_t n_elem, int32_t npe,
                                 const int32_t *conn, int32_t n_vars,
                                 int64_t *n_dofs, int32_t *elem_dofs);

/* Dof set constrained by a homogeneous DirichletBoundary on the sides whose
 * boundary id is in bids[0..n_bids) for the variables vars[0..n_vars_bc)
 * (ConstrainDirichlet, src/base/dof_map_constraints.C:257-1560: for LAGRANGE
 * every dof of every node on a matching side).  constrained[n_dofs] gets 0/1. */
lmg_status lmg_dirichlet_dofs(int64_t n_elem, int32_t elem_type, int32_t n_vars,
                              const int32_t *elem_dofs, const int8_t *side_bid,
                              const int32_t *bids, int32_t n_bids,
                              const int32_t *vars, int32_t n_vars_bc,
                              int64_t n_dofs, uint8_t *constrained);

/* Dofs per element of FEType fe_order (| LMG_HIERARCHIC) on elem_type for
 * n_vars variables: n_vars * nodes for the nodal cases, 64 for
 * FEType{THIRD, HIERARCHIC} on HEX27 and 20 on TET14 (HIERARCHIC_n_dofs,
 * src/fe/fe_hierarchic.C:94-141, 440-470). */
lmg_status lmg_fe_dofs_per_elem(int32_t elem_type, int32_t fe_order, int32_t n_vars, int32_t *n);

/* DofMap::distribute_dofs + dof_indices for an FEType: the nodal cases as
 * lmg_dofmap_distribute; FEType{THIRD, HIERARCHIC} on HEX27 (one variable)
 * with HIERARCHIC_n_dofs_at_node's per-node counts (vertex 1, edge node 2,
 * face node 4, centre 0) and 8 element-interior dofs, or on TET14 (vertex 1,
 * edge node 2, face node 1, no interior dofs), numbered per element
 * nodes-then-element (src/base/dof_map.C:1417-1537), non-vertex node dofs
 * listed last to first (include/base/dof_map.h:2685-2712).
 * elem_dofs [n_elem][lmg_fe_dofs_per_elem]. */
lmg_status lmg_dofmap_distribute_fe(int64_t n_nodes, int64_t n_elem, int32_t elem_type, const int32_t *conn,
                                    int32_t n_vars, int32_t fe_order, int64_t *n_dofs, int32_t *elem_dofs);

/* The same numbering and dof_indices formed on `device`: the sequential sweep
 * of distribute_local_dofs_var_major as an exclusive scan (each node's first
 * touch, the smallest element position holding it, carries its dof count;
 * each element's interior dofs follow its nodes).  Host arrays in and out,
 * bit for bit the lists of lmg_dofmap_distribute_fe; the call synchronizes
 * the device and allocates device memory for its duration. */
lmg_status lmg_dofmap_distribute_device(int32_t device, int64_t n_nodes, int64_t n_elem, int32_t elem_type,
                                        const int32_t *conn, int32_t n_vars, int32_t fe_order, int64_t *n_dofs,
                                        int32_t *elem_dofs);

/* lmg_dirichlet_dofs for an FEType: for FEType{THIRD, HIERARCHIC} every dof
 * of every node of a matching side (vertex, edge and face dofs). */
lmg_status lmg_dirichlet_dofs_fe(int64_t n_elem, int32_t elem_type, int32_t fe_order, int32_t n_vars,
                                 const int32_t *elem_dofs, const int8_t *side_bid, const int32_t *bids,
                                 int32_t n_bids, const int32_t *vars, int32_t n_vars_bc, int64_t n_dofs,
                                 uint8_t *constrained);

/* DofMap::compute_sparsity on the host (the same pattern lmg_sparsity_build
 * puts on the device): PETSc-AIJ CSR with sorted columns, full coupling of the
 * dofs of each element.  Call with row_ptr = col_idx = NULL to get nnz. */
lmg_status lmg_host_sparsity(int64_t n_elem, int32_t npe, int32_t n_vars, int64_t n_dofs,
                             const int32_t *elem_dofs, int64_t *nnz, int32_t *row_ptr,
                             int32_t *col_idx);

/* h-refinement of an unjittered HEX8 / HEX27 build_cube mesh
 * (MeshRefinement::refine_and_coarsen_elements, src/mesh/mesh_refinement.C:482-786;
 * Elem::refine, src/geom/elem_refinement.C:87-150): `cycles` rounds, each
 * flagging floor(fraction * n_active) distinct active elements drawn from a
 * splitmix64 stream seeded with `seed`, then flagging every coarser face
 * neighbor of a flagged element until the level-one rule holds, then refining
 * (children appended in parent id order, new nodes by the embedding matrices,
 * nodes renumbered first-touch over all elements as
 * ReplicatedMesh::renumber_nodes_and_elements does).  Afterwards the mesh
 * holds the active elements in id order (lmg_mesh_info / lmg_mesh_copy). */
lmg_status lmg_mesh_refine(lmg_mesh *m, int32_t cycles, double fraction, uint64_t seed);
/* The refinement tree: every element ever created (all_conn [n_all][npe],
 * parent id or -1, level) and the ids of the active elements (active_ids
 * [n_elem], the rows of lmg_mesh_copy's conn).  NULL arrays are skipped. */
lmg_status lmg_mesh_tree(const lmg_mesh *m, int64_t *n_all, int32_t *all_conn, int32_t *parent,
                         int8_t *level, int32_t *active_ids);

/* DofMap::create_dof_constraints + process_constraints for LAGRANGE variables
 * on the active mesh (src/base/dof_map_constraints.C:1736-1895, 4341-4490):
 * hanging-node rows (lagrange_compute_constraints, src/fe/fe_lagrange.C:867-1063:
 * coefficient = parent-side shape at the hanging node, kept when
 * 1e-5 < |c| < 0.999), then empty rows for the dofs flagged in dirichlet[n_dofs]
 * that are still free (AddPrimalConstraint), then chains substituted until
 * every row refers to free dofs.  Output: constrained[n_dofs] 0/1 and the rows
 * as CSR over all dofs: cons_ptr[n_dofs+1], cons_col / cons_val ascending per
 * row.  Call with cons_col = cons_val = NULL to get cons_ptr only (the size is
 * cons_ptr[n_dofs]); cap is the capacity of cons_col / cons_val. */
lmg_status lmg_constraint_rows(const lmg_mesh *m, int32_t n_vars, const int32_t *elem_dofs,
                               int64_t n_dofs, const uint8_t *dirichlet, uint8_t *constrained,
                               int64_t *cons_ptr, int32_t *cons_col, double *cons_val, int64_t cap);

/* The same rows with the hanging-node rows formed on `device`
 * (lagrange_compute_constraints, src/fe/fe_lagrange.C:867-1063, one thread
 * per (variable, active element, side), the first visit of a dof in
 * libMesh's loop order writing its row); the Dirichlet rows and
 * process_constraints (dof_map_constraints.C:4341-4490) follow on the host.
 * Same arguments and outputs as lmg_constraint_rows, bit for bit; the call
 * synchronizes the device and allocates device memory for its duration. */
lmg_status lmg_constraint_rows_device(const lmg_mesh *m, int32_t device, int32_t n_vars,
                                      const int32_t *elem_dofs, int64_t n_dofs, const uint8_t *dirichlet,
                                      uint8_t *constrained, int64_t *cons_ptr, int32_t *cons_col,
                                      double *cons_val, int64_t cap);

/* DofMap::compute_sparsity with constraints (find_connected_dofs,
 * src/base/dof_map.C:2915-2970): every element couples the union of its dofs
 * and of the dofs that constrain them.  elem_dofs [n_elem][dofs_per_elem]. */
lmg_status lmg_host_sparsity_constrained(int64_t n_elem, int32_t dofs_per_elem, int64_t n_dofs,
                                         const int32_t *elem_dofs, const int64_t *cons_ptr,
                                         const int32_t *cons_col, int64_t *nnz, int32_t *row_ptr,
                                         int32_t *col_idx);

/* ------------------------------------------------------------------------- */
/* Device context: the assembly drop-in.                                     */
/* ------------------------------------------------------------------------- */

typedef struct lmg_ctx lmg_ctx;

lmg_status lmg_context_create(lmg_ctx **ctx, int32_t device);
lmg_status lmg_context_destroy(lmg_ctx *ctx);
/* Run every kernel and copy of this context on `stream` (a cudaStream_t). */
lmg_status lmg_context_set_stream(lmg_ctx *ctx, void *stream);

/* Geometry: xyz [n_nodes][3], conn [n_elem][npe] in libMesh node order.
 * Uniform element type per context.  The host arrays may be freed on return. */
lmg_status lmg_mesh_upload(lmg_ctx *ctx, int64_t n_nodes, const double *xyz,
                           int64_t n_elem, int32_t elem_type, const int32_t *conn);

/* Exact DofMap::dof_indices output: elem_dofs[e][v*npe + a] for n_vars variables. */
lmg_status lmg_dofmap_upload(lmg_ctx *ctx, int32_t n_vars, int64_t n_dofs,
                             const int32_t *elem_dofs);

/* dof_indices output for an FEType whose dofs are not one per node and
 * variable: elem_dofs[e][0 .. lmg_fe_dofs_per_elem) as
 * lmg_dofmap_distribute_fe lists them.  FEType{THIRD, HIERARCHIC} on HEX27 or
 * TET14 (one variable, affine elements, POISSON, LMG_FP64) assembles on the
 * general path: full element matrices per orientation pattern, constraint
 * product, slot gather. */
lmg_status lmg_dofmap_upload_fe(lmg_ctx *ctx, int32_t n_vars, int32_t fe_order, int64_t n_dofs,
                                const int32_t *elem_dofs);

/* Constrained dofs with empty constraint rows and zero values (homogeneous
 * Dirichlet), as DofMap::_dof_constraints holds them. constrained[n_dofs]. */
lmg_status lmg_constraints_upload(lmg_ctx *ctx, const uint8_t *constrained);

/* Constraint rows with coefficients (hanging nodes; DofMap::_dof_constraints
 * after process_constraints, e.g. from lmg_constraint_rows): constrained[n_dofs]
 * and the rows as CSR over all dofs, cons_ptr[n_dofs+1], cons_col / cons_val
 * ascending per row, empty rows for Dirichlet dofs; every row must refer to
 * free dofs only.  The assembly then applies constrain_element_matrix_and_vector
 * in full (C^T K C on the element's dofs plus its constraining dofs,
 * asymmetric constraint rows; src/base/dof_map_constraints.C:2439-2515,
 * 3433-3540) and lmg_sparsity_build adds the constraint couplings
 * (find_connected_dofs).  That path takes one variable, affine elements and
 * LMG_FP64; lmg_constraints_upload drops the rows again. */
lmg_status lmg_constraint_rows_upload(lmg_ctx *ctx, const uint8_t *constrained, const int64_t *cons_ptr,
                                      const int32_t *cons_col, const double *cons_val);

/* DofMap::compute_sparsity: PETSc-AIJ CSR (sorted column indices per row).
 * Built on the device: the block path's block graph, and with constraint
 * rows the enlarged element lists of find_connected_dofs and their union per
 * row; the host builds a pattern whose rows outgrow the device buffers. */
lmg_status lmg_sparsity_build(lmg_ctx *ctx, int64_t *nnz);
/* 1 when the last lmg_sparsity_build formed the pattern on the device, else 0. */
lmg_status lmg_sparsity_on_device(lmg_ctx *ctx, int32_t *on_device);
lmg_status lmg_sparsity_copy(lmg_ctx *ctx, int32_t *row_ptr, int32_t *col_idx);
/* The general path's insertion plan (each element's constraint matrix of
 * DofMap::build_constraint_matrix, dof_map_constraints.C:3433-3540, and the
 * CSR slots' element-order contributions of PetscMatrix::add_matrix,
 * petsc_matrix.C:735-755): built on the device with on = 1 (the default) and
 * on the host with on = 0; both give the same arrays bit for bit.  The host
 * build also takes over where an element's list or constraint matrix
 * outgrows the device buffers.  Takes effect at the next plan build. */
lmg_status lmg_context_set_plan_on_device(lmg_ctx *ctx, int32_t on);
/* 1 when the last general-path plan was built on the device, else 0. */
lmg_status lmg_plan_on_device(lmg_ctx *ctx, int32_t *on_device);

/* FE family flag OR'ed into fe_order (libMesh FEType{order, family}):
 * LMG_HIERARCHIC selects HIERARCHIC (FIRST on HEX8 / TET4 / PRISM6, SECOND on
 * HEX27 / TET10, THIRD on HEX27 and TET14; shapes of src/fe/fe_hierarchic_shape_3D.C
 * with cube_indices' edge and face orientation on hexes and the edge flips and
 * orient_triangle face order on tets, derivatives by central differences
 * as FE<3,HIERARCHIC>::shape_deriv takes them).  Without it the family is LAGRANGE. */
enum { LMG_HIERARCHIC = 0x100 };

/* Weak form and its data.  fe_order: 1 FIRST / 2 SECOND LAGRANGE (| LMG_HIERARCHIC).
 * q_order: QGauss order (libMesh Order value).  params: POISSON none;
 * ELASTICITY {nu}; ADVDIFF {kappa, n_modes, then per mode a[3], k[3], phase}
 * (one variable, affine elements, LMG_FP64).  elem_coef[n_elem]: k_e (POISSON) or E_e (ELASTICITY),
 * NULL = 1.  nodal_f[n_nodes][n_vars]: load interpolated with phi, NULL = 0. */
lmg_status lmg_form_set(lmg_ctx *ctx, int32_t form, int32_t fe_order, int32_t q_order,
                        const double *params, int32_t n_params,
                        const double *elem_coef, const double *nodal_f);

/* Refresh the per-step inputs from host memory (any may be NULL = unchanged). */
lmg_status lmg_inputs_update(lmg_ctx *ctx, const double *xyz, const double *elem_coef,
                             const double *nodal_f);

/* Assemble K (CSR values, nnz) and F (n_dofs) from zero.  K and F may be host
 * or device pointers (out_on_device = 0 / 1); NULL keeps the result only in the
 * context's own device buffers (see lmg_result_device). */
lmg_status lmg_assemble(lmg_ctx *ctx, int32_t precision, double *K, double *F,
                        int32_t out_on_device);
lmg_status lmg_result_device(lmg_ctx *ctx, double **K, double **F);
/* Copy the last assembled K and F from the context's device buffers to host
 * arrays (either may be NULL), waiting for the context's stream. */
lmg_status lmg_result_copy(lmg_ctx *ctx, double *K, double *F);

/* With device (or no) outputs lmg_assemble returns once the work is queued on
 * the context's stream; lmg_synchronize waits for it and returns its status. */
lmg_status lmg_synchronize(lmg_ctx *ctx);

/* Jacobi-preconditioned CG on the last assembled K (LinearImplicitSystem::solve
 * with KSPCG, src/systems/linear_implicit_system.C:122-165): solves K x = rhs
 * (host array; NULL = the last assembled F) until ||r|| <= rtol ||rhs|| or maxit
 * iterations; x is a host array of n_dofs.  A right-hand side holding NaN or
 * Inf returns LMG_ERR_ARG without iterating. */
lmg_status lmg_cg_solve(lmg_ctx *ctx, const double *rhs, double *x, double rtol, int32_t maxit,
                        int32_t *iters, double *relres);

/* lmg_cg_solve_noalloc — no counterpart in libMesh.  The solve of lmg_cg_solve
 * for callers that cannot allocate device memory: a solver plug-in run from
 * inside another library's solve (a PETSc shell preconditioner, say) whose
 * device memory that library owns and pools, or a service that fixes its
 * device footprint at start-up.  cudaMalloc and cudaFree also synchronize the
 * whole device and stall the caller's other streams.  lmg_cg_solve allocates
 * its work vectors on every call; this variant allocates nothing (no cudaMalloc,
 * no cudaFree, no allocating library routine).  It runs the same kernels in the
 * same reduction order, so it returns the same iterates, on caller-owned device
 * arrays: row_ptr[n_dofs + 1], col_idx, val (the CSR of lmg_sparsity_copy /
 * lmg_assemble), rhs[n_dofs], x[n_dofs] (output).  Its work vectors live in one
 * fixed device array inside the library, 5 x LMG_CG_NOALLOC_MAX_DOFS doubles
 * (20 MiB); n_dofs above LMG_CG_NOALLOC_MAX_DOFS returns LMG_ERR_ARG and says
 * so in msg.  The first call on each device does the set-up: it looks up that
 * array's address on the current device (cudaGetSymbolAddress), and looks it up
 * again whenever the current driver context is a new one (after
 * cudaDeviceReset, say).  Every call on a device shares the one array, so calls whose
 * work overlaps on the GPU (other streams, other host threads) race and give
 * wrong results: serialize them.  The scalar slots are cleared at the start of
 * every call; every other word is written before it is read.  stream is a
 * cudaStream_t (NULL = the legacy default stream); each call synchronizes that
 * stream and reads the residual back to the host while it iterates, and
 * returns once the solve has finished on it.  A right-hand side holding NaN or
 * Inf returns LMG_ERR_ARG, as lmg_cg_solve does.  msg (may be NULL) receives
 * the error text. */
#define LMG_CG_NOALLOC_MAX_DOFS 524288
lmg_status lmg_cg_solve_noalloc(int64_t n_dofs, const int32_t *row_ptr, const int32_t *col_idx,
                                const double *val, const double *rhs, double *x, double rtol,
                                int32_t maxit, void *stream, int32_t *iters, double *relres,
                                char *msg, int32_t msg_len);

/* R = K u - F for the current form and inputs without forming K: what
 * LinearImplicitSystem::assembly computes as the residual (R = A u - b,
 * src/systems/linear_implicit_system.C:367-381) on the assembled,
 * constrained system (a Dirichlet row gives (elements touching the dof) * u_i).
 * Affine elements of the block path (POISSON, ELASTICITY), FP64 arithmetic as
 * the drop-in's (double-float contraction).  u, R [n_dofs] are host arrays, or
 * device arrays when on_device = 1 (then the call returns asynchronously). */
lmg_status lmg_residual(lmg_ctx *ctx, const double *u, double *R, int32_t on_device);

/* Adjoint sensitivities (ImplicitSystem::adjoint_qoi_parameter_sensitivity,
 * src/systems/implicit_system.C:517-623, with the element coefficients of the
 * form as parameters; ParameterVector, src/systems/parameter_vector.C:28-132).
 * lmg_qoi_region_load: q[n_dofs] = derivative of the QoI "integral of the
 * solution over the marked elements" (in_region[n_elem] 0/1), the right-hand
 * side of the adjoint solve K^T z = q (lmg_cg_solve with rhs = q; K is
 * symmetric).  lmg_vjp_coef: dq/dcoef_e = -z_e^T (dK_e/dcoef_e) u_e for every
 * element, exact (K is linear in each coefficient and F does not depend on it),
 * geometry recomputed per quadrature point.  u, z, q, dq_dcoef are host arrays. */
lmg_status lmg_qoi_region_load(lmg_ctx *ctx, const uint8_t *in_region, double *q);
lmg_status lmg_vjp_coef(lmg_ctx *ctx, const double *u, const double *z, double *dq_dcoef);
/* Node-coordinate sensitivities of the same QoI (Poisson and elasticity forms;
 * for elasticity the QoI integrates the sum of u's components, as
 * lmg_qoi_region_load's vector does; the reference's ParameterVector over node
 * coordinates): dq/dx = dq/dx|_u - z^T d(K u - F)/dx
 * for every node, by reverse mode through detJ and J^{-1} at every quadrature
 * point.  in_region[n_elem] marks the QoI elements (NULL: no explicit term);
 * dq_dxyz [n_nodes][3]; all arrays on the host. */
lmg_status lmg_vjp_xyz(lmg_ctx *ctx, const double *u, const double *z, const uint8_t *in_region,
                       double *dq_dxyz);

/* First failing element of the last call (-1 if none) and a message. */
lmg_status lmg_last_error(lmg_ctx *ctx, int64_t *elem_id, char *msg, int32_t msg_len);

/* PerfLog-style stage timing (the reference's PerfLog scopes "assemble()" /
 * "matrix insertion", include/utils/perf_log.h:153-280): when enabled, every
 * lmg_assemble records CUDA events around its element kernels and its global
 * insertion; lmg_perflog_read waits for the stream, returns the summed times
 * and the number of logged calls, and resets the totals. */
lmg_status lmg_perflog_enable(lmg_ctx *ctx, int32_t on);
lmg_status lmg_perflog_read(lmg_ctx *ctx, double *elements_ms, double *gather_ms, int64_t *calls);

/* Mixed form on non-affine elements (the reference's per-point form, where
 * the affine reference-tensor shortcut does not apply): with on = 1 (the
 * default) the per-point products sum_q JxW B_q^T D B_q run as Gram products
 * E^T E on the tensor cores (tcgen05, BF16 three-way split, FP32 accumulation;
 * TET4 / TET10 elasticity, TET10 / HEX8 Poisson), with on = 0 on the CUDA
 * cores in FP32.  Same weak form (systems_of_equations_ex6.C:222-230,
 * introduction_ex4.C:467); the FP64 drop-in is unaffected. */
lmg_status lmg_context_set_tensor_cores(lmg_ctx *ctx, int32_t on);

/* Element-kernel grid of this context in CTAs per SM (0 = default 32); the
 * batch autotuner sets it. */
lmg_status lmg_context_set_grid(lmg_ctx *ctx, int32_t ctas_per_sm);

/* ------------------------------------------------------------------------- */
/* Batched assembly of many systems as one CUDA graph.                       */
/* ------------------------------------------------------------------------- */
/* libMesh assembles each System with its own System::assemble call
 * (src/systems/system.C:554-561).  A batch holds any number of set-up contexts
 * (each its own mesh, element type, form and FE family):
 * lmg_batch_add registers a context (its sparsity and form must be set; it
 * keeps its own stream); lmg_batch_tune times each context's element kernel at
 * {2, 4, 8, 16, 32} CTAs per SM (reps assemblies each) and keeps the fastest;
 * lmg_batch_assemble assembles every context into its own device K and F
 * (lmg_result_device): the first call per precision runs each context once
 * eagerly, then captures all of them into one CUDA graph (one branch per
 * context, forked from and joined into the batch stream), and every call
 * launches that graph on the batch stream and returns without waiting.
 * lmg_batch_synchronize waits and reports the first failing context.
 * Changing a context's inputs with lmg_inputs_update between replays is
 * allowed (same buffers; synchronize first); changing its mesh, dof map,
 * constraints, sparsity or form, or its stream, requires a new batch.  Do not
 * call a member's own entry points while a replay is in flight. */
typedef struct lmg_batch lmg_batch;
lmg_status lmg_batch_create(lmg_batch **batch, int32_t device);
lmg_status lmg_batch_destroy(lmg_batch *batch);
lmg_status lmg_batch_add(lmg_batch *batch, lmg_ctx *ctx);
lmg_status lmg_batch_tune(lmg_batch *batch, int32_t precision, int32_t reps);
lmg_status lmg_batch_assemble(lmg_batch *batch, int32_t precision);
lmg_status lmg_batch_synchronize(lmg_batch *batch, int64_t *first_failed);
/* The batch stream, kernels per graph replay, and the tuned CTAs per SM of
 * the first n contexts (any pointer may be NULL). */
/* Persistent mode (on = 1): each replay is one persistent kernel launch (after
 * a clear of its queue counters) whose CTAs take work items from a global
 * queue -- every member's element tiles (per-pattern form: the HIERARCHIC
 * members' own tables, and for one-variable affine Poisson members of the
 * block path tables made from their FE tables), then ranges of every
 * member's insertion, each waiting on its member's tiles.  Results equal the
 * members' own assemblies to rounding (1e-13 of the entry); a member that
 * cannot take the per-pattern form makes lmg_batch_assemble return
 * LMG_ERR_UNSUPPORTED.  lmg_batch_tune then picks the elements per CTA tile
 * (8, 16, 32) and the CTAs per SM of the launch by timing replays.  With
 * on = 2 the persistent launch takes only the per-pattern (HIERARCHIC)
 * members, and the other members' own kernels run beside it as branches of
 * the same graph (their results bit-identical to their own assemblies).
 * on = 0 returns to the graph of every member's own kernels. */
lmg_status lmg_batch_set_persistent(lmg_batch *batch, int32_t on);
/* The message of the batch's last failure (NUL-terminated, cut to cap). */
lmg_status lmg_batch_last_error(lmg_batch *batch, char *msg, int32_t cap);
/* Tuned tile and CTAs per SM (0: as many as fit) and the work items of a replay. */
lmg_status lmg_batch_persistent_info(lmg_batch *batch, int32_t *tile, int32_t *ctas_per_sm, int64_t *items);
lmg_status lmg_batch_info(lmg_batch *batch, void **stream, int64_t *launches_per_replay,
                          int32_t *ctas_per_sm, int32_t n);

/* Number of kernels this context has launched since creation. */
lmg_status lmg_launch_count(lmg_ctx *ctx, int64_t *count);

/* Measured FP64 FMA throughput of `device` in TFLOP/s (independent DFMA
 * chains on every SM): the roofline denominator of the FP64 element kernels. */
lmg_status lmg_probe_fp64(int32_t device, double *tflops);

/* Measured FP64 tensor-core throughput of `device` in TFLOP/s (chains of
 * mma.sync m8n8k4 f64 products on every SM): the rate an FP64 DMMA form of the
 * element contractions would be bound by. */
lmg_status lmg_probe_fp64_tensor(int32_t device, double *tflops);

/* The exact FP32 -> FP64 conversion of the kernels' double-float results
 * (bit moves for normal numbers), applied on `device` to n host values: out[i] is in[i]
 * as a double (a check of that conversion against the hardware's). */
lmg_status lmg_probe_f2d(int32_t device, int64_t n, const float *in, double *out);

#ifdef __cplusplus
}
#endif

#endif /* LIBMESH_GB300_H */
