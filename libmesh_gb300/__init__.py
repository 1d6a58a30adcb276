"""libmesh_gb300: GB300-native finite-element assembly behind libMesh's assembly API.

Python mirror of the libMesh objects the assembly path touches, over the C ABI
in include/libmesh_gb300.h (liblmg.so):

  Mesh.build_cube        MeshTools::Generation::build_cube (+ all_tri / all_second_order)
  DofMap                 DofMap::distribute_dofs / dof_indices / add_dirichlet_boundary
  GpuAssembly            a System::Assembly whose assemble() is one device pass
  LinearImplicitSystem   attach_assemble_object / init (compute_sparsity) / assemble

Every numeric path goes through the native library; a missing library raises."""
import ctypes as C

import numpy as np

from . import _capi
from ._capi import (ADVDIFF, ELASTICITY, FP64, HEX8, HEX27, HIERARCHIC, MIXED, POISSON, PRISM6, PRISM18, PRISM21,
                    TET4, TET10, TET14, DegenerateMap, LmgError, check, lib, ptr)

FIRST, SECOND, THIRD, FOURTH, FIFTH = 1, 2, 3, 4, 5

__all__ = ["Mesh", "DofMap", "GpuAssembly", "Batch", "LinearImplicitSystem", "DegenerateMap", "LmgError",
           "HEX8", "HEX27", "TET4", "TET10", "TET14", "PRISM6", "PRISM18", "PRISM21", "POISSON", "ELASTICITY", "ADVDIFF", "FP64", "MIXED", "HIERARCHIC",
           "FIRST", "SECOND", "THIRD", "FOURTH", "FIFTH"]


class Mesh:
    """Host mesh: xyz [n_nodes,3], conn [n_elem,npe] (libMesh node order),
    side_bid [n_elem,n_sides] (boundary id per side, -1 interior)."""

    def __init__(self, xyz, conn, elem_type, side_bid=None):
        self.xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.conn = np.ascontiguousarray(conn, dtype=np.int32)
        self.elem_type = int(elem_type)
        self.side_bid = None if side_bid is None else np.ascontiguousarray(side_bid, dtype=np.int8)

    @property
    def n_nodes(self):
        return self.xyz.shape[0]

    @property
    def n_elem(self):
        return self.conn.shape[0]

    _handle = None

    @staticmethod
    def _arrays(h):
        L = lib()
        nn, ne = C.c_int64(), C.c_int64()
        et, npe, ns = C.c_int32(), C.c_int32(), C.c_int32()
        check(L.lmg_mesh_info(h, C.byref(nn), C.byref(ne), C.byref(et), C.byref(npe), C.byref(ns)))
        xyz = np.empty((nn.value, 3), np.float64)
        conn = np.empty((ne.value, npe.value), np.int32)
        sb = np.empty((ne.value, ns.value), np.int8)
        check(L.lmg_mesh_copy(h, ptr(xyz), ptr(conn), ptr(sb)))
        return xyz, conn, et.value, sb

    @classmethod
    def build_cube(cls, nx, ny, nz, elem_type=HEX8, jitter=0.0, seed=0):
        L = lib()
        h = C.c_void_p()
        check(L.lmg_mesh_cube(nx, ny, nz, elem_type, float(jitter), int(seed), C.byref(h)))
        try:
            xyz, conn, et, sb = cls._arrays(h)
        finally:
            L.lmg_mesh_free(h)
        return cls(xyz, conn, et, sb)

    @classmethod
    def build_refined_cube(cls, n, elem_type, cycles, fraction, seed):
        """build_cube(n,n,n) followed by `cycles` rounds of random h-refinement
        (MeshRefinement with the level-one rule); the mesh keeps its native
        refinement tree for the hanging-node constraints."""
        L = lib()
        h = C.c_void_p()
        check(L.lmg_mesh_cube(n, n, n, elem_type, 0.0, 0, C.byref(h)))
        try:
            check(L.lmg_mesh_refine(h, int(cycles), float(fraction), int(seed)))
            xyz, conn, et, sb = cls._arrays(h)
        except Exception:
            L.lmg_mesh_free(h)
            raise
        m = cls(xyz, conn, et, sb)
        m._handle = h
        return m

    def tree(self):
        """(all_conn, parent, level, active_ids) of the refinement tree."""
        assert self._handle is not None
        L = lib()
        n = C.c_int64()
        check(L.lmg_mesh_tree(self._handle, C.byref(n), None, None, None, None))
        npe = self.conn.shape[1]
        all_conn = np.empty((n.value, npe), np.int32)
        parent = np.empty(n.value, np.int32)
        level = np.empty(n.value, np.int8)
        act = np.empty(self.n_elem, np.int32)
        check(L.lmg_mesh_tree(self._handle, C.byref(n), ptr(all_conn), ptr(parent), ptr(level), ptr(act)))
        return all_conn, parent, level, act

    def __del__(self):
        if self._handle is not None:
            lib().lmg_mesh_free(self._handle)
            self._handle = None


class DofMap:
    """Var-major first-touch numbering of n_vars variables (one VariableGroup);
    elem_dofs[e] is DofMap::dof_indices(elem).  fe_order (| HIERARCHIC) picks
    the FEType whose dofs are numbered: nodal types give one dof per node and
    variable; 3 | HIERARCHIC gives 64 dofs per element on HEX27, 20 on TET14
    and 40 on PRISM21; 2 | HIERARCHIC 18 on PRISM18.  device: number on that
    GPU (the same lists bit for bit)."""

    def __init__(self, mesh, n_vars=1, fe_order=None, device=None):
        self.mesh = mesh
        self.n_vars = int(n_vars)
        self.fe_order = 0 if fe_order is None else int(fe_order)
        n = C.c_int32()
        if self.fe_order:
            check(lib().lmg_fe_dofs_per_elem(mesh.elem_type, self.fe_order, self.n_vars, C.byref(n)))
        else:
            n.value = self.n_vars * mesh.conn.shape[1]
        self.elem_dofs = np.empty((mesh.n_elem, n.value), np.int32)
        nd = C.c_int64()
        if device is None:
            check(lib().lmg_dofmap_distribute_fe(mesh.n_nodes, mesh.n_elem, mesh.elem_type, ptr(mesh.conn),
                                                 self.n_vars, self.fe_order, C.byref(nd), ptr(self.elem_dofs)))
        else:
            check(lib().lmg_dofmap_distribute_device(int(device), mesh.n_nodes, mesh.n_elem, mesh.elem_type,
                                                     ptr(mesh.conn), self.n_vars, self.fe_order, C.byref(nd),
                                                     ptr(self.elem_dofs)))
        self.n_dofs = nd.value
        self.constrained = np.zeros(self.n_dofs, np.uint8)

    def dof_indices(self, e, var=None):
        d = self.elem_dofs[e]
        if var is None:
            return d.copy()
        npe = self.mesh.conn.shape[1]
        return d[var * npe:(var + 1) * npe].copy()

    def add_dirichlet_boundary(self, bids, variables):
        """Homogeneous DirichletBoundary on the listed side ids / variables."""
        bids = np.ascontiguousarray(bids, np.int32)
        variables = np.ascontiguousarray(variables, np.int32)
        c = np.zeros(self.n_dofs, np.uint8)
        check(lib().lmg_dirichlet_dofs_fe(self.mesh.n_elem, self.mesh.elem_type, self.fe_order, self.n_vars,
                                          ptr(self.elem_dofs), ptr(self.mesh.side_bid), ptr(bids),
                                          len(bids), ptr(variables), len(variables), self.n_dofs, ptr(c)))
        self.constrained |= c
        return c

    def is_constrained_dof(self, d):
        return bool(self.constrained[d])

    cons_ptr = cons_col = cons_val = None

    def create_dof_constraints(self, device=None):
        """DofMap::create_dof_constraints + process_constraints: hanging-node
        rows of a refined mesh, then empty rows for the Dirichlet dofs still
        free, chains substituted.  Sets constrained and the rows (CSR over all
        dofs: cons_ptr, cons_col, cons_val).  device: form the hanging-node
        rows on that GPU (the same rows bit for bit)."""
        L = lib()
        h = self.mesh._handle
        owned = h is None
        if owned:  # an unrefined mesh has no hanging nodes: rebuild a handle-free result
            self.cons_ptr = np.zeros(self.n_dofs + 1, np.int64)
            self.cons_ptr[1:] = 0
            self.cons_col = np.zeros(0, np.int32)
            self.cons_val = np.zeros(0, np.float64)
            return
        dirichlet = self.constrained.copy()
        cons = np.zeros(self.n_dofs, np.uint8)
        cp = np.zeros(self.n_dofs + 1, np.int64)
        if device is None:
            rows = lambda *a: L.lmg_constraint_rows(h, *a)  # noqa: E731
        else:
            rows = lambda *a: L.lmg_constraint_rows_device(h, int(device), *a)  # noqa: E731
        check(rows(self.n_vars, ptr(self.elem_dofs), self.n_dofs, ptr(dirichlet), ptr(cons), ptr(cp), None, None, 0))
        total = int(cp[-1])
        col = np.zeros(max(total, 1), np.int32)
        val = np.zeros(max(total, 1), np.float64)
        check(rows(self.n_vars, ptr(self.elem_dofs), self.n_dofs, ptr(dirichlet), ptr(cons), ptr(cp), ptr(col),
                   ptr(val), total))
        self.constrained = cons
        self.cons_ptr, self.cons_col, self.cons_val = cp, col[:total], val[:total]


class GpuAssembly:
    """System::Assembly replacement: one device context per system holding the
    mesh, dof map, constraints, sparsity, scatter plan and form data."""

    def __init__(self, form, fe_order, q_order, elem_coef=None, nodal_f=None, nu=0.3, device=0, params=None):
        """params: the form's parameter list when it has more than nu (ADVDIFF:
        {kappa, n_modes, then per mode a[3], k[3], phase})."""
        self.form, self.fe_order, self.q_order = int(form), int(fe_order), int(q_order)
        self.params = None if params is None else np.ascontiguousarray(params, np.float64)
        self.elem_coef = None if elem_coef is None else np.ascontiguousarray(elem_coef, np.float64)
        self.nodal_f = None if nodal_f is None else np.ascontiguousarray(nodal_f, np.float64)
        self.nu = float(nu)
        self.device = device
        self.ctx = None
        self.nnz = 0

    def _ok(self, st):
        check(st, self.ctx)

    def init(self, mesh, dof_map):
        L = lib()
        if self.ctx is None:
            h = C.c_void_p()
            check(L.lmg_context_create(C.byref(h), self.device))
            self.ctx = h
        self.mesh, self.dof_map = mesh, dof_map
        self._ok(L.lmg_mesh_upload(self.ctx, mesh.n_nodes, ptr(mesh.xyz), mesh.n_elem, mesh.elem_type,
                                   ptr(mesh.conn)))
        self._ok(L.lmg_dofmap_upload_fe(self.ctx, dof_map.n_vars, getattr(dof_map, "fe_order", 0), dof_map.n_dofs,
                                        ptr(dof_map.elem_dofs)))
        if dof_map.cons_ptr is not None and len(dof_map.cons_col):
            self._ok(L.lmg_constraint_rows_upload(self.ctx, ptr(dof_map.constrained), ptr(dof_map.cons_ptr),
                                                  ptr(dof_map.cons_col), ptr(dof_map.cons_val)))
        else:
            self._ok(L.lmg_constraints_upload(self.ctx, ptr(dof_map.constrained)))
        nnz = C.c_int64()
        self._ok(L.lmg_sparsity_build(self.ctx, C.byref(nnz)))
        self.nnz = nnz.value
        params = np.array([self.nu], np.float64) if self.params is None else self.params
        self._ok(L.lmg_form_set(self.ctx, self.form, self.fe_order, self.q_order, ptr(params), len(params),
                                ptr(self.elem_coef), ptr(self.nodal_f)))

    def sparsity(self):
        rp = np.empty(self.dof_map.n_dofs + 1, np.int32)
        ci = np.empty(self.nnz, np.int32)
        self._ok(lib().lmg_sparsity_copy(self.ctx, ptr(rp), ptr(ci)))
        return rp, ci

    def update_inputs(self, xyz=None, elem_coef=None, nodal_f=None):
        self._ok(lib().lmg_inputs_update(self.ctx, ptr(xyz), ptr(elem_coef), ptr(nodal_f)))

    def set_plan_on_device(self, on=True):
        """Build the general path's insertion plan on the device (default) or
        on the host; both give the same plan."""
        self._ok(lib().lmg_context_set_plan_on_device(self.ctx, 1 if on else 0))

    def plan_on_device(self):
        """Whether the last general-path plan was built on the device."""
        v = C.c_int32()
        self._ok(lib().lmg_plan_on_device(self.ctx, C.byref(v)))
        return bool(v.value)

    def sparsity_on_device(self):
        """Whether the sparsity pattern was formed on the device."""
        v = C.c_int32()
        self._ok(lib().lmg_sparsity_on_device(self.ctx, C.byref(v)))
        return bool(v.value)

    def assemble(self, precision=FP64):
        K = np.empty(self.nnz, np.float64)
        F = np.empty(self.dof_map.n_dofs, np.float64)
        self._ok(lib().lmg_assemble(self.ctx, precision, ptr(K), ptr(F), 0))
        return K, F

    def assemble_device(self, precision=FP64, K_dev=None, F_dev=None):
        """Assemble into device buffers (raw pointers, e.g. torch data_ptr());
        None keeps the result in the context's own buffers.  Asynchronous."""
        on_dev = 1 if (K_dev is not None or F_dev is not None) else 0
        self._ok(lib().lmg_assemble(self.ctx, precision,
                                    None if K_dev is None else C.c_void_p(K_dev),
                                    None if F_dev is None else C.c_void_p(F_dev), on_dev))

    def synchronize(self):
        self._ok(lib().lmg_synchronize(self.ctx))

    def set_stream(self, stream_ptr):
        self._ok(lib().lmg_context_set_stream(self.ctx, C.c_void_p(stream_ptr)))

    def solve(self, rhs=None, rtol=1e-10, maxit=20000):
        """CG on the last assembled system; returns (x, iterations, relative residual)."""
        x = np.empty(self.dof_map.n_dofs, np.float64)
        it, rr = C.c_int32(), C.c_double()
        b = None if rhs is None else np.ascontiguousarray(rhs, np.float64)
        self._ok(lib().lmg_cg_solve(self.ctx, ptr(b), ptr(x), float(rtol), int(maxit), C.byref(it), C.byref(rr)))
        return x, it.value, rr.value

    def qoi_region_load(self, in_region):
        """dq/du of q(u) = integral of u over the marked elements."""
        q = np.empty(self.dof_map.n_dofs, np.float64)
        self._ok(lib().lmg_qoi_region_load(self.ctx, ptr(np.ascontiguousarray(in_region, np.uint8)), ptr(q)))
        return q

    def vjp_coef(self, u, z):
        """dq/dcoef_e = -z_e^T dK_e/dcoef_e u_e for every element."""
        g = np.empty(self.mesh.n_elem, np.float64)
        self._ok(lib().lmg_vjp_coef(self.ctx, ptr(np.ascontiguousarray(u, np.float64)),
                                    ptr(np.ascontiguousarray(z, np.float64)), ptr(g)))
        return g

    def residual(self, u):
        """R = K u - F without forming K (affine elements of the block path)."""
        R = np.empty(self.dof_map.n_dofs, np.float64)
        self._ok(lib().lmg_residual(self.ctx, ptr(np.ascontiguousarray(u, np.float64)), ptr(R), 0))
        return R

    def residual_device(self, u_dev, R_dev):
        """The same on device vectors (raw pointers); asynchronous."""
        self._ok(lib().lmg_residual(self.ctx, C.c_void_p(u_dev), C.c_void_p(R_dev), 1))

    def vjp_xyz(self, u, z, in_region=None):
        """dq/dx for every node coordinate (Poisson form): [n_nodes, 3]."""
        g = np.empty((self.mesh.n_nodes, 3), np.float64)
        reg = None if in_region is None else np.ascontiguousarray(in_region, np.uint8)
        self._ok(lib().lmg_vjp_xyz(self.ctx, ptr(np.ascontiguousarray(u, np.float64)),
                                   ptr(np.ascontiguousarray(z, np.float64)), ptr(reg), ptr(g)))
        return g

    def set_tensor_cores(self, on=True):
        """Mixed form on non-affine elements: per-point Gram products on the
        tensor cores (default) or on the CUDA cores."""
        self._ok(lib().lmg_context_set_tensor_cores(self.ctx, 1 if on else 0))

    def perflog_enable(self, on=True):
        self._ok(lib().lmg_perflog_enable(self.ctx, 1 if on else 0))

    def perflog_read(self):
        """(element-kernel ms, insertion ms, calls) summed since the last read."""
        a, b, n = C.c_double(), C.c_double(), C.c_int64()
        self._ok(lib().lmg_perflog_read(self.ctx, C.byref(a), C.byref(b), C.byref(n)))
        return a.value, b.value, n.value

    def assemble_into(self, K_ptr, F_ptr, precision=FP64, on_device=False):
        """Assemble into caller buffers given as raw addresses (host or device)."""
        self._ok(lib().lmg_assemble(self.ctx, precision, C.c_void_p(K_ptr), C.c_void_p(F_ptr),
                                    1 if on_device else 0))

    def result(self):
        """(K, F) of the last assembly, copied from the device."""
        K = np.empty(self.nnz, np.float64)
        F = np.empty(self.dof_map.n_dofs, np.float64)
        self._ok(lib().lmg_result_copy(self.ctx, ptr(K), ptr(F)))
        return K, F

    def set_grid(self, ctas_per_sm):
        self._ok(lib().lmg_context_set_grid(self.ctx, int(ctas_per_sm)))

    def launch_count(self):
        n = C.c_int64()
        self._ok(lib().lmg_launch_count(self.ctx, C.byref(n)))
        return n.value

    def close(self):
        if self.ctx is not None:
            lib().lmg_context_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def probe_fp64(device=0):
    """Measured FP64 FMA throughput (TFLOP/s) of the device."""
    t = C.c_double()
    check(lib().lmg_probe_fp64(device, C.byref(t)))
    return t.value


def probe_fp64_tensor(device=0):
    """Measured FP64 tensor-core (DMMA m8n8k4) throughput (TFLOP/s) of the device."""
    t = C.c_double()
    check(lib().lmg_probe_fp64_tensor(device, C.byref(t)))
    return t.value


def probe_f2d(values, device=0):
    """The kernels' exact FP32 -> FP64 conversion applied on the device."""
    x = np.ascontiguousarray(values, np.float32)
    out = np.empty(x.shape, np.float64)
    check(lib().lmg_probe_f2d(device, x.size, ptr(x), ptr(out)))
    return out


class LinearImplicitSystem:
    """The parts of libMesh's LinearImplicitSystem the assembly path uses."""

    def __init__(self, mesh, n_vars=1):
        self.mesh = mesh
        self.dof_map = DofMap(mesh, n_vars)
        self.assembly = None
        self.matrix = None
        self.rhs = None

    def attach_assemble_object(self, assembly):
        self.assembly = assembly

    def init(self):
        self.assembly.init(self.mesh, self.dof_map)
        self.row_ptr, self.col_idx = self.assembly.sparsity()

    def assemble(self, precision=FP64):
        K, F = self.assembly.assemble(precision)
        self.matrix, self.rhs = K, F
        return K, F

    def adjoint_qoi_parameter_sensitivity(self, in_region, rtol=1e-12, maxit=50000):
        """q(u) = integral of u over the marked elements; returns (q, dq/dcoef_e for
        every element) from one primal and one adjoint solve and one VJP pass
        (ImplicitSystem::adjoint_qoi_parameter_sensitivity with the element
        coefficients as the ParameterVector)."""
        a = self.assembly
        a.assemble()
        u, _, _ = a.solve(rtol=rtol, maxit=maxit)
        qv = a.qoi_region_load(in_region)
        z, _, _ = a.solve(rhs=qv, rtol=rtol, maxit=maxit)
        return float(qv @ u), a.vjp_coef(u, z)

    def matrix_csr(self):
        import scipy.sparse as sp
        n = self.dof_map.n_dofs
        return sp.csr_matrix((self.matrix, self.col_idx, self.row_ptr), shape=(n, n))


class Batch:
    """Many set-up GpuAssembly objects assembled as one CUDA graph
    (lmg_batch_*): add, tune, then assemble / synchronize repeatedly."""

    def __init__(self, device=0):
        h = C.c_void_p()
        check(lib().lmg_batch_create(C.byref(h), device))
        self.h = h
        self.members = []

    def add(self, assembly):
        check(lib().lmg_batch_add(self.h, assembly.ctx))
        self.members.append(assembly)

    def _ok(self, status):
        if status != 0:
            buf = C.create_string_buffer(512)
            lib().lmg_batch_last_error(self.h, buf, 512)
            raise LmgError(status, buf.value.decode(errors="replace"))

    def tune(self, precision=FP64, reps=3):
        self._ok(lib().lmg_batch_tune(self.h, precision, reps))

    def assemble(self, precision=FP64):
        self._ok(lib().lmg_batch_assemble(self.h, precision))

    def synchronize(self):
        bad = C.c_int64(-1)
        self._ok(lib().lmg_batch_synchronize(self.h, C.byref(bad)))

    def set_persistent(self, on=True, hybrid=False):
        """One persistent kernel launch per replay (every member's element
        tiles and insertion from one work queue); with hybrid=True only the
        per-pattern (HIERARCHIC) members go through it and the others' own
        kernels run beside it in the same graph."""
        check(lib().lmg_batch_set_persistent(self.h, (2 if hybrid else 1) if on else 0))

    def persistent_info(self):
        t, c, n = C.c_int32(), C.c_int32(), C.c_int64()
        check(lib().lmg_batch_persistent_info(self.h, C.byref(t), C.byref(c), C.byref(n)))
        return t.value, c.value, n.value

    def info(self):
        s, l = C.c_void_p(), C.c_int64()
        g = np.zeros(len(self.members), np.int32)
        check(lib().lmg_batch_info(self.h, C.byref(s), C.byref(l), ptr(g), len(self.members)))
        return s.value, l.value, g

    def close(self):
        if self.h is not None:
            lib().lmg_batch_destroy(self.h)
            self.h = None
