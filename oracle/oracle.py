"""ctypes front end of the CPU oracle (oracle.cpp).  Test infrastructure only:
tests/, __graft_entry__.smoke() and bench.py's CPU legs use it as the checker."""
import ctypes as C
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import build as _build  # noqa: E402

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = C.CDLL(_build.build())
        v, i32, i64, f64 = C.c_void_p, C.c_int32, C.c_int64, C.c_double
        _lib.orc_qgauss.argtypes = [i32, i32, v, v, i32]
        _lib.orc_shapes.argtypes = [i32, i32, i32, v, v, v]
        _lib.orc_has_affine_map.argtypes = [i32, v]
        _lib.orc_distribute_dofs.argtypes = [i64, i64, i32, v, i32, v, C.POINTER(i64)]
        _lib.orc_dirichlet.argtypes = [i64, i32, i32, v, v, v, i32, v, i32, v]
        _lib.orc_sparsity.argtypes = [i64, i64, i32, v, C.POINTER(i64), v, v]
        _lib.orc_assemble.argtypes = [i32, i32, i32, i32, i64, v, i64, v, i32, v, i64, v, v, v, f64,
                                      v, v, v, v, i32, i64, i64, C.POINTER(i64), C.POINTER(f64)]
        _lib.orc_assemble2.argtypes = _lib.orc_assemble.argtypes + [v, v, v, v, i32]
        _lib.orc_constraint_rows.argtypes = [i32, i64, v, i64, v, v, v, i64, v, i32, v, i64, v, v, v, v, v, i64]
        _lib.orc_constraint_rows.restype = i64
        _lib.orc_sparsity_constrained.argtypes = [i64, i64, i32, v, v, v, C.POINTER(i64), v, v]
        _lib.orc_shapes_hier3.argtypes = [v, i32, v, v, v]
        _lib.orc_distribute_dofs_hier3.argtypes = [i64, i64, v, v, C.POINTER(i64)]
        _lib.orc_dirichlet_hier3.argtypes = [i64, v, v, v, i32, v]
        _lib.orc_shapes_tet3.argtypes = [v, i32, v, v, v]
        _lib.orc_shapes_hier_hex.argtypes = [v, i32, i32, v, v, v]
        _lib.orc_shapes_hier_hex.restype = C.c_int32
        _lib.orc_shapes_hier_prism.argtypes = [v, i32, i32, v, v, v]
        _lib.orc_shapes_hier_prism.restype = C.c_int32
        _lib.orc_distribute_dofs_prism.argtypes = [i32, i64, i64, v, v, C.POINTER(i64)]
        _lib.orc_distribute_dofs_prism.restype = C.c_int32
        _lib.orc_dirichlet_prism.argtypes = [i32, i64, v, v, v, i32, v]
        _lib.orc_dirichlet_prism.restype = C.c_int32
        _lib.orc_distribute_dofs_tet3.argtypes = [i64, i64, v, v, C.POINTER(i64)]
        _lib.orc_dirichlet_tet3.argtypes = [i64, v, v, v, i32, v]
        _lib.orc_mesh_cube.argtypes = [i32, i32, i32, i32, f64, C.c_uint64]
        _lib.orc_mesh_cube.restype = v
        _lib.orc_mesh_info.argtypes = [v, C.POINTER(i64), C.POINTER(i64), C.POINTER(i32), C.POINTER(i32)]
        _lib.orc_mesh_info.restype = None
        _lib.orc_mesh_copy.argtypes = [v, v, v, v]
        _lib.orc_mesh_copy.restype = None
        _lib.orc_mesh_free.argtypes = [v]
        _lib.orc_mesh_free.restype = None
        for f in (_lib.orc_qgauss, _lib.orc_shapes, _lib.orc_has_affine_map, _lib.orc_distribute_dofs,
                  _lib.orc_dirichlet, _lib.orc_sparsity, _lib.orc_assemble, _lib.orc_assemble2,
                  _lib.orc_sparsity_constrained, _lib.orc_shapes_hier3, _lib.orc_distribute_dofs_hier3,
                  _lib.orc_dirichlet_hier3, _lib.orc_shapes_tet3, _lib.orc_distribute_dofs_tet3,
                  _lib.orc_dirichlet_tet3):
            f.restype = C.c_int32
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def qgauss(elem_type, order):
    pts = np.zeros((1000, 3))
    w = np.zeros(1000)
    n = lib().orc_qgauss(elem_type, order, _p(pts), _p(w), 1000)
    assert n > 0
    return pts[:n].copy(), w[:n].copy()


def shapes(elem_type, order, pts):
    pts = np.ascontiguousarray(pts, np.float64)
    np_ = pts.shape[0]
    phi = np.zeros((64, np_))
    dphi = np.zeros((3, 64, np_))
    n = lib().orc_shapes(elem_type, order, np_, _p(pts), _p(phi), _p(dphi.reshape(-1)))
    assert n > 0
    dphi = dphi.reshape(-1)[:3 * n * np_].reshape(3, n, np_)
    return phi.reshape(-1)[:n * np_].reshape(n, np_).copy(), dphi.copy()


def mesh_cube(n, elem_type, jitter=0.0, seed=0):
    """build_cube(n^3) restated (oracle_mesh.cpp): HEX8 / HEX27 directly, TET4 /
    TET10 through all_tri [and all_second_order], interior vertices jittered
    by +-jitter*h before the split.  Returns (xyz [n_nodes][3], conn
    [n_elem][npe], side_bid [n_elem][n_sides])."""
    h = lib().orc_mesh_cube(n, n, n, elem_type, float(jitter), seed)
    assert h, "orc_mesh_cube: bad argument"
    try:
        nn, ne, npe, ns = C.c_int64(), C.c_int64(), C.c_int32(), C.c_int32()
        lib().orc_mesh_info(h, C.byref(nn), C.byref(ne), C.byref(npe), C.byref(ns))
        xyz = np.zeros((nn.value, 3))
        conn = np.zeros((ne.value, npe.value), np.int32)
        sb = np.zeros((ne.value, ns.value), np.int8)
        lib().orc_mesh_copy(h, _p(xyz), _p(conn), _p(sb))
    finally:
        lib().orc_mesh_free(h)
    return xyz, conn, sb


def has_affine_map(elem_type, X):
    return bool(lib().orc_has_affine_map(elem_type, _p(np.ascontiguousarray(X, np.float64))))


def distribute_dofs(n_nodes, conn, n_vars):
    conn = np.ascontiguousarray(conn, np.int32)
    ed = np.zeros((conn.shape[0], n_vars * conn.shape[1]), np.int32)
    nd = C.c_int64()
    lib().orc_distribute_dofs(n_nodes, conn.shape[0], conn.shape[1], _p(conn), n_vars, _p(ed), C.byref(nd))
    return ed, nd.value


def shapes_hier3(X27, pts):
    """Cubic HIERARCHIC shapes of one HEX27 (node coordinates X27 [27][3]) at
    reference points: phi [64][np], dphi [3][64][np]."""
    pts = np.ascontiguousarray(pts, np.float64)
    phi = np.zeros((64, len(pts)))
    dphi = np.zeros((3, 64, len(pts)))
    lib().orc_shapes_hier3(_p(np.ascontiguousarray(X27, np.float64)), len(pts), _p(pts), _p(phi), _p(dphi))
    return phi, dphi


def distribute_dofs_hier3(n_nodes, conn):
    """FEType{THIRD, HIERARCHIC} dof numbering and dof_indices on HEX27: [n_elem][64]."""
    conn = np.ascontiguousarray(conn, np.int32)
    ed = np.zeros((conn.shape[0], 64), np.int32)
    nd = C.c_int64()
    lib().orc_distribute_dofs_hier3(n_nodes, conn.shape[0], _p(conn), _p(ed), C.byref(nd))
    return ed, nd.value


def dirichlet_hier3(elem_dofs, side_bid, bids, n_dofs):
    bids = np.ascontiguousarray(bids, np.int32)
    c = np.zeros(n_dofs, np.uint8)
    lib().orc_dirichlet_hier3(elem_dofs.shape[0], _p(np.ascontiguousarray(elem_dofs, np.int32)),
                              _p(np.ascontiguousarray(side_bid, np.int8)), _p(bids), len(bids), _p(c))
    return c


def shapes_hier_hex(X27, order, pts):
    """HIERARCHIC shapes of order 2 or 3 of one HEX27 (node coordinates X27
    [27][3]) with its edge and face orientation: phi [n][np], dphi [3][n][np]."""
    pts = np.ascontiguousarray(pts, np.float64)
    n = (order + 1) ** 3
    phi = np.zeros((n, len(pts)))
    dphi = np.zeros((3, n, len(pts)))
    assert lib().orc_shapes_hier_hex(_p(np.ascontiguousarray(X27, np.float64)), order, len(pts), _p(pts), _p(phi),
                                     _p(dphi)) == n
    return phi, dphi


def shapes_hier_prism(X6, order, pts):
    """HIERARCHIC shapes of order 2 or 3 on one prism (vertex coordinates X6
    [6][3]) at reference points: phi [n][np], dphi [3][n][np]."""
    pts = np.ascontiguousarray(pts, np.float64)
    n = (order + 1) * (order + 1) * (order + 2) // 2
    phi = np.zeros((n, len(pts)))
    dphi = np.zeros((3, n, len(pts)))
    assert lib().orc_shapes_hier_prism(_p(np.ascontiguousarray(np.asarray(X6)[:6], np.float64)), order, len(pts),
                                       _p(pts), _p(phi), _p(dphi)) == n
    return phi, dphi


def distribute_dofs_prism(p, n_nodes, conn):
    """HIERARCHIC dof numbering and dof_indices of order p = 2 on PRISM18 or
    p = 3 on PRISM21: [n_elem][(p+1)^2 (p+2)/2]."""
    conn = np.ascontiguousarray(conn, np.int32)
    nl = (p + 1) * (p + 1) * (p + 2) // 2
    ed = np.zeros((conn.shape[0], nl), np.int32)
    nd = C.c_int64()
    lib().orc_distribute_dofs_prism(p, n_nodes, conn.shape[0], _p(conn), _p(ed), C.byref(nd))
    return ed, nd.value


def dirichlet_prism(p, elem_dofs, side_bid, bids, n_dofs):
    """Dofs on the nodes of the boundary sides with ids in bids (homogeneous Dirichlet)."""
    cons = np.zeros(n_dofs, np.uint8)
    bids = np.ascontiguousarray(bids, np.int32)
    lib().orc_dirichlet_prism(p, elem_dofs.shape[0], _p(np.ascontiguousarray(elem_dofs, np.int32)),
                              _p(np.ascontiguousarray(side_bid, np.int8)), _p(bids), len(bids), _p(cons))
    return cons


def shapes_tet3(X14, pts):
    """Cubic HIERARCHIC shapes of one TET14 (node coordinates X14 [14][3]) at
    reference points: phi [20][np], dphi [3][20][np]."""
    pts = np.ascontiguousarray(pts, np.float64)
    phi = np.zeros((20, len(pts)))
    dphi = np.zeros((3, 20, len(pts)))
    lib().orc_shapes_tet3(_p(np.ascontiguousarray(X14, np.float64)), len(pts), _p(pts), _p(phi), _p(dphi))
    return phi, dphi


def distribute_dofs_tet3(n_nodes, conn):
    """FEType{THIRD, HIERARCHIC} dof numbering and dof_indices on TET14: [n_elem][20]."""
    conn = np.ascontiguousarray(conn, np.int32)
    ed = np.zeros((conn.shape[0], 20), np.int32)
    nd = C.c_int64()
    lib().orc_distribute_dofs_tet3(n_nodes, conn.shape[0], _p(conn), _p(ed), C.byref(nd))
    return ed, nd.value


def dirichlet_tet3(elem_dofs, side_bid, bids, n_dofs):
    bids = np.ascontiguousarray(bids, np.int32)
    c = np.zeros(n_dofs, np.uint8)
    lib().orc_dirichlet_tet3(elem_dofs.shape[0], _p(np.ascontiguousarray(elem_dofs, np.int32)),
                             _p(np.ascontiguousarray(side_bid, np.int8)), _p(bids), len(bids), _p(c))
    return c


def dirichlet(elem_type, n_vars, elem_dofs, side_bid, bids, variables, n_dofs):
    bids = np.ascontiguousarray(bids, np.int32)
    variables = np.ascontiguousarray(variables, np.int32)
    c = np.zeros(n_dofs, np.uint8)
    lib().orc_dirichlet(elem_dofs.shape[0], elem_type, n_vars, _p(np.ascontiguousarray(elem_dofs)),
                        _p(np.ascontiguousarray(side_bid, np.int8)), _p(bids), len(bids), _p(variables),
                        len(variables), _p(c))
    return c


def sparsity(n_dofs, elem_dofs):
    ed = np.ascontiguousarray(elem_dofs, np.int32)
    nnz = C.c_int64()
    lib().orc_sparsity(n_dofs, ed.shape[0], ed.shape[1], _p(ed), C.byref(nnz), None, None)
    rp = np.zeros(n_dofs + 1, np.int32)
    col = np.zeros(nnz.value, np.int32)
    lib().orc_sparsity(n_dofs, ed.shape[0], ed.shape[1], _p(ed), C.byref(nnz), _p(rp), _p(col))
    return rp, col


ADVDIFF = 2


def constraint_rows(elem_type, xyz, all_conn, parent, level, active_ids, n_vars, elem_dofs, n_dofs, dirichlet):
    """Hanging-node rows + Dirichlet rows + process_constraints on a refined
    hex mesh.  Returns (constrained, cons_ptr, cons_col, cons_val)."""
    xyz = np.ascontiguousarray(xyz, np.float64)
    all_conn = np.ascontiguousarray(all_conn, np.int32)
    parent = np.ascontiguousarray(parent, np.int32)
    level = np.ascontiguousarray(level, np.int8)
    act = np.ascontiguousarray(active_ids, np.int32)
    ed = np.ascontiguousarray(elem_dofs, np.int32)
    dr = None if dirichlet is None else np.ascontiguousarray(dirichlet, np.uint8)
    cons = np.zeros(n_dofs, np.uint8)
    ptr_ = np.zeros(n_dofs + 1, np.int64)
    args = (elem_type, xyz.shape[0], _p(xyz), all_conn.shape[0], _p(all_conn), _p(parent), _p(level),
            act.shape[0], _p(act), n_vars, _p(ed), n_dofs, _p(dr), _p(cons), _p(ptr_))
    total = lib().orc_constraint_rows(*args, None, None, 0)
    col = np.zeros(max(total, 1), np.int32)
    val = np.zeros(max(total, 1), np.float64)
    assert lib().orc_constraint_rows(*args, _p(col), _p(val), total) == total
    return cons, ptr_, col[:total], val[:total]


def sparsity_constrained(n_dofs, elem_dofs, cons_ptr, cons_col):
    ed = np.ascontiguousarray(elem_dofs, np.int32)
    cp = np.ascontiguousarray(cons_ptr, np.int64)
    cc = np.ascontiguousarray(cons_col, np.int32)
    nnz = C.c_int64()
    lib().orc_sparsity_constrained(n_dofs, ed.shape[0], ed.shape[1], _p(ed), _p(cp), _p(cc), C.byref(nnz), None, None)
    rp = np.zeros(n_dofs + 1, np.int32)
    col = np.zeros(nnz.value, np.int32)
    lib().orc_sparsity_constrained(n_dofs, ed.shape[0], ed.shape[1], _p(ed), _p(cp), _p(cc), C.byref(nnz), _p(rp),
                                   _p(col))
    return rp, col


def assemble(form, elem_type, fe_order, q_order, xyz, conn, n_vars, elem_dofs, n_dofs, constrained,
             row_ptr, col, coef=None, nodal_f=None, nu=0.3, n_threads=1, e_range=None, timing=None,
             cons_rows=None, params=None):
    """Returns (K values, F, status, first bad element); timing (a dict) gets
    the wall time of the element loop under "seconds".  cons_rows =
    (cons_ptr, cons_col, cons_val) gives the constraint rows (default: empty
    rows); params the form parameters (ADVDIFF)."""
    xyz = np.ascontiguousarray(xyz, np.float64)
    conn = np.ascontiguousarray(conn, np.int32)
    ed = np.ascontiguousarray(elem_dofs, np.int32)
    cons = np.ascontiguousarray(constrained, np.uint8)
    coef = None if coef is None else np.ascontiguousarray(coef, np.float64)
    nodal_f = None if nodal_f is None else np.ascontiguousarray(nodal_f, np.float64)
    K = np.zeros(int(row_ptr[-1]))
    F = np.zeros(n_dofs)
    b, e = (0, conn.shape[0]) if e_range is None else e_range
    bad = C.c_int64(-1)
    secs = C.c_double(0)
    cr = (None, None, None) if cons_rows is None else (np.ascontiguousarray(cons_rows[0], np.int64),
                                                         np.ascontiguousarray(cons_rows[1], np.int32),
                                                         np.ascontiguousarray(cons_rows[2], np.float64))
    pr = None if params is None else np.ascontiguousarray(params, np.float64)
    st = lib().orc_assemble2(form, elem_type, fe_order, q_order, xyz.shape[0], _p(xyz), conn.shape[0],
                             _p(conn), n_vars, _p(ed), n_dofs, _p(cons), _p(coef), _p(nodal_f), nu,
                             _p(np.ascontiguousarray(row_ptr, np.int32)), _p(np.ascontiguousarray(col, np.int32)),
                             _p(K), _p(F), n_threads, b, e, C.byref(bad), C.byref(secs),
                             _p(cr[0]), _p(cr[1]), _p(cr[2]), _p(pr), 0 if pr is None else len(pr))
    if timing is not None:
        timing["seconds"] = secs.value
    return K, F, st, bad.value


def adjoint_qoi_parameter_sensitivity(form, elem_type, fe_order, q_order, xyz, conn, n_vars, elem_dofs, n_dofs,
                                      constrained, row_ptr, col, coef, nodal_f, in_region, params, nu=0.3):
    """Restatement of ImplicitSystem::adjoint_qoi_parameter_sensitivity
    (src/systems/implicit_system.C:474-623) for q(u) = integral of u over the
    marked elements and the element coefficients listed in `params`:
    u from K u = F; z from K^T z = dq/du (constrained dofs held at zero);
    for each parameter p: delta = 1e-6 max(|p|, 1e-3), the residual R = K u - F
    assembled at p - delta and p + delta, -dR/dp = (R(p-d) - R(p+d)) / (2 d),
    dq/dp = (q(p+d) - q(p-d)) / (2 d) (zero here: q does not depend on p),
    sensitivity = dq/dp + (-dR/dp) . z.  Small meshes only (two full
    assemblies per parameter).  Returns (q, sensitivities)."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n = n_dofs
    K, F, st, _ = assemble(form, elem_type, fe_order, q_order, xyz, conn, n_vars, elem_dofs, n_dofs, constrained,
                           row_ptr, col, coef=coef, nodal_f=nodal_f, nu=nu)
    assert st == 0
    A = sp.csc_matrix(sp.csr_matrix((K, col, row_ptr), shape=(n, n)))
    u = spla.spsolve(A, F)
    sel = np.nonzero(np.asarray(in_region) != 0)[0]
    ones = np.ones((xyz.shape[0], n_vars))
    _, qv, st, _ = assemble(form, elem_type, fe_order, q_order, xyz, conn[sel], n_vars, elem_dofs[sel], n_dofs,
                            np.zeros(n_dofs, np.uint8), row_ptr, col, coef=coef[sel], nodal_f=ones, nu=nu)
    assert st == 0
    qv[np.asarray(constrained) != 0] = 0.0
    z = spla.spsolve(A.T.tocsc(), qv)
    sens = []
    for j in params:
        old = coef[j]
        d = 1e-6 * max(abs(old), 1e-3)
        cm, cp = coef.copy(), coef.copy()
        cm[j], cp[j] = old - d, old + d
        Km, Fm, _, _ = assemble(form, elem_type, fe_order, q_order, xyz, conn, n_vars, elem_dofs, n_dofs, constrained,
                                row_ptr, col, coef=cm, nodal_f=nodal_f, nu=nu)
        Kp, Fp, _, _ = assemble(form, elem_type, fe_order, q_order, xyz, conn, n_vars, elem_dofs, n_dofs, constrained,
                                row_ptr, col, coef=cp, nodal_f=nodal_f, nu=nu)
        Rm = sp.csr_matrix((Km, col, row_ptr), shape=(n, n)) @ u - Fm
        Rp = sp.csr_matrix((Kp, col, row_ptr), shape=(n, n)) @ u - Fp
        neg = (Rm - Rp) / (2 * d)
        sens.append(0.0 + neg @ z)
    return float(qv @ u), np.array(sens)


def coordinate_sensitivity(form, elem_type, fe_order, q_order, xyz, conn, elem_dofs, n_dofs, constrained, row_ptr,
                           col, coef, nodal_f, in_region, params, n_vars=1):
    """adjoint_qoi_parameter_sensitivity (src/systems/implicit_system.C:474-623)
    with node coordinates as the ParameterVector: params = [(node, direction)].
    For each p = xyz[node, direction]: delta = 1e-6 max(|p|, 1e-3);
    dq/dp = (q(u; p+d) - q(u; p-d)) / 2d at the fixed primal u (the QoI is the
    integral of u over the marked elements, so it moves with the geometry);
    -dR/dp = (R(p-d) - R(p+d)) / 2d with R = K u - F;
    sensitivity = dq/dp + (-dR/dp) . z.  n_vars = 3 (elasticity): the QoI
    integrates the sum of the components.  Small meshes."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla
    n = n_dofs
    sel = np.nonzero(np.asarray(in_region) != 0)[0]

    def system(x):
        K, F, st, _ = assemble(form, elem_type, fe_order, q_order, x, conn, n_vars, elem_dofs, n_dofs, constrained,
                               row_ptr, col, coef=coef, nodal_f=nodal_f)
        assert st == 0
        return sp.csr_matrix((K, col, row_ptr), shape=(n, n)), F

    def qload(x):
        ones = np.ones((x.shape[0], n_vars))
        _, qv, st, _ = assemble(form, elem_type, fe_order, q_order, x, conn[sel], n_vars, elem_dofs[sel], n_dofs,
                                np.zeros(n_dofs, np.uint8), row_ptr, col, coef=coef[sel], nodal_f=ones)
        assert st == 0
        qv[np.asarray(constrained) != 0] = 0.0
        return qv

    A, F = system(xyz)
    u = spla.spsolve(A.tocsc(), F)
    qv = qload(xyz)
    z = spla.spsolve(A.T.tocsc(), qv)
    out = []
    for node, d in params:
        p = xyz[node, d]
        h = 1e-6 * max(abs(p), 1e-3)
        xm, xp = xyz.copy(), xyz.copy()
        xm[node, d] -= h
        xp[node, d] += h
        Am, Fm = system(xm)
        Ap, Fp = system(xp)
        neg = ((Am @ u - Fm) - (Ap @ u - Fp)) / (2 * h)
        dq = (qload(xp) @ u - qload(xm) @ u) / (2 * h)
        out.append(dq + neg @ z)
    return float(qv @ u), np.array(out)
