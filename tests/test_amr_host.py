"""Host mirror of h-refinement, hanging-node constraint rows and the
constrained sparsity pattern, against the oracle's restatements of
lagrange_compute_constraints (with FEMap::inverse_map), process_constraints
and compute_sparsity + find_connected_dofs (CPU)."""
import ctypes as C

import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from libmesh_gb300 import _capi

CASES = [(4, lm.HEX27, 3, 2), (3, lm.HEX8, 3, 5), (5, lm.HEX27, 2, 7)]


def refined(n, et, cycles, seed, dirichlet):
    m = lm.Mesh.build_refined_cube(n, et, cycles, 0.2, seed)
    dm = lm.DofMap(m, 1)
    if dirichlet:
        dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    mask = dm.constrained.copy()
    dm.create_dof_constraints()
    return m, dm, mask


@pytest.mark.parametrize("n,et,cycles,seed", CASES)
def test_refinement_is_a_conforming_partition(n, et, cycles, seed):
    m = lm.Mesh.build_refined_cube(n, et, cycles, 0.2, seed)
    all_conn, parent, level, act = m.tree()
    x = m.xyz[m.conn]
    vol = np.prod(x[:, 6] - x[:, 0], axis=1)
    assert abs(vol.sum() - 1.0) < 1e-12                          # active elements tile the cube
    assert np.all(vol > 0)
    assert len(np.unique(m.xyz.round(12), axis=0)) == m.n_nodes    # no duplicate nodes
    assert level[act].max() <= cycles and level[act].min() >= 0
    assert np.all(parent[act[level[act] > 0]] >= 0)
    kids = np.bincount(parent[parent >= 0])
    assert np.all(kids[kids > 0] == 8)                            # every refined element has 8 children


@pytest.mark.parametrize("n,et,cycles,seed", CASES)
@pytest.mark.parametrize("dirichlet", [False, True])
def test_constraint_rows_match_oracle(n, et, cycles, seed, dirichlet):
    m, dm, mask = refined(n, et, cycles, seed, dirichlet)
    all_conn, parent, level, act = m.tree()
    c2, p2, col2, val2 = orc.constraint_rows(m.elem_type, m.xyz, all_conn, parent, level, act, 1, dm.elem_dofs,
                                             dm.n_dofs, mask)
    assert (c2 == dm.constrained).all()
    assert (p2 == dm.cons_ptr).all() and (col2 == dm.cons_col).all()
    # the product maps hanging nodes to exact lattice coordinates, the oracle by Newton
    np.testing.assert_allclose(dm.cons_val, val2, rtol=0, atol=1e-13)
    assert (np.diff(dm.cons_ptr) > 0).sum() > 0


@pytest.mark.parametrize("n,et,cycles,seed", CASES)
def test_constraint_rows_reproduce_the_element_space(n, et, cycles, seed):
    """Without Dirichlet rows every hanging dof equals its row applied to any
    field of the element space (quadratic for HEX27, trilinear for HEX8)."""
    m, dm, _ = refined(n, et, cycles, seed, False)
    nd = np.zeros(dm.n_dofs, np.int64)
    nd[dm.elem_dofs.reshape(-1)] = m.conn.reshape(-1)
    p = m.xyz[nd]
    if et == lm.HEX27:
        u = 1 + p[:, 0] + 2 * p[:, 1] * p[:, 2] + 0.5 * p[:, 0] ** 2 - p[:, 2] ** 2 * p[:, 1] ** 2
    else:
        u = 1 + p[:, 0] - 2 * p[:, 1] + 3 * p[:, 2] + p[:, 0] * p[:, 1] * p[:, 2]
    rp = dm.cons_ptr
    for d in np.nonzero(np.diff(rp) > 0)[0]:
        s = slice(rp[d], rp[d + 1])
        assert abs((dm.cons_val[s] * u[dm.cons_col[s]]).sum() - u[d]) < 1e-13
    assert np.all(dm.constrained[np.diff(rp) > 0])


@pytest.mark.parametrize("n,et,cycles,seed", CASES[:2])
def test_constrained_sparsity_matches_oracle(n, et, cycles, seed):
    m, dm, _ = refined(n, et, cycles, seed, True)
    rp_o, col_o = orc.sparsity_constrained(dm.n_dofs, dm.elem_dofs, dm.cons_ptr, dm.cons_col)
    L = _capi.lib()
    nnz = C.c_int64()
    args = (dm.elem_dofs.shape[0], dm.elem_dofs.shape[1], dm.n_dofs, _capi.ptr(dm.elem_dofs),
            _capi.ptr(dm.cons_ptr), _capi.ptr(dm.cons_col), C.byref(nnz))
    assert L.lmg_host_sparsity_constrained(*args, None, None) == 0
    rp = np.zeros(dm.n_dofs + 1, np.int32)
    col = np.zeros(nnz.value, np.int32)
    assert L.lmg_host_sparsity_constrained(*args, _capi.ptr(rp), _capi.ptr(col)) == 0
    assert np.array_equal(rp, rp_o) and np.array_equal(col, col_o)
    # constraint couplings enlarge the plain element pattern
    rp0, _ = orc.sparsity(dm.n_dofs, dm.elem_dofs)
    assert rp[-1] > rp0[-1]


def test_refine_rejects_jittered_and_tet_meshes():
    L = _capi.lib()
    for et, jit in [(lm.HEX8, 0.1), (lm.TET4, 0.0)]:
        h = C.c_void_p()
        assert L.lmg_mesh_cube(2, 2, 2, et, jit, 0, C.byref(h)) == 0
        assert L.lmg_mesh_refine(h, 1, 0.5, 1) == _capi.ERR_ARG
        L.lmg_mesh_free(h)
