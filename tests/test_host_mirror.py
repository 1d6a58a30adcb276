"""Host mirror of libMesh's setup (CPU): mesh generation, DofMap numbering,
Dirichlet dof sets and sparsity, bit-exact against the oracle's restatement."""
import ctypes as C

import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from libmesh_gb300._capi import lib, ptr

CASES = [(lm.HEX8, 1, 4), (lm.HEX27, 1, 3), (lm.TET4, 1, 3), (lm.TET10, 3, 3), (lm.TET10, 1, 2),
         (lm.HEX8, 3, 3), (lm.PRISM6, 1, 3), (lm.PRISM6, 3, 2)]


def host_sparsity(dm):
    nnz = C.c_int64()
    npe = dm.mesh.conn.shape[1]
    assert lib().lmg_host_sparsity(dm.mesh.n_elem, npe, dm.n_vars, dm.n_dofs, ptr(dm.elem_dofs),
                                   C.byref(nnz), None, None) == 0
    rp = np.empty(dm.n_dofs + 1, np.int32)
    col = np.empty(nnz.value, np.int32)
    assert lib().lmg_host_sparsity(dm.mesh.n_elem, npe, dm.n_vars, dm.n_dofs, ptr(dm.elem_dofs),
                                   C.byref(nnz), ptr(rp), ptr(col)) == 0
    return rp, col


@pytest.mark.parametrize("et,nv,n", CASES)
def test_dofs_and_sparsity_match_oracle(et, nv, n):
    m = lm.Mesh.build_cube(n, n, n, et, jitter=0.2 if et in (lm.TET4, lm.TET10) else 0.0, seed=1)
    dm = lm.DofMap(m, nv)
    ed, nd = orc.distribute_dofs(m.n_nodes, m.conn, nv)
    assert nd == dm.n_dofs == m.n_nodes * nv
    assert np.array_equal(ed, dm.elem_dofs)
    rp, col = orc.sparsity(nd, ed)
    rp2, col2 = host_sparsity(dm)
    assert np.array_equal(rp, rp2) and np.array_equal(col, col2)
    for r in range(nd):  # PETSc AIJ: strictly ascending columns per row
        assert np.all(np.diff(col2[rp2[r]:rp2[r + 1]]) > 0)


@pytest.mark.parametrize("et,nv,n", CASES)
def test_dirichlet_matches_oracle_and_geometry(et, nv, n):
    m = lm.Mesh.build_cube(n, n, n, et, jitter=0.2 if et in (lm.TET4, lm.TET10) else 0.0, seed=1)
    dm = lm.DofMap(m, nv)
    for bids in ([0, 1, 2, 3, 4, 5], [4], [0, 5]):
        c = np.zeros(dm.n_dofs, np.uint8)
        dm2 = lm.DofMap(m, nv)
        c = dm2.add_dirichlet_boundary(bids, list(range(nv)))
        co = orc.dirichlet(et, nv, dm.elem_dofs, m.side_bid, bids, list(range(nv)), dm.n_dofs)
        assert np.array_equal(c, co)
        # build_cube side ids: 0 z=0, 1 y=0, 2 x=1, 3 y=1, 4 x=0, 5 z=1
        face = {0: (2, 0.0), 1: (1, 0.0), 2: (0, 1.0), 3: (1, 1.0), 4: (0, 0.0), 5: (2, 1.0)}
        on = np.zeros(m.n_nodes, bool)
        for b in bids:
            d, v = face[b]
            on |= m.xyz[:, d] == v
        npe = m.conn.shape[1]
        node_of = np.empty(dm.n_dofs, np.int64)
        for v in range(nv):
            node_of[dm.elem_dofs[:, v * npe:(v + 1) * npe].ravel()] = m.conn.ravel()
        assert np.array_equal(c.astype(bool), on[node_of])


def test_tet_split_six_per_hex_positive_volume():
    m = lm.Mesh.build_cube(3, 2, 2, lm.TET4, jitter=0.2, seed=3)
    assert m.n_elem == 6 * 12
    X = m.xyz[m.conn]
    vol = np.einsum("ij,ij->i", X[:, 1] - X[:, 0], np.cross(X[:, 2] - X[:, 0], X[:, 3] - X[:, 0])) / 6
    assert np.all(vol > 0)
    assert abs(vol.sum() - 1.0) < 1e-13


def test_tet10_midpoints_and_affine():
    m = lm.Mesh.build_cube(3, 3, 3, lm.TET10, jitter=0.2, seed=1)
    X = m.xyz[m.conn]
    E = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
    for k, (a, b) in enumerate(E):
        np.testing.assert_array_equal(X[:, 4 + k], (X[:, a] + X[:, b]) / 2)
    assert all(orc.has_affine_map(lm.TET10, x) for x in X)


def test_first_touch_node_numbering():
    for et in (lm.HEX8, lm.HEX27, lm.TET10):
        m = lm.Mesh.build_cube(3, 2, 2, et, jitter=0.1 if et == lm.TET10 else 0.0, seed=1)
        seen, nxt = set(), 0
        for c in m.conn.ravel():
            if c not in seen:
                assert c == nxt
                seen.add(c)
                nxt += 1
        assert nxt == m.n_nodes


def test_hex_affine_and_distorted():
    m = lm.Mesh.build_cube(2, 2, 2, lm.HEX8)
    assert all(orc.has_affine_map(lm.HEX8, x) for x in m.xyz[m.conn])
    x = m.xyz[m.conn[0]].copy()
    x[6] += 0.05
    assert not orc.has_affine_map(lm.HEX8, x)
    m27 = lm.Mesh.build_cube(2, 2, 2, lm.HEX27)
    assert all(orc.has_affine_map(lm.HEX27, x) for x in m27.xyz[m27.conn])


def test_bad_arguments_are_errors():
    with pytest.raises(lm.LmgError):
        lm.Mesh.build_cube(0, 1, 1, lm.HEX8)
    with pytest.raises(lm.LmgError):
        lm.Mesh.build_cube(1, 1, 1, 99)
    conn = np.array([[0, 1, 2, 3, 4, 5, 6, 99]], np.int32)
    nd = C.c_int64()
    ed = np.empty((1, 8), np.int32)
    assert lib().lmg_dofmap_distribute(8, 1, 8, ptr(conn), 1, C.byref(nd), ptr(ed)) == 5


@pytest.mark.parametrize("rotate", [False, True])
def test_hier3_dofs_and_dirichlet_match_oracle(rotate):
    """FEType{THIRD, HIERARCHIC} on HEX27: per-node dof counts, element dofs,
    reversed non-vertex dofs, and the Dirichlet set, against the oracle."""
    from test_hier3_oracle import rotated_cube
    m = rotated_cube(3, 11) if rotate else lm.Mesh.build_cube(3, 3, 3, lm.HEX27)
    dm = lm.DofMap(m, 1, fe_order=3 | lm.HIERARCHIC)
    ed, nd = orc.distribute_dofs_hier3(m.n_nodes, m.conn)
    assert nd == dm.n_dofs and np.array_equal(ed, dm.elem_dofs)
    for bids in ([0, 1, 2, 3, 4, 5], [2], [0, 5]):
        c = lm.DofMap(m, 1, fe_order=3 | lm.HIERARCHIC).add_dirichlet_boundary(bids, [0])
        assert np.array_equal(c, orc.dirichlet_hier3(ed, m.side_bid, bids, nd))


@pytest.mark.parametrize("et,p", [(lm.PRISM18, 2), (lm.PRISM21, 3)])
def test_prism_dofs_and_dirichlet_match_oracle(et, p):
    """HIERARCHIC SECOND on PRISM18 and THIRD on PRISM21: per-node dof counts
    (edge, quad-face, triangle-face and interior nodes), element dofs with
    reversed non-vertex dofs, and the Dirichlet set, against the oracle."""
    m = lm.Mesh.build_cube(3, 2, 2, et)
    dm = lm.DofMap(m, 1, fe_order=p | lm.HIERARCHIC)
    ed, nd = orc.distribute_dofs_prism(p, m.n_nodes, m.conn)
    assert nd == dm.n_dofs and np.array_equal(ed, dm.elem_dofs)
    for bids in ([0, 1, 2, 3, 4, 5], [2], [0, 5], [1, 4]):
        c = lm.DofMap(m, 1, fe_order=p | lm.HIERARCHIC).add_dirichlet_boundary(bids, [0])
        assert np.array_equal(c, orc.dirichlet_prism(p, ed, m.side_bid, bids, nd))


@pytest.mark.parametrize("et,n,jit", [(lm.HEX8, 5, 0.0), (lm.HEX8, 4, 0.2), (lm.HEX27, 3, 0.0), (lm.TET4, 4, 0.2),
                                      (lm.TET10, 5, 0.2), (lm.TET10, 6, 0.0), (lm.TET10, 16, 0.2),
                                      (lm.PRISM18, 3, 0.0), (lm.PRISM21, 3, 0.0), (lm.PRISM21, 1, 0.0)])
def test_mesh_generation_matches_oracle(et, n, jit):
    """build_cube (+ all_tri, all_second_order) through the C ABI against the
    oracle's step-by-step restatement: coordinates, connectivity and side
    boundary ids bit for bit."""
    m = lm.Mesh.build_cube(n, n, n, et, jitter=jit, seed=1)
    xyz, conn, sb = orc.mesh_cube(n, et, jit, 1)
    assert np.array_equal(xyz, m.xyz)
    assert np.array_equal(conn, m.conn)
    assert np.array_equal(sb, m.side_bid)
