"""Cubic HIERARCHIC hexes (FEType{THIRD, HIERARCHIC} on HEX27) in the oracle (CPU).

The reference's fe_hierarchic_test.C checks that projected polynomial fields
are reproduced; the orientation logic of cube_indices exists so that shapes
of neighbouring elements agree on shared edges and faces whatever their local
node order.  Both are checked here on build_cube meshes whose elements are
given random proper rotations of their local node order:
  * the 64 shapes of every element span the tensor cubics Q3;
  * a global field sum_i u_i phi_i is continuous across every interior face
    of build_cube; with rotated elements the vertex and edge dofs stay
    continuous and the face dofs' traces span the same space;
  * dof counts and the Dirichlet set follow the per-node dof counts."""
import itertools

import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc

# tensor position of each HEX27 node: 0 -> -1, 1 -> +1, 2 -> 0
H27_I = np.array([
    [0, 1, 1, 0, 0, 1, 1, 0, 2, 1, 2, 0, 0, 1, 1, 0, 2, 1, 2, 0, 2, 2, 1, 2, 0, 2, 2],
    [0, 0, 1, 1, 0, 0, 1, 1, 0, 2, 1, 2, 0, 0, 1, 1, 0, 2, 1, 2, 2, 0, 2, 1, 2, 2, 2],
    [0, 0, 0, 0, 1, 1, 1, 1, 0, 0, 0, 0, 2, 2, 2, 2, 1, 1, 1, 1, 0, 2, 2, 2, 2, 1, 2]]).T
REF = np.where(H27_I == 0, -1.0, np.where(H27_I == 1, 1.0, 0.0))
H27_SIDES = [[0, 3, 2, 1, 11, 10, 9, 8, 20], [0, 1, 5, 4, 8, 13, 16, 12, 21], [1, 2, 6, 5, 9, 14, 17, 13, 22],
             [2, 3, 7, 6, 10, 15, 18, 14, 23], [3, 0, 4, 7, 11, 12, 19, 15, 24], [4, 5, 6, 7, 16, 17, 18, 19, 25]]


def rotations():
    out = []
    for perm in itertools.permutations(range(3)):
        for signs in itertools.product([-1, 1], repeat=3):
            R = np.zeros((3, 3))
            for r, (c, s) in enumerate(zip(perm, signs)):
                R[r, c] = s
            if np.linalg.det(R) > 0:
                out.append(R)
    return out


def rotated_cube(n, seed):
    """build_cube(n, n, n, HEX27) with every element's local node order rotated
    by a random proper cube rotation (the cells stay the same); side ids
    recomputed from the geometry."""
    m = lm.Mesh.build_cube(n, n, n, lm.HEX27)
    rng = np.random.default_rng(seed)
    rots = rotations()
    key = {tuple(p): a for a, p in enumerate(REF.astype(int))}
    conn = m.conn.copy()
    for e in range(m.n_elem):
        R = rots[rng.integers(len(rots))]
        conn[e] = [m.conn[e, key[tuple((R @ REF[a]).astype(int))]] for a in range(27)]
    sb = -np.ones((m.n_elem, 6), np.int8)
    face = {0: (2, 0.0), 1: (1, 0.0), 2: (0, 1.0), 3: (1, 1.0), 4: (0, 0.0), 5: (2, 1.0)}
    for e in range(m.n_elem):
        for s, nodes in enumerate(H27_SIDES):
            P = m.xyz[conn[e, nodes]]
            for b, (d, v) in face.items():
                if np.all(P[:, d] == v):
                    sb[e, s] = b
    return lm.Mesh(m.xyz, conn, lm.HEX27, sb)


def affine_map(X):
    """x(xi) = X0 + A (xi + 1) for an affine hex with local nodes X [27][3]."""
    A = np.column_stack([(X[1] - X[0]) / 2, (X[3] - X[0]) / 2, (X[4] - X[0]) / 2])
    return X[0], A


def test_hier3_shapes_span_q3():
    m = rotated_cube(1, 3)
    X = m.xyz[m.conn[0]]
    rng = np.random.default_rng(1)
    pts = rng.uniform(-1, 1, (100, 3))
    phi, _ = orc.shapes_hier3(X, pts)
    assert np.linalg.matrix_rank(phi, tol=1e-10) == 64
    # a random tensor cubic lies in their span
    c = rng.normal(size=(4, 4, 4))
    u = np.einsum("ijk,pi,pj,pk->p", c, *[np.stack([pts[:, d] ** i for i in range(4)], 1) for d in range(3)])
    coef, *_ = np.linalg.lstsq(phi.T, u, rcond=None)
    assert np.abs(phi.T @ coef - u).max() < 1e-11


def test_hier3_dof_counts_and_dirichlet():
    n = 2
    m = rotated_cube(n, 4)
    ed, nd = orc.distribute_dofs_hier3(m.n_nodes, m.conn)
    g = 2 * n + 1
    n_vert, n_edge = (n + 1) ** 3, 3 * n * (n + 1) ** 2
    n_face = 3 * n * n * (n + 1)
    assert nd == n_vert + 2 * n_edge + 4 * n_face + 8 * n ** 3
    assert ed.shape == (m.n_elem, 64) and len(np.unique(ed)) == nd and m.n_nodes == g ** 3
    for e in range(m.n_elem):
        assert len(np.unique(ed[e])) == 64
    c = orc.dirichlet_hier3(ed, m.side_bid, [0, 1, 2, 3, 4, 5], nd)
    # interior dofs: 8 per element, interior edges / faces / vertices of the grid
    interior = (n - 1) ** 3 + 2 * 3 * (n - 1) ** 2 * n + 4 * 3 * (n - 1) * n * n + 8 * n ** 3
    assert nd - int(c.sum()) == interior


def shared_face_traces(m, ed, rng):
    """For every interior face: the two elements, the sample points' shape
    values on each side [64][np], and the shared global dofs."""
    owners = {}
    for e in range(m.n_elem):
        for a in range(20, 26):
            owners.setdefault(m.conn[e, a], []).append(e)
    for node, els in owners.items():
        if len(els) != 2:
            continue
        c = m.xyz[node]
        X0 = m.xyz[m.conn[els[0]]]
        d = [k for k in range(3) if np.all(X0[:, k] >= c[k]) or np.all(X0[:, k] <= c[k])][0]
        P = np.tile(c, (8, 1))
        for k in range(3):
            if k != d:
                P[:, k] += rng.uniform(-0.25, 0.25, 8)
        phis = []
        for e in els:
            X = m.xyz[m.conn[e]]
            x0, A = affine_map(X)
            xi = np.linalg.solve(A, (P - x0).T).T - 1.0
            assert np.all(np.abs(xi) <= 1 + 1e-12)
            phis.append(orc.shapes_hier3(X, xi)[0])
        yield els, phis, sorted(set(ed[els[0]]) & set(ed[els[1]]))


def test_hier3_global_field_is_continuous_on_build_cube():
    m = lm.Mesh.build_cube(2, 2, 2, lm.HEX27)
    ed, nd = orc.distribute_dofs_hier3(m.n_nodes, m.conn)
    u = np.random.default_rng(2).normal(size=nd)
    n_faces = 0
    for els, phis, _ in shared_face_traces(m, ed, np.random.default_rng(3)):
        v = [phi.T @ u[ed[e]] for e, phi in zip(els, phis)]
        assert np.abs(v[0] - v[1]).max() < 1e-12 * np.abs(u).max()
        n_faces += 1
    assert n_faces == 3 * 2 * 2


@pytest.mark.parametrize("seed", [5, 6, 7])
def test_hier3_traces_on_rotated_elements(seed):
    """Rotated local node orders: every vertex and edge dof has the same trace
    from both sides of a face.  The face dofs' traces span the same space from
    both sides; which face function a dof is depends on cube_indices' case
    table, and the reference's table pairs some face cases (e.g. face 1 with
    its minimum at node 4) so that a dof's two traces differ by a swap of the
    in-face axes or a sign -- the restatement keeps that."""
    m = rotated_cube(2, seed)
    ed, nd = orc.distribute_dofs_hier3(m.n_nodes, m.conn)
    for els, phis, shared in shared_face_traces(m, ed, np.random.default_rng(seed)):
        loc = [{g: i for i, g in enumerate(ed[e])} for e in els]
        face = []
        for g in shared:
            i0, i1 = loc[0][g], loc[1][g]
            assert (i0 < 32) == (i1 < 32)
            if i0 < 32:
                assert np.abs(phis[0][i0] - phis[1][i1]).max() < 1e-13
            else:
                face.append((i0, i1))
        assert len(face) == 4
        A = np.array([phis[0][i] for i, _ in face])
        B = np.array([phis[1][j] for _, j in face])
        coef, *_ = np.linalg.lstsq(A.T, B.T, rcond=None)
        assert np.abs(A.T @ coef - B.T).max() < 1e-12
        assert np.allclose(np.abs(coef), np.round(np.abs(coef)), atol=1e-9)  # a signed permutation
