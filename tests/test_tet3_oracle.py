"""FEType{THIRD, HIERARCHIC} on TET14 (cubic hierarchic tets), CPU side:
the TET14 mesh (MeshBase::all_complete_order), its LAGRANGE map basis, the
host dof numbering and Dirichlet dofs against the oracle, and the oracle's
cubic shapes (fe_hierarchic_shape_3D.C:2361-2440) checked for cubic
reproduction and for H1 conformity across every interior face, which pins the
edge flips and the reversed listing of the edge dofs together."""
import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc

HIER3 = 3 | lm.HIERARCHIC
TET_EDGES = [(0, 1), (1, 2), (0, 2), (0, 3), (1, 3), (2, 3)]
TET_FACES = [(0, 2, 1), (0, 1, 3), (1, 2, 3), (2, 0, 3)]


def test_tet14_mesh_nodes_at_midpoints_and_centroids():
    m = lm.Mesh.build_cube(3, 3, 3, lm.TET14, jitter=0.2, seed=2)
    assert m.conn.shape == (162, 14)
    X = m.xyz[m.conn]
    for k, (a, b) in enumerate(TET_EDGES):
        np.testing.assert_allclose(X[:, 4 + k], (X[:, a] + X[:, b]) / 2, atol=1e-15)
    for f, (a, b, c) in enumerate([(0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3)]):
        np.testing.assert_allclose(X[:, 10 + f], (X[:, a] + X[:, b] + X[:, c]) / 3, atol=1e-15)
    # every node of the mesh is used and the elements share their edge and face nodes
    assert np.unique(m.conn).size == m.n_nodes
    for e in range(m.n_elem):
        assert orc.lib().orc_has_affine_map(lm.TET14, orc._p(np.ascontiguousarray(X[e]))) == 1


def test_tet14_lagrange_map_basis():
    """The 14 LAGRANGE TET14 shapes: Kronecker at the nodes, partition of
    unity, quadratic reproduction and gradients consistent with differences."""
    ref = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    nodes = np.vstack([ref, [(ref[a] + ref[b]) / 2 for a, b in TET_EDGES],
                       [ref[list(f)].mean(0) for f in [(0, 1, 2), (0, 1, 3), (1, 2, 3), (0, 2, 3)]]])
    phi, _ = orc.shapes(lm.TET14, 3, nodes)
    np.testing.assert_allclose(phi, np.eye(14), atol=1e-14)
    rng = np.random.default_rng(1)
    pts = rng.dirichlet([1, 1, 1, 1], 30)[:, :3]
    phi, dphi = orc.shapes(lm.TET14, 3, pts)
    np.testing.assert_allclose(phi.sum(0), 1.0, atol=1e-14)
    u = lambda P: 1 + P[:, 0] - 2 * P[:, 1] * P[:, 2] + 3 * P[:, 0] ** 2  # noqa: E731
    np.testing.assert_allclose(phi.T @ u(nodes), u(pts), atol=1e-13)
    np.testing.assert_allclose(dphi[0].T @ u(nodes), 1 + 6 * pts[:, 0], atol=1e-12)
    h = 1e-7
    for c in range(3):
        dp = np.zeros(3)
        dp[c] = h
        fd = (orc.shapes(lm.TET14, 3, pts + dp)[0] - orc.shapes(lm.TET14, 3, pts - dp)[0]) / (2 * h)
        np.testing.assert_allclose(dphi[c], fd, atol=1e-6)


@pytest.mark.parametrize("n,jit", [(2, 0.0), (3, 0.2)])
def test_cubic_tet_dofs_match_oracle(n, jit):
    m = lm.Mesh.build_cube(n, n, n, lm.TET14, jitter=jit, seed=4)
    dm = lm.DofMap(m, 1, fe_order=HIER3)
    ed, nd = orc.distribute_dofs_tet3(m.n_nodes, m.conn)
    assert nd == dm.n_dofs and np.array_equal(ed, dm.elem_dofs)
    # vertices 1, edges 2, faces 1 dof each, nothing interior
    conn = m.conn
    edges = {tuple(sorted((v[a], v[b]))) for v in conn[:, :4] for a, b in TET_EDGES}
    faces = {tuple(sorted(v[list(f)])) for v in conn[:, :4] for f in TET_FACES}
    n_vert = len(np.unique(conn[:, :4]))
    assert dm.n_dofs == n_vert + 2 * len(edges) + len(faces)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    c = orc.dirichlet_tet3(dm.elem_dofs, m.side_bid, [0, 1, 2, 3, 4, 5], dm.n_dofs)
    assert np.array_equal(c, dm.constrained)


def test_cubic_tet_shapes_reproduce_cubics():
    m = lm.Mesh.build_cube(2, 2, 2, lm.TET14, jitter=0.2, seed=3)
    rng = np.random.default_rng(0)
    pts = rng.dirichlet([1, 1, 1, 1], 60)[:, 1:]
    f = lambda p: 1 + p[:, 0] - 2 * p[:, 1] ** 2 + p[:, 0] * p[:, 1] * p[:, 2] + 3 * p[:, 2] ** 3  # noqa: E731
    for e in (0, 7, 31):
        phi, dphi = orc.shapes_tet3(m.xyz[m.conn[e]], pts)
        coef, *_ = np.linalg.lstsq(phi.T, f(pts), rcond=None)
        assert np.abs(phi.T @ coef - f(pts)).max() < 1e-13
        # the difference-quotient gradients follow the same combination
        gx = 1 + pts[:, 1] * pts[:, 2]
        assert np.abs(dphi[0].T @ coef - gx).max() < 1e-8


def test_cubic_tet_conformity_across_faces():
    """Each global dof's basis function has the same trace on a face from
    both elements that share it (continuity of the assembled space)."""
    m = lm.Mesh.build_cube(2, 2, 2, lm.TET14, jitter=0.25, seed=9)
    dm = lm.DofMap(m, 1, fe_order=HIER3)
    conn, X = m.conn, m.xyz
    owner = {}
    for e in range(m.n_elem):
        for f in TET_FACES:
            owner.setdefault(tuple(sorted(conn[e, list(f)])), []).append(e)
    rng = np.random.default_rng(3)
    bary = rng.dirichlet([1, 1, 1], 7)
    checked = 0
    for key, els in owner.items():
        if len(els) != 2:
            continue
        P = bary @ X[list(key)]  # physical points on the shared face
        traces = []
        for e in els:
            V = X[conn[e, :4]]
            J = (V[1:] - V[0]).T  # affine map x = V0 + J xi
            xi = np.linalg.solve(J, (P - V[0]).T).T
            phi, _ = orc.shapes_tet3(X[conn[e]], xi)
            traces.append({int(d): phi[i] for i, d in enumerate(dm.elem_dofs[e])})
        common = set(traces[0]) & set(traces[1])
        assert len(common) == 3 + 3 * 2 + 1  # the face's vertex, edge and face dofs
        for d in common:
            np.testing.assert_allclose(traces[0][d], traces[1][d], atol=1e-12)
        for t in traces:
            for d in set(t) - common:
                assert np.abs(t[d]).max() < 1e-12  # off-face dofs vanish on the face
        checked += 1
    assert checked > 50
