"""Pins the CPU oracle to the reference's own known-answer tests (CPU only).

  tests/quadrature/quadrature_test.C  QGauss integrates monomials up to its order exactly
  tests/fe/fe_test.h                  LAGRANGE shapes reproduce polynomial fields, partition of unity
  tests/mesh/mesh_generation_test.C   build_cube element / node counts
  tests/geom/volume_test.C            element volumes (here: sum of JxW through the load vector)
"""
import math

import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from helpers import make_problem, oracle_assemble


def hex_exact(i, j, k):
    e = lambda p: 0.0 if p % 2 else 2.0 / (p + 1)
    return e(i) * e(j) * e(k)


def tet_exact(i, j, k):
    return math.factorial(i) * math.factorial(j) * math.factorial(k) / math.factorial(i + j + k + 3)


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5, 6, 7, 8, 9])
def test_qgauss_hex_monomials(order):
    pts, w = orc.qgauss(lm.HEX8, order)
    assert len(w) == (order // 2 + 1) ** 3
    for i in range(order + 1):
        for j in range(order + 1):
            for k in range(order + 1):
                val = np.sum(w * pts[:, 0] ** i * pts[:, 1] ** j * pts[:, 2] ** k)
                assert abs(val - hex_exact(i, j, k)) < 1e-14


@pytest.mark.parametrize("order,npts", [(1, 1), (2, 4), (3, 5), (4, 11), (5, 14), (6, 24)])
def test_qgauss_tet_monomials(order, npts):
    pts, w = orc.qgauss(lm.TET10, order)
    assert len(w) == npts
    if order == 4:  # the Keast rule carries one negative weight
        assert (w < 0).sum() == 1
    for i in range(order + 1):
        for j in range(order + 1 - i):
            for k in range(order + 1 - i - j):
                val = np.sum(w * pts[:, 0] ** i * pts[:, 1] ** j * pts[:, 2] ** k)
                assert abs(val - tet_exact(i, j, k)) < 1e-15


def prism_exact(i, j, k):
    return (math.factorial(i) * math.factorial(j) / math.factorial(i + j + 2)) * (0.0 if k % 2 else 2.0 / (k + 1))


@pytest.mark.parametrize("order,npts", [(1, 1 * 1), (2, 3 * 2), (3, 4 * 2), (4, 6 * 3), (5, 7 * 3)])
def test_qgauss_prism_monomials(order, npts):
    """Prism QGauss = triangle rule x 1-D Gauss rule (quadrature_gauss_3D.C:507-525):
    exact for x^i y^j z^k with i + j <= order and k <= order."""
    pts, w = orc.qgauss(lm.PRISM6, order)
    assert len(w) == npts
    for i in range(order + 1):
        for j in range(order + 1 - i):
            for k in range(order + 1):
                val = np.sum(w * pts[:, 0] ** i * pts[:, 1] ** j * pts[:, 2] ** k)
                assert abs(val - prism_exact(i, j, k)) < 1e-15


REF_NODES = {
    lm.HEX8: np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                       [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], float),
    lm.TET4: np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float),
}
_t = REF_NODES[lm.TET4]
REF_NODES[lm.TET10] = np.vstack([_t, (_t[[0, 1, 0, 0, 1, 2]] + _t[[1, 2, 2, 3, 3, 3]]) / 2])
_h = REF_NODES[lm.HEX8]
_e = [(0, 1), (1, 2), (2, 3), (3, 0), (0, 4), (1, 5), (2, 6), (3, 7), (4, 5), (5, 6), (6, 7), (7, 4)]
_f = [(0, 1, 2, 3), (0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (3, 0, 4, 7), (4, 5, 6, 7)]
REF_NODES[lm.PRISM6] = np.array([[0, 0, -1], [1, 0, -1], [0, 1, -1], [0, 0, 1], [1, 0, 1], [0, 1, 1]], float)
REF_NODES[lm.HEX27] = np.vstack([_h, [(_h[a] + _h[b]) / 2 for a, b in _e],
                                 [_h[list(f)].mean(0) for f in _f], [[0, 0, 0]]])


@pytest.mark.parametrize("et,order", [(lm.HEX8, 1), (lm.HEX27, 2), (lm.TET4, 1), (lm.TET10, 2), (lm.PRISM6, 1)])
def test_lagrange_reproduces_polynomials(et, order):
    rng = np.random.default_rng(5)
    if et in (lm.HEX8, lm.HEX27):
        pts = rng.uniform(-1, 1, (20, 3))
    else:
        pts = rng.dirichlet([1, 1, 1, 1], 20)[:, :3]
    if et == lm.PRISM6:
        pts = np.column_stack([rng.dirichlet(np.ones(3), 20)[:, 1:], rng.uniform(-1, 1, 20)])
    phi, dphi = orc.shapes(et, order, pts)
    X = REF_NODES[et]
    assert phi.shape[0] == len(X)
    np.testing.assert_allclose(phi.sum(0), 1.0, atol=1e-14)        # partition of unity
    np.testing.assert_allclose(dphi.sum(1), 0.0, atol=1e-13)
    # Kronecker property at the nodes
    pn, _ = orc.shapes(et, order, X)
    np.testing.assert_allclose(pn, np.eye(len(X)), atol=1e-14)
    # exact reproduction of every monomial of total degree <= order and its gradient
    for i in range(order + 1):
        for j in range(order + 1 - i):
            for k in range(order + 1 - i - j):
                u = lambda P: P[:, 0] ** i * P[:, 1] ** j * P[:, 2] ** k
                np.testing.assert_allclose(phi.T @ u(X), u(pts), atol=1e-13)
                gx = i * pts[:, 0] ** max(i - 1, 0) * pts[:, 1] ** j * pts[:, 2] ** k
                np.testing.assert_allclose(dphi[0].T @ u(X), gx, atol=1e-12)


@pytest.mark.parametrize("et,n,ne,nn", [(lm.HEX8, 3, 27, 64), (lm.HEX27, 2, 8, 125),
                                        (lm.TET4, 2, 48, 27), (lm.TET10, 2, 48, 125),
                                        (lm.TET10, 48, 663552, 912673), (lm.TET14, 2, 48, 245),
                                        (lm.PRISM6, 3, 54, 64)])
def test_build_cube_counts(et, n, ne, nn):
    m = lm.Mesh.build_cube(n, n, n, et, jitter=0.2 if et in (lm.TET4, lm.TET10) else 0.0, seed=1)
    assert (m.n_elem, m.n_nodes) == (ne, nn)


@pytest.mark.parametrize("et,nv,form,fo,qo", [(lm.HEX8, 1, lm.POISSON, 1, 2), (lm.HEX27, 1, lm.POISSON, 2, 5),
                                              (lm.TET4, 1, lm.POISSON, 1, 2), (lm.TET10, 3, lm.ELASTICITY, 2, 4),
                                              (lm.PRISM6, 1, lm.POISSON, 1, 3), (lm.PRISM6, 3, lm.ELASTICITY, 1, 2)])
def test_oracle_volume_through_load(et, nv, form, fo, qo):
    """Sum of F for f = 1 per component is the domain volume per component
    (partition of unity), for jittered meshes too."""
    mesh, dm, k, _ = make_problem(3, et, nv, form, jitter=0.15 if et in (lm.TET4, lm.TET10, lm.PRISM6) else 0.0,
                                  bids=[])
    rp, col = orc.sparsity(dm.n_dofs, dm.elem_dofs)
    f = np.ones((mesh.n_nodes, nv))
    K, F, st, _ = oracle_assemble(form, mesh, dm, fo, qo, rp, col, k, f)
    assert st == 0
    for v in range(nv):
        sel = dm.elem_dofs[:, v * mesh.conn.shape[1]:(v + 1) * mesh.conn.shape[1]]
        assert abs(F[np.unique(sel)].sum() - 1.0) < 1e-13


@pytest.mark.parametrize("et,order", [(10, 1), (12, 2), (8, 1), (9, 2), (13, 1)])
def test_hierarchic_shapes_span_the_lagrange_space(et, order):
    """HIERARCHIC hex (tet) shapes of order p lie in Q_p (P_p) (fe_hierarchic_test.C checks
    reproduction of polynomial fields): each equals the LAGRANGE interpolant of
    its nodal values, and its central-difference derivative (eps = 1e-6) equals
    the interpolant's exact derivative to the difference error."""
    rng = np.random.default_rng(0)
    nodes = orc.shapes(et, order, np.zeros((1, 3)))[0].shape[0]
    lag_nodes = {10: np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1], [-1, -1, 1], [1, -1, 1], [1, 1, 1],
                               [-1, 1, 1]], float)}
    if et == 12:
        off = [[0, 0, 0], [2, 0, 0], [2, 2, 0], [0, 2, 0], [0, 0, 2], [2, 0, 2], [2, 2, 2], [0, 2, 2], [1, 0, 0],
               [2, 1, 0], [1, 2, 0], [0, 1, 0], [0, 0, 1], [2, 0, 1], [2, 2, 1], [0, 2, 1], [1, 0, 2], [2, 1, 2],
               [1, 2, 2], [0, 1, 2], [1, 1, 0], [1, 0, 1], [2, 1, 1], [1, 2, 1], [0, 1, 1], [1, 1, 2], [1, 1, 1]]
        lag_nodes[12] = np.array(off, float) - 1.0
    tv = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1]], float)
    lag_nodes[8] = tv
    lag_nodes[9] = np.vstack([tv, 0.5 * (tv[[0, 1, 2, 0, 1, 2]] + tv[[1, 2, 0, 3, 3, 3]])])
    lag_nodes[13] = REF_NODES[lm.PRISM6]
    X = lag_nodes[et]
    pts = rng.uniform(-1, 1, (20, 3))
    if et in (8, 9):
        pts = rng.dirichlet(np.ones(4), 20)[:, 1:]
    if et == 13:
        pts = np.column_stack([rng.dirichlet(np.ones(3), 20)[:, 1:], rng.uniform(-1, 1, 20)])
    hv, hd = orc.shapes(et, order | 0x100, pts)
    hn, _ = orc.shapes(et, order | 0x100, X)          # hierarchic values at the Lagrange nodes
    lv, ld = orc.shapes(et, order, pts)
    assert hv.shape[0] == nodes
    np.testing.assert_allclose(hv, hn @ lv, atol=1e-14)
    for c in range(3):
        np.testing.assert_allclose(hd[c], hn @ ld[c], atol=1e-9)
