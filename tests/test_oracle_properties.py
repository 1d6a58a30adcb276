"""Analytic invariants of the oracle's assembled systems (CPU): the checks that
stand in for the golden K/F values no reference test holds."""
import numpy as np
import pytest
import scipy.sparse as sp

import libmesh_gb300 as lm
import oracle as orc
from helpers import make_problem, oracle_assemble


def assemble(n, et, nv, form, fo, qo, jitter=0.0, bids=None, coef=True):
    mesh, dm, k, f = make_problem(n, et, nv, form, jitter=jitter, bids=bids, coef=coef)
    rp, col = orc.sparsity(dm.n_dofs, dm.elem_dofs)
    K, F, st, _ = oracle_assemble(form, mesh, dm, fo, qo, rp, col, k, f)
    assert st == 0
    A = sp.csr_matrix((K, col, rp), shape=(dm.n_dofs, dm.n_dofs))
    return mesh, dm, A, F


@pytest.mark.parametrize("et,fo,qo,jit", [(lm.HEX8, 1, 2, 0.0), (lm.HEX27, 2, 5, 0.0), (lm.TET4, 1, 2, 0.2),
                                          (lm.TET10, 2, 4, 0.2)])
def test_laplacian_annihilates_affine_fields(et, fo, qo, jit):
    mesh, dm, A, _ = assemble(3, et, 1, lm.POISSON, fo, qo, jitter=jit, bids=[], coef=False)
    node_of = np.empty(dm.n_dofs, np.int64)
    node_of[dm.elem_dofs.ravel()] = mesh.conn.ravel()
    x = mesh.xyz[node_of]
    for u in (np.ones(dm.n_dofs), x[:, 0] - 2 * x[:, 1] + 0.5 * x[:, 2]):
        r = A @ u
        bnd = ((mesh.xyz[node_of] == 0) | (mesh.xyz[node_of] == 1)).any(1)
        scale = abs(A).max()
        if u.std() == 0:
            assert np.abs(r).max() < 1e-13 * scale * 10
        else:
            assert np.abs(r[~bnd]).max() < 1e-12 * scale
    assert abs(A - A.T).max() == 0.0  # dphi_i.dphi_j is symmetric operation by operation


def test_dirichlet_rows_and_diagonal_count():
    mesh, dm, A, F = assemble(3, lm.HEX8, 1, lm.POISSON, 1, 2)
    c = dm.constrained.astype(bool)
    A = A.tocsr()
    count = np.bincount(dm.elem_dofs.ravel(), minlength=dm.n_dofs)
    for d in np.nonzero(c)[0]:
        row = A.getrow(d)
        assert row.nnz > 0
        assert row[0, d] == count[d]          # one 1 per element touching the dof
        assert abs(row).sum() == count[d]
        assert F[d] == 0.0
    assert abs(A[:, np.nonzero(c)[0]][~c]).max() == 0.0


def test_elasticity_rigid_modes_and_symmetry():
    mesh, dm, A, _ = assemble(2, lm.TET10, 3, lm.ELASTICITY, 2, 4, jitter=0.2, bids=[])
    node_of = np.empty(dm.n_dofs, np.int64)
    comp = np.empty(dm.n_dofs, np.int64)
    npe = mesh.conn.shape[1]
    for v in range(3):
        node_of[dm.elem_dofs[:, v * npe:(v + 1) * npe].ravel()] = mesh.conn.ravel()
        comp[dm.elem_dofs[:, v * npe:(v + 1) * npe].ravel()] = v
    x = mesh.xyz[node_of]
    scale = abs(A).max()
    modes = []
    for v in range(3):
        modes.append((comp == v).astype(float))
    for (a, b) in [(0, 1), (1, 2), (2, 0)]:
        u = np.zeros(dm.n_dofs)
        u[comp == a] = -x[comp == a, b]
        u[comp == b] = x[comp == b, a]
        modes.append(u)
    for u in modes:
        assert np.abs(A @ u).max() < 1e-12 * scale
    assert abs(A - A.T).max() < 1e-15 * scale


def test_threaded_oracle_matches_serial():
    mesh, dm, k, f = make_problem(4, lm.TET10, 3, lm.ELASTICITY, jitter=0.2)
    rp, col = orc.sparsity(dm.n_dofs, dm.elem_dofs)
    K1, F1, _, _ = oracle_assemble(lm.ELASTICITY, mesh, dm, 2, 4, rp, col, k, f, n_threads=1)
    K4, F4, _, _ = oracle_assemble(lm.ELASTICITY, mesh, dm, 2, 4, rp, col, k, f, n_threads=4)
    np.testing.assert_allclose(K4, K1, rtol=1e-13, atol=1e-13 * abs(K1).max())
    np.testing.assert_allclose(F4, F1, rtol=1e-13, atol=1e-13 * abs(F1).max())


def test_degenerate_element_reported():
    mesh, dm, k, f = make_problem(2, lm.HEX8, 1, lm.POISSON, bids=[])
    xyz = mesh.xyz.copy()
    c = mesh.conn[3]
    xyz[c[6]] = xyz[c[0]]  # collapse one hex corner onto its opposite corner
    rp, col = orc.sparsity(dm.n_dofs, dm.elem_dofs)
    K, F, st, bad = orc.assemble(lm.POISSON, lm.HEX8, 1, 2, xyz, mesh.conn, 1, dm.elem_dofs, dm.n_dofs,
                                 dm.constrained, rp, col)
    assert st == 4 and bad >= 0
