"""Matrix-free residual (lmg_residual): R = K u - F without forming K, against
the assembled GPU system and the oracle's K u - F (LinearImplicitSystem::assembly,
src/systems/linear_implicit_system.C:367-381).

Bar: |R - R_ref| <= 1e-12 (|K| |u| + |F|) per row (the products sum in a
different order than the assembled matrix's rows)."""
import numpy as np
import pytest
import scipy.sparse as sp

import libmesh_gb300 as lm
from helpers import make_problem, oracle_assemble

pytestmark = pytest.mark.gpu


def check(mesh, dm, form, fo, qo, k, f):
    asm = lm.GpuAssembly(form, fo, qo, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    rp, col = asm.sparsity()
    K, F = asm.assemble()
    u = np.random.default_rng(3).normal(size=dm.n_dofs)
    R = asm.residual(u)
    R2 = asm.residual(u)
    asm.close()
    assert np.array_equal(R, R2)                      # deterministic
    A = sp.csr_matrix((K, col, rp), shape=(dm.n_dofs, dm.n_dofs))
    absA = sp.csr_matrix((np.abs(K), col, rp), shape=(dm.n_dofs, dm.n_dofs))
    scale = absA @ np.abs(u) + np.abs(F)
    assert np.all(np.abs(R - (A @ u - F)) <= 1e-12 * scale)
    Kr, Fr, st, _ = oracle_assemble(form, mesh, dm, fo, qo, rp, col, k, f)
    assert st == 0
    Ar = sp.csr_matrix((Kr, col, rp), shape=(dm.n_dofs, dm.n_dofs))
    assert np.all(np.abs(R - (Ar @ u - Fr)) <= 1e-12 * scale)


@pytest.mark.parametrize("et,fo,qo,n", [(lm.HEX8, 1, 2, 5), (lm.HEX27, 2, 5, 3), (lm.TET10, 2, 4, 3),
                                        (lm.PRISM6, 1, 3, 4)])
def test_residual_poisson(et, fo, qo, n):
    mesh, dm, k, f = make_problem(n, et, 1, lm.POISSON, jitter=0.2 if et == lm.TET10 else 0.0)
    check(mesh, dm, lm.POISSON, fo, qo, k, f)


@pytest.mark.parametrize("et,fo,qo,n", [(lm.TET10, 2, 4, 4), (lm.HEX8, 1, 2, 3)])
def test_residual_elasticity(et, fo, qo, n):
    mesh, dm, k, f = make_problem(n, et, 3, lm.ELASTICITY, jitter=0.2 if et == lm.TET10 else 0.0)
    check(mesh, dm, lm.ELASTICITY, fo, qo, k, f)


def test_residual_refuses_nonaffine():
    mesh, dm, k, f = make_problem(3, lm.HEX8, 1, lm.POISSON, jitter=0.2)
    asm = lm.GpuAssembly(lm.POISSON, 1, 2, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    with pytest.raises(lm.LmgError):
        asm.residual(np.zeros(dm.n_dofs))
    asm.close()
