"""Mixed form (FP32 contraction, FP64 Jacobians / diagonal / accumulation) and the
device CG solve, against the FP64 drop-in and the oracle.

Bar (the benchmark spec's tolerance for the mixed form): relative error of the
CG-solved field <= 1e-6; reported alongside: relative Frobenius error of K and F."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import libmesh_gb300 as lm
import oracle as orc
from helpers import make_problem, oracle_assemble

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_c1_solve_against_oracle_direct_solve():
    """Poisson HEX8 32^3: GPU CG (FP64 and mixed K) against a direct solve of the oracle's K."""
    mesh, dm, k, f = make_problem(32, lm.HEX8, 1, lm.POISSON, coef=False, seed=0)
    asm = lm.GpuAssembly(lm.POISSON, 1, 2, nodal_f=f)
    asm.init(mesh, dm)
    rp, col = asm.sparsity()
    Kr, Fr, st, _ = oracle_assemble(lm.POISSON, mesh, dm, 1, 2, rp, col, None, f)
    u_ref = spla.spsolve(sp.csc_matrix(sp.csr_matrix((Kr, col, rp))), Fr)
    asm.assemble(lm.FP64)
    u64, it, rr = asm.solve(rtol=1e-12)
    assert rr <= 1e-12 and rel(u64, u_ref) < 1e-9
    K32, F32 = asm.assemble(lm.MIXED)
    u32, it, rr = asm.solve(rtol=1e-12)
    assert rel(K32, Kr) < 1e-6 and rel(F32, Fr) < 1e-14
    assert rel(u32, u_ref) < 1e-6
    asm.close()


@pytest.mark.parametrize("n", [6, 12])
def test_elasticity_mixed_field_error(n):
    mesh, dm, k, f = make_problem(n, lm.TET10, 3, lm.ELASTICITY, jitter=0.2, seed=1)
    asm = lm.GpuAssembly(lm.ELASTICITY, 2, 4, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    K64, F64 = asm.assemble(lm.FP64)
    u64, it64, rr64 = asm.solve(rtol=1e-12, maxit=50000)
    K32, F32 = asm.assemble(lm.MIXED)
    u32, it32, rr32 = asm.solve(rtol=1e-12, maxit=50000)
    assert rr64 <= 1e-12 and rr32 <= 1e-12
    assert rel(K32, K64) < 1e-6
    # the same double-float element loads, summed per dof in element order by
    # the same kernel in both forms
    assert np.array_equal(F32, F64)
    assert rel(u32, u64) < 1e-6, rel(u32, u64)
    asm.close()


def test_mixed_keeps_translations_in_the_kernel():
    """Without constraints the mixed K annihilates rigid translations to FP64
    roundoff (diagonal blocks are rebuilt from the stored off-diagonal blocks)."""
    mesh, dm, k, f = make_problem(5, lm.TET10, 3, lm.ELASTICITY, jitter=0.2, bids=[])
    asm = lm.GpuAssembly(lm.ELASTICITY, 2, 4, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    rp, col = asm.sparsity()
    K32, _ = asm.assemble(lm.MIXED)
    K64, _ = asm.assemble(lm.FP64)
    A32 = sp.csr_matrix((K32, col, rp))
    A64 = sp.csr_matrix((K64, col, rp))
    npe = 10
    comp = np.empty(dm.n_dofs, np.int64)
    for v in range(3):
        comp[dm.elem_dofs[:, v * npe:(v + 1) * npe].ravel()] = v
    scale = np.abs(K64).max()
    for v in range(3):
        t = (comp == v).astype(float)
        assert np.abs(A32 @ t).max() < 1e-13 * scale
        assert np.abs(A64 @ t).max() < 1e-13 * scale
    asm.close()


def test_mixed_poisson_hex27_and_general_path():
    mesh, dm, k, f = make_problem(3, lm.HEX27, 1, lm.POISSON)
    asm = lm.GpuAssembly(lm.POISSON, 2, 5, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    K64, _ = asm.assemble(lm.FP64)
    K32, _ = asm.assemble(lm.MIXED)
    assert rel(K32, K64) < 1e-6
    asm.close()
    mesh, dm, k, f = make_problem(4, lm.HEX8, 1, lm.POISSON, jitter=0.2)
    asm = lm.GpuAssembly(lm.POISSON, 1, 2, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    K64, _ = asm.assemble(lm.FP64)
    K32, _ = asm.assemble(lm.MIXED)
    assert rel(K32, K64) < 1e-6
    asm.close()
