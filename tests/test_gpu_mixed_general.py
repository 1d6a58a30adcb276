"""Mixed form on the general path (FP32 element contraction and constraint
products, FP64 map, FP64 global sums): hanging-node constrained Poisson and
convection-diffusion on refined HEX27, and cubic HIERARCHIC hexes and tets,
against the FP64 drop-in and the oracle.

Bar (the benchmark spec's tolerance for the mixed form): relative error of the
solved field <= 1e-6 (direct solves of the nonsymmetric convection-diffusion
systems, device CG for the symmetric ones); reported alongside: relative
Frobenius error of K and F."""
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

import libmesh_gb300 as lm
import oracle as orc

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def cd_params(seed=3, n_modes=8, kappa=1e-2):
    rng = np.random.default_rng(seed)
    p = [kappa, n_modes]
    for _ in range(n_modes):
        p += list(rng.uniform(-1, 1, 3)) + list(2 * np.pi * rng.uniform(-1.5, 1.5, 3)) + [rng.uniform(0, 2 * np.pi)]
    return np.array(p)


@pytest.mark.parametrize("form,n,cycles,seed", [(lm.POISSON, 4, 2, 2), (lm.ADVDIFF, 4, 2, 2), (lm.ADVDIFF, 3, 3, 11)])
def test_mixed_constrained_hex27(form, n, cycles, seed):
    m = lm.Mesh.build_refined_cube(n, lm.HEX27, cycles, 0.2, seed)
    dm = lm.DofMap(m, 1)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    dm.create_dof_constraints()
    rng = np.random.default_rng(seed)
    f = rng.uniform(-1, 1, (m.n_nodes, 1))
    k = np.exp(rng.normal(0, 0.5, m.n_elem))
    params = cd_params() if form == lm.ADVDIFF else None
    asm = lm.GpuAssembly(form, 2, 5, elem_coef=k, nodal_f=f, params=params)
    asm.init(m, dm)
    rp, ci = asm.sparsity()
    K64, F64 = asm.assemble(lm.FP64)
    K32, F32 = asm.assemble(lm.MIXED)
    K32b, F32b = asm.assemble(lm.MIXED)      # repeat: deterministic
    asm.close()
    assert np.array_equal(K32, K32b) and np.array_equal(F32, F32b)
    Kr, Fr, st, _ = orc.assemble(form, m.elem_type, 2, 5, m.xyz, m.conn, 1, dm.elem_dofs, dm.n_dofs, dm.constrained,
                                 rp, ci, coef=k, nodal_f=f, cons_rows=(dm.cons_ptr, dm.cons_col, dm.cons_val),
                                 params=params)
    assert st == 0
    n_d = dm.n_dofs
    u_ref = spla.spsolve(sp.csc_matrix(sp.csr_matrix((Kr, ci, rp), shape=(n_d, n_d))), Fr)
    u32 = spla.spsolve(sp.csc_matrix(sp.csr_matrix((K32, ci, rp), shape=(n_d, n_d))), F32)
    print("mixed general form %d: ||dK||/||K|| %.3g  ||dF||/||F|| %.3g  ||du||/||u|| %.3g"
          % (form, rel(K32, Kr), rel(F32, Fr), rel(u32, u_ref)))
    assert rel(K32, Kr) < 1e-6 and rel(F32, Fr) < 1e-6
    assert rel(u32, u_ref) <= 1e-6


@pytest.mark.parametrize("et,n", [(lm.HEX27, 3), (lm.TET14, 3)])
def test_mixed_cubic_hierarchic(et, n):
    m = lm.Mesh.build_cube(n, n, n, et)
    dm = lm.DofMap(m, 1, fe_order=3 | lm.HIERARCHIC)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    rng = np.random.default_rng(3)
    k = rng.uniform(0.1, 10.0, m.n_elem)
    f = rng.uniform(-1.0, 1.0, (m.n_nodes, 1))
    asm = lm.GpuAssembly(lm.POISSON, 3 | lm.HIERARCHIC, 7 if et == lm.HEX27 else 6, elem_coef=k, nodal_f=f)
    asm.init(m, dm)
    K64, F64 = asm.assemble(lm.FP64)
    u64, _, rr64 = asm.solve(rtol=1e-13, maxit=100000)
    K32, F32 = asm.assemble(lm.MIXED)
    u32, _, rr32 = asm.solve(rtol=1e-13, maxit=100000)
    asm.close()
    print("mixed cubic %d: ||dK||/||K|| %.3g  ||du||/||u|| %.3g" % (et, rel(K32, K64), rel(u32, u64)))
    assert rel(K32, K64) < 1e-6 and np.array_equal(F32, F64)
    assert rel(u32, u64) <= 1e-6
