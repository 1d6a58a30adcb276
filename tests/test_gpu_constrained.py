"""Constrained / convection-diffusion assembly on the GPU (general path:
full element matrices, C^T K C with hanging-node rows, slot gather) against
the oracle's literal restatement of constrain_element_matrix_and_vector.
Bar: |K - K_ref| <= 1e-13 max(|K_ref|, row max), the same for F; CSR
pattern identical to the oracle's compute_sparsity with find_connected_dofs."""
import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from helpers import csr_rows, k_tolerance

pytestmark = pytest.mark.gpu


def cd_params(seed=3, n_modes=8, kappa=1e-2):
    """Transport velocity b = curl sum_m a_m sin(k_m . x + phase_m)."""
    rng = np.random.default_rng(seed)
    p = [kappa, n_modes]
    for _ in range(n_modes):
        p += list(rng.uniform(-1, 1, 3)) + list(2 * np.pi * rng.uniform(-1.5, 1.5, 3)) + [rng.uniform(0, 2 * np.pi)]
    return np.array(p)


def problem(n, et, cycles, seed, dirichlet=True):
    m = lm.Mesh.build_refined_cube(n, et, cycles, 0.2, seed) if cycles else lm.Mesh.build_cube(n, n, n, et)
    dm = lm.DofMap(m, 1)
    if dirichlet:
        dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    dm.create_dof_constraints()
    rng = np.random.default_rng(seed)
    f = rng.uniform(-1, 1, (m.n_nodes, 1))
    k = np.exp(rng.normal(0, 0.5, m.n_elem))
    return m, dm, k, f


def run(form, m, dm, k, f, fo, qo, params=None):
    asm = lm.GpuAssembly(form, fo, qo, elem_coef=k, nodal_f=f, params=params)
    asm.init(m, dm)
    rp, ci = asm.sparsity()
    assert asm.sparsity_on_device()  # find_connected_dofs on the device (compared with the oracle's below)
    K, F = asm.assemble()
    K2, F2 = asm.assemble()      # repeat: deterministic
    asm.close()
    rows = None if dm.cons_ptr is None else (dm.cons_ptr, dm.cons_col, dm.cons_val)
    Kr, Fr, st, _ = orc.assemble(form, m.elem_type, fo, qo, m.xyz, m.conn, 1, dm.elem_dofs, dm.n_dofs,
                                 dm.constrained, rp, ci, coef=k, nodal_f=f, cons_rows=rows, params=params)
    assert st == 0
    return rp, ci, K, F, K2, F2, Kr, Fr


CASES = [  # (form, elem, n, cycles, seed, fe_order, q_order)
    (lm.POISSON, lm.HEX27, 3, 2, 2, 2, 5),
    (lm.ADVDIFF, lm.HEX27, 3, 2, 2, 2, 5),
    (lm.ADVDIFF, lm.HEX27, 2, 3, 11, 2, 5),
    (lm.POISSON, lm.HEX8, 3, 3, 5, 1, 3),
    (lm.ADVDIFF, lm.HEX8, 4, 2, 9, 1, 4),
    (lm.ADVDIFF, lm.HEX27, 4, 0, 1, 2, 5),     # unrefined: convection form alone
]


@pytest.mark.parametrize("form,et,n,cycles,seed,fo,qo", CASES)
def test_constrained_assembly_matches_oracle(form, et, n, cycles, seed, fo, qo):
    m, dm, k, f = problem(n, et, cycles, seed)
    params = cd_params() if form == lm.ADVDIFF else None
    rp, ci, K, F, K2, F2, Kr, Fr = run(form, m, dm, k, f, fo, qo, params)
    rp_o, ci_o = orc.sparsity_constrained(dm.n_dofs, dm.elem_dofs, dm.cons_ptr, dm.cons_col)
    assert np.array_equal(rp, rp_o) and np.array_equal(ci, ci_o)
    assert np.array_equal(K, K2) and np.array_equal(F, F2)
    tol = k_tolerance(Kr, rp)
    assert np.all(np.abs(K - Kr) <= tol), np.max(np.abs(K - Kr) / np.maximum(tol, 1e-300))
    ftol = 1e-13 * max(np.abs(Fr).max(), 1e-300)
    assert np.all(np.abs(F - Fr) <= np.maximum(1e-13 * np.abs(Fr), ftol))


def test_constrained_rows_hold_the_constraint():
    """Constrained rows: 1 on the diagonal, -c at the constraining dofs
    (asymmetric constraint rows), times the number of elements that touch the dof."""
    m, dm, k, f = problem(3, lm.HEX27, 2, 2)
    rp, ci, K, F, *_ = run(lm.POISSON, m, dm, k, f, 2, 5)
    r = csr_rows(rp)
    cnt = np.bincount(dm.elem_dofs.reshape(-1), minlength=dm.n_dofs)
    for d in np.nonzero(np.diff(dm.cons_ptr) > 0)[0][:200]:
        row = dict(zip(ci[rp[d]:rp[d + 1]], K[rp[d]:rp[d + 1]]))
        assert abs(row[d] - cnt[d]) < 1e-12
        for j, c in zip(dm.cons_col[dm.cons_ptr[d]:dm.cons_ptr[d + 1]], dm.cons_val[dm.cons_ptr[d]:dm.cons_ptr[d + 1]]):
            assert abs(row[j] + c * cnt[d]) < 1e-12 * cnt[d]
        assert F[d] == 0.0
    assert len(r) == len(K)


def test_constant_is_in_the_kernel_without_dirichlet():
    """K 1 = 0 for the hanging-node constrained Laplacian and convection-diffusion
    operators (constants lie in the constrained space)."""
    for form in (lm.POISSON, lm.ADVDIFF):
        m, dm, k, f = problem(3, lm.HEX27, 2, 4, dirichlet=False)
        rp, ci, K, *_ = run(form, m, dm, k, f, 2, 5, cd_params() if form == lm.ADVDIFF else None)
        r = csr_rows(rp)
        s = np.bincount(r, weights=K, minlength=dm.n_dofs)
        scale = np.maximum.reduceat(np.abs(K), rp[:-1])
        assert np.all(np.abs(s) <= 1e-11 * scale)
