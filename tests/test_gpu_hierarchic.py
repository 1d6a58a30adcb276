"""HIERARCHIC hex, tet and prism elements (FEType{FIRST/SECOND, HIERARCHIC}) on the GPU:
FP64 drop-in Poisson on the symmetric block path and convection-diffusion on
the general path, against the oracle's restatement of
fe_hierarchic_3D_shape / cube_indices / fe_fdm_deriv.
Bar: |K - K_ref| <= 1e-13 max(|K_ref|, row max); F likewise."""
import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from helpers import k_tolerance

pytestmark = pytest.mark.gpu


def check(form, m, dm, k, f, fo, qo, params=None):
    asm = lm.GpuAssembly(form, fo | lm.HIERARCHIC, qo, elem_coef=k, nodal_f=f, params=params)
    asm.init(m, dm)
    rp, ci = asm.sparsity()
    K, F = asm.assemble()
    asm.close()
    Kr, Fr, st, _ = orc.assemble(form, m.elem_type, fo | 0x100, qo, m.xyz, m.conn, 1, dm.elem_dofs, dm.n_dofs,
                                 dm.constrained, rp, ci, coef=k, nodal_f=f, params=params)
    assert st == 0
    tol = k_tolerance(Kr, rp)
    assert np.all(np.abs(K - Kr) <= tol), np.max(np.abs(K - Kr) / np.maximum(tol, 1e-300))
    ftol = 1e-13 * np.abs(Fr).max()
    assert np.all(np.abs(F - Fr) <= np.maximum(1e-13 * np.abs(Fr), ftol))
    return K, Kr


def problem(n, et, jitter=0.0, seed=3):
    m = lm.Mesh.build_cube(n, n, n, et, jitter=jitter, seed=seed)
    dm = lm.DofMap(m, 1)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    rng = np.random.default_rng(seed)
    return m, dm, np.exp(rng.normal(0, 0.5, m.n_elem)), rng.uniform(-1, 1, (m.n_nodes, 1))


@pytest.mark.parametrize("et,fo,qo,n,jit", [(lm.HEX8, 1, 3, 6, 0.0), (lm.HEX8, 1, 3, 5, 0.2),
                                           (lm.HEX27, 2, 5, 4, 0.0), (lm.TET4, 1, 2, 4, 0.2),
                                           (lm.TET10, 2, 4, 3, 0.0), (lm.TET10, 2, 4, 3, 0.2),
                                           (lm.PRISM6, 1, 3, 4, 0.0), (lm.PRISM6, 1, 3, 3, 0.2)])
def test_hierarchic_poisson_matches_oracle(et, fo, qo, n, jit):
    m, dm, k, f = problem(n, et, jit)
    check(lm.POISSON, m, dm, k, f, fo, qo)


def test_hierarchic_convection_diffusion_matches_oracle():
    from test_gpu_constrained import cd_params
    m, dm, k, f = problem(4, lm.HEX27)
    dm.create_dof_constraints()
    check(lm.ADVDIFF, m, dm, k, f, 2, 5, cd_params())


def test_hierarchic_differs_from_lagrange_but_shares_the_pattern():
    """SECOND HIERARCHIC spans the same space as SECOND LAGRANGE on HEX27 with a
    different basis: same sparsity, different entries."""
    m, dm, k, f = problem(3, lm.HEX27)
    out = []
    for fo in (2, 2 | lm.HIERARCHIC):
        asm = lm.GpuAssembly(lm.POISSON, fo, 5, elem_coef=k, nodal_f=f)
        asm.init(m, dm)
        out.append((asm.sparsity(), asm.assemble()[0]))
        asm.close()
    (rp0, c0), K0 = out[0]
    (rp1, c1), K1 = out[1]
    assert np.array_equal(rp0, rp1) and np.array_equal(c0, c1)
    assert np.abs(K0 - K1).max() > 1e-3


@pytest.mark.parametrize("rotate,qo,n", [(False, 7, 3), (True, 7, 3), (True, 6, 2)])
def test_hierarchic_cubic_hex_matches_oracle(rotate, qo, n):
    """FEType{THIRD, HIERARCHIC} on HEX27 (64 dofs per element): per-element
    shape variants from cube_indices' edge / face orientation, elements with
    randomly rotated local node order, homogeneous Dirichlet on every side."""
    from test_hier3_oracle import rotated_cube
    m = rotated_cube(n, 21) if rotate else lm.Mesh.build_cube(n, n, n, lm.HEX27)
    dm = lm.DofMap(m, 1, fe_order=3 | lm.HIERARCHIC)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    rng = np.random.default_rng(8)
    k = np.exp(rng.normal(0, 0.5, m.n_elem))
    f = rng.uniform(-1, 1, (m.n_nodes, 1))
    asm = lm.GpuAssembly(lm.POISSON, 3 | lm.HIERARCHIC, qo, elem_coef=k, nodal_f=f)
    asm.init(m, dm)
    rp, ci = asm.sparsity()
    K, F = asm.assemble()
    asm.close()
    rpo, cio = orc.sparsity(dm.n_dofs, dm.elem_dofs)
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    Kr, Fr, st, _ = orc.assemble(lm.POISSON, m.elem_type, 3 | 0x100, qo, m.xyz, m.conn, 1, dm.elem_dofs, dm.n_dofs,
                                 dm.constrained, rp, ci, coef=k, nodal_f=f)
    assert st == 0
    tol = k_tolerance(Kr, rp)
    assert np.all(np.abs(K - Kr) <= tol), np.max(np.abs(K - Kr) / np.maximum(tol, 1e-300))
    ftol = 1e-13 * np.abs(Fr).max()
    assert np.all(np.abs(F - Fr) <= np.maximum(1e-13 * np.abs(Fr), ftol))


@pytest.mark.parametrize("n,jit,qo", [(2, 0.0, 6), (3, 0.25, 6), (3, 0.1, 5)])
def test_hierarchic_cubic_tet_matches_oracle(n, jit, qo):
    """FEType{THIRD, HIERARCHIC} on TET14 (20 dofs per element): the order-3
    edge bases flipped by positive_edge_orientation and the face bubbles
    multiplied in orient_triangle's order, per element; homogeneous Dirichlet
    on every side; QGauss SIXTH / FIFTH."""
    m = lm.Mesh.build_cube(n, n, n, lm.TET14, jitter=jit, seed=5)
    dm = lm.DofMap(m, 1, fe_order=3 | lm.HIERARCHIC)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    rng = np.random.default_rng(11)
    k = np.exp(rng.normal(0, 0.5, m.n_elem))
    f = rng.uniform(-1, 1, (m.n_nodes, 1))
    asm = lm.GpuAssembly(lm.POISSON, 3 | lm.HIERARCHIC, qo, elem_coef=k, nodal_f=f)
    asm.init(m, dm)
    rp, ci = asm.sparsity()
    K, F = asm.assemble()
    asm.close()
    rpo, cio = orc.sparsity(dm.n_dofs, dm.elem_dofs)
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    Kr, Fr, st, _ = orc.assemble(lm.POISSON, m.elem_type, 3 | 0x100, qo, m.xyz, m.conn, 1, dm.elem_dofs, dm.n_dofs,
                                 dm.constrained, rp, ci, coef=k, nodal_f=f)
    assert st == 0
    tol = k_tolerance(Kr, rp)
    assert np.all(np.abs(K - Kr) <= tol), np.max(np.abs(K - Kr) / np.maximum(tol, 1e-300))
    ftol = 1e-13 * np.abs(Fr).max()
    assert np.all(np.abs(F - Fr) <= np.maximum(1e-13 * np.abs(Fr), ftol))


@pytest.mark.parametrize("et,p,dims,qo", [(lm.PRISM18, 2, (3, 3, 3), 4), (lm.PRISM18, 2, (2, 3, 2), 5),
                                          (lm.PRISM21, 3, (2, 2, 2), 5), (lm.PRISM21, 3, (3, 2, 3), 4)])
def test_hierarchic_prism_matches_oracle(et, p, dims, qo):
    """HIERARCHIC SECOND on PRISM18 and THIRD on PRISM21: the per-element
    shapes of prism_indices (quadrilateral-face cases, vertical-edge
    reflections, triangle-edge flips, face 2's first case as the reference
    indexes it) grouped by orientation pattern; homogeneous Dirichlet on every
    side; the FP64 drop-in against the oracle at 1e-13, and the mixed form
    within FP32 rounding of it with the same load vector."""
    m = lm.Mesh.build_cube(*dims, et)
    dm = lm.DofMap(m, 1, fe_order=p | lm.HIERARCHIC)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    rng = np.random.default_rng(13)
    k = np.exp(rng.normal(0, 0.5, m.n_elem))
    f = rng.uniform(-1, 1, (m.n_nodes, 1))
    K, _ = check(lm.POISSON, m, dm, k, f, p, qo)
    asm = lm.GpuAssembly(lm.POISSON, p | lm.HIERARCHIC, qo, elem_coef=k, nodal_f=f)
    asm.init(m, dm)
    K64, F64 = asm.assemble(lm.FP64)
    K32, F32 = asm.assemble(lm.MIXED)
    asm.close()
    assert np.array_equal(K64, K)
    assert np.linalg.norm(K32 - K64) <= 1e-6 * np.linalg.norm(K64)
    assert np.abs(F32 - F64).max() <= 1e-13 * np.abs(F64).max()
