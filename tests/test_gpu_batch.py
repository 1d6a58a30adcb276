"""Batched assembly (lmg_batch_*): systems of different element types (hexes,
tets, prisms), forms and FE families (HIERARCHIC up to cubic) tuned and
replayed as one CUDA graph give the same K and F
as each system assembled on its own, bit for bit, over repeated replays and
after an input update."""
import numpy as np
import pytest

import libmesh_gb300 as lm
from helpers import make_problem
from test_gpu_constrained import cd_params, problem as cd_problem

pytestmark = pytest.mark.gpu


def members():
    out = []
    m, dm, k, f = make_problem(5, lm.HEX8, 1, lm.POISSON, seed=1)
    out.append((lm.GpuAssembly(lm.POISSON, 1 | lm.HIERARCHIC, 3, elem_coef=k, nodal_f=f), m, dm))
    m, dm, k, f = make_problem(3, lm.TET10, 3, lm.ELASTICITY, jitter=0.2, seed=2)
    out.append((lm.GpuAssembly(lm.ELASTICITY, 2, 4, elem_coef=k, nodal_f=f), m, dm))
    m, dm, k, f = cd_problem(3, lm.HEX27, 2, 2)
    out.append((lm.GpuAssembly(lm.ADVDIFF, 2, 5, elem_coef=k, nodal_f=f, params=cd_params()), m, dm))
    m, dm, k, f = make_problem(4, lm.HEX27, 1, lm.POISSON, seed=4)
    out.append((lm.GpuAssembly(lm.POISSON, 2, 5, elem_coef=k, nodal_f=f), m, dm))
    m = lm.Mesh.build_cube(3, 3, 3, lm.HEX27)
    dm = lm.DofMap(m, 1, fe_order=3 | lm.HIERARCHIC)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    rng = np.random.default_rng(5)
    out.append((lm.GpuAssembly(lm.POISSON, 3 | lm.HIERARCHIC, 7, elem_coef=rng.uniform(0.1, 10, m.n_elem),
                               nodal_f=rng.uniform(-1, 1, (m.n_nodes, 1))), m, dm))
    m, dm, k, f = make_problem(4, lm.PRISM6, 1, lm.POISSON, jitter=0.2, seed=6)
    out.append((lm.GpuAssembly(lm.POISSON, 1 | lm.HIERARCHIC, 3, elem_coef=k, nodal_f=f), m, dm))
    m = lm.Mesh.build_cube(3, 3, 3, lm.TET14, jitter=0.2, seed=7)
    dm = lm.DofMap(m, 1, fe_order=3 | lm.HIERARCHIC)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    out.append((lm.GpuAssembly(lm.POISSON, 3 | lm.HIERARCHIC, 6, elem_coef=rng.uniform(0.1, 10, m.n_elem),
                               nodal_f=rng.uniform(-1, 1, (m.n_nodes, 1))), m, dm))
    for et, p, q in ((lm.PRISM18, 2, 4), (lm.PRISM21, 3, 5)):
        m = lm.Mesh.build_cube(3, 2, 2, et)
        dm = lm.DofMap(m, 1, fe_order=p | lm.HIERARCHIC)
        dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
        out.append((lm.GpuAssembly(lm.POISSON, p | lm.HIERARCHIC, q, elem_coef=rng.uniform(0.1, 10, m.n_elem),
                                   nodal_f=rng.uniform(-1, 1, (m.n_nodes, 1))), m, dm))
    for a, m, dm in out:
        a.init(m, dm)
    return out


def test_batch_matches_individual_assembly():
    mem = members()
    a0 = mem[0][0]
    k1 = a0.elem_coef.copy()
    a0.update_inputs(elem_coef=2.0 * k1)
    ref2 = a0.assemble()                              # the first member with new inputs
    a0.update_inputs(elem_coef=k1)
    ref = [a.assemble() for a, _, _ in mem]           # each on its own stream
    b = lm.Batch()
    for a, _, _ in mem:
        b.add(a)
    b.tune(lm.FP64, reps=2)
    _, launches, grids = b.info()
    assert all(g in (2, 4, 8, 16, 32) for g in grids)
    for _ in range(2):
        b.assemble(lm.FP64)
        b.synchronize()
        for (a, _, _), (K0, F0) in zip(mem, ref):
            K, F = a.result()
            assert np.array_equal(K, K0) and np.array_equal(F, F0)
    _, launches, _ = b.info()
    assert launches >= 2 * len(mem)                   # one graph holds every member's kernels
    # new inputs between replays flow through the same graph
    a0.update_inputs(elem_coef=2.0 * k1)
    b.assemble(lm.FP64)
    b.synchronize()
    K, F = a0.result()
    assert np.array_equal(K, ref2[0]) and np.array_equal(F, ref2[1])
    b.close()
    # the members keep working on their own streams afterwards
    a0.update_inputs(elem_coef=k1)
    K, F = a0.assemble()
    assert np.array_equal(K, ref[0][0]) and np.array_equal(F, ref[0][1])
    for a, _, _ in mem:
        a.close()


def test_batch_mixed_precision_graph():
    """Every member in the mixed form (fused row kernel, FP32 element blocks,
    FP32 general-path contraction) replays bit for bit as assembled alone."""
    mem = members()
    ref = [a.assemble(lm.MIXED) for a, _, _ in mem]
    b = lm.Batch()
    for a, _, _ in mem:
        b.add(a)
    b.tune(lm.MIXED, reps=2)
    for _ in range(2):
        b.assemble(lm.MIXED)
        b.synchronize()
        for (a, _, _), (K0, F0) in zip(mem, ref):
            K, F = a.result()
            assert np.array_equal(K, K0) and np.array_equal(F, F0)
    b.close()
    for a, _, _ in mem:
        a.close()


def poisson_members():
    """Affine one-variable Poisson systems of every element kind the
    persistent batch takes: block-path LAGRANGE / HIERARCHIC p <= 2 and the
    per-pattern HIERARCHIC members."""
    rng = np.random.default_rng(21)
    out = []
    for et, fo, q, dims, jit in ((lm.HEX8, 1 | lm.HIERARCHIC, 3, (5, 4, 4), 0.0), (lm.HEX27, 2, 5, (3, 3, 3), 0.0),
                                 (lm.TET4, 1, 2, (4, 4, 3), 0.2), (lm.TET10, 2, 4, (3, 3, 3), 0.2),
                                 (lm.PRISM6, 1 | lm.HIERARCHIC, 3, (4, 3, 3), 0.0),
                                 (lm.HEX27, 3 | lm.HIERARCHIC, 7, (3, 2, 3), 0.0),
                                 (lm.TET14, 3 | lm.HIERARCHIC, 6, (3, 3, 2), 0.2),
                                 (lm.PRISM18, 2 | lm.HIERARCHIC, 4, (3, 2, 2), 0.0),
                                 (lm.PRISM21, 3 | lm.HIERARCHIC, 5, (2, 3, 2), 0.0)):
        m = lm.Mesh.build_cube(*dims, et, jitter=jit, seed=3)
        dm = lm.DofMap(m, 1, fe_order=fo if (fo & 0xff) == 3 or et == lm.PRISM18 else None)
        dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
        a = lm.GpuAssembly(lm.POISSON, fo, q, elem_coef=rng.uniform(0.1, 10, m.n_elem),
                           nodal_f=rng.uniform(-1, 1, (m.n_nodes, 1)))
        a.init(m, dm)
        out.append(a)
    return out


@pytest.mark.parametrize("prec", [lm.FP64, lm.MIXED])
def test_persistent_hybrid_batch(prec):
    """One persistent launch over the per-pattern members, the block-path
    members' own kernels beside it in the same graph: the block-path members'
    K and F equal their own assemblies bit for bit, the others to rounding."""
    mem = poisson_members()
    own = [a.assemble(prec) for a in mem]
    b = lm.Batch()
    for a in mem:
        b.add(a)
    b.set_persistent(True, hybrid=True)
    b.tune(prec, reps=1)
    _, launches, _ = b.info()
    assert launches > 1
    for _ in range(2):
        b.assemble(prec)
        b.synchronize()
        for i, (a, (K0, F0)) in enumerate(zip(mem, own)):
            K, F = a.result()
            if i < 5:  # the block-path members (poisson_members lists them first)
                assert np.array_equal(K, K0) and np.array_equal(F, F0)
                continue
            rp = a.sparsity()[0]
            rowmax = np.maximum.reduceat(np.abs(K0), rp[:-1])
            rows = np.repeat(np.arange(len(rowmax)), np.diff(rp))
            tol = 1e-12 if prec == lm.FP64 else 1e-6
            assert np.all(np.abs(K - K0) <= tol * np.maximum(np.abs(K0), rowmax[rows]))
            assert np.all(np.abs(F - F0) <= 1e-12 * np.maximum(np.abs(F0), np.abs(F0).max()))
    b.close()
    for a in mem:
        a.close()


@pytest.mark.parametrize("prec", [lm.FP64, lm.MIXED])
def test_persistent_batch_one_launch(prec):
    """Every member in one persistent launch per replay: each member's K and F
    equal its own assembly to rounding (the per-pattern arithmetic of the
    element tiles: 1e-12 of the row scale for the FP64 drop-in, FP32
    rounding for the mixed form), over repeated and re-tuned replays."""
    mem = poisson_members()
    own = [a.assemble(prec) for a in mem]
    b = lm.Batch()
    for a in mem:
        b.add(a)
    b.set_persistent(True)
    b.tune(prec, reps=1)
    tile, ctas, items = b.persistent_info()
    assert tile in (8, 16, 32) and items > len(mem)
    _, launches, _ = b.info()
    assert launches == 1
    for _ in range(2):
        b.assemble(prec)
        b.synchronize()
        for a, (K0, F0) in zip(mem, own):
            K, F = a.result()
            if prec == lm.FP64:
                rowmax = np.maximum.reduceat(np.abs(K0), a.sparsity()[0][:-1])
                rows = np.repeat(np.arange(len(rowmax)), np.diff(a.sparsity()[0]))
                assert np.all(np.abs(K - K0) <= 1e-12 * np.maximum(np.abs(K0), rowmax[rows]))
                assert np.all(np.abs(F - F0) <= 1e-12 * np.maximum(np.abs(F0), np.abs(F0).max()))
            else:
                assert np.linalg.norm(K - K0) <= 1e-6 * np.linalg.norm(K0)
                assert np.linalg.norm(F - F0) <= 1e-12 * np.linalg.norm(F0)
    b.close()
    for a in mem:
        a.close()
