"""GPU parity: the CUDA assembly through the C ABI against the CPU oracle.

Bar: sparsity bit-exact (row_ptr and col_idx equal); K per entry within
1e-13 * max(|K_ref_ij|, max_j |K_ref_ij| of its row); F within 1e-13 of the
entry or, for entries that cancel to ~0, 1e-13 of max |F_ref|."""
import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from helpers import k_tolerance, make_problem, max_scaled_err, oracle_assemble

pytestmark = pytest.mark.gpu


def gpu_system(mesh, dm, form, fo, qo, k, f, nu=0.3):
    asm = lm.GpuAssembly(form, fo, qo, elem_coef=k, nodal_f=f, nu=nu)
    asm.init(mesh, dm)
    rp, col = asm.sparsity()
    return asm, rp, col


def check_parity(mesh, dm, form, fo, qo, k, f, nu=0.3, precision=lm.FP64):
    asm, rp, col = gpu_system(mesh, dm, form, fo, qo, k, f, nu)
    rpo, colo = orc.sparsity(dm.n_dofs, dm.elem_dofs)
    assert np.array_equal(rp, rpo) and np.array_equal(col, colo), "sparsity differs"
    K, F = asm.assemble(precision)
    Kr, Fr, st, _ = oracle_assemble(form, mesh, dm, fo, qo, rpo, colo, k, f, nu=nu)
    assert st == 0
    err = max_scaled_err(K, Kr, rp)
    assert np.all(np.abs(K - Kr) <= k_tolerance(Kr, rp)), "K scaled error %.3g" % (err * 1e13)
    ftol = 1e-13 * np.maximum(np.abs(Fr), np.abs(Fr).max())
    assert np.all(np.abs(F - Fr) <= ftol)
    asm.close()
    return K, F, Kr, Fr


@pytest.mark.parametrize("n,coef", [(4, False), (5, True)])
def test_poisson_hex8(n, coef):
    mesh, dm, k, f = make_problem(n, lm.HEX8, 1, lm.POISSON, coef=coef)
    check_parity(mesh, dm, lm.POISSON, 1, 2, k, f)


def test_poisson_hex8_c1_full_size():
    """Plain FP64 Poisson, build_cube 32^3 HEX8, QGauss 2x2x2, nodal f ~ U[-1,1],
    homogeneous Dirichlet on all six faces."""
    mesh, dm, k, f = make_problem(32, lm.HEX8, 1, lm.POISSON, coef=False, seed=0)
    assert (mesh.n_elem, mesh.n_nodes) == (32768, 35937)
    K, F, Kr, Fr = check_parity(mesh, dm, lm.POISSON, 1, 2, None, f)
    assert len(K) == 912673


def test_poisson_hex8_nonaffine():
    """Jittered hexes take the per-quadrature-point map (compute_map, not compute_affine_map)."""
    mesh, dm, k, f = make_problem(4, lm.HEX8, 1, lm.POISSON, jitter=0.2)
    assert not all(orc.has_affine_map(lm.HEX8, x) for x in mesh.xyz[mesh.conn])
    check_parity(mesh, dm, lm.POISSON, 1, 2, k, f)


@pytest.mark.parametrize("et,fo,qo,n,jit", [(lm.HEX27, 2, 5, 3, 0.0), (lm.TET4, 1, 2, 4, 0.2),
                                            (lm.TET10, 2, 4, 3, 0.2), (lm.TET10, 2, 3, 2, 0.0),
                                            (lm.PRISM6, 1, 3, 4, 0.0), (lm.PRISM6, 1, 5, 3, 0.2)])
def test_poisson_other_elements(et, fo, qo, n, jit):
    mesh, dm, k, f = make_problem(n, et, 1, lm.POISSON, jitter=jit)
    check_parity(mesh, dm, lm.POISSON, fo, qo, k, f)


@pytest.mark.parametrize("n", [2, 6])
def test_elasticity_tet10(n):
    mesh, dm, k, f = make_problem(n, lm.TET10, 3, lm.ELASTICITY, jitter=0.2)
    check_parity(mesh, dm, lm.ELASTICITY, 2, 4, k, f)


def test_elasticity_tet10_curved():
    """Mid-edge nodes moved off the straight edges: every tet is non-affine."""
    mesh, dm, k, f = make_problem(3, lm.TET10, 3, lm.ELASTICITY, jitter=0.1)
    rng = np.random.default_rng(7)
    mid = np.unique(mesh.conn[:, 4:])
    xyz = mesh.xyz.copy()
    inner = ~((xyz[mid] == 0) | (xyz[mid] == 1)).any(1)
    xyz[mid[inner]] += rng.uniform(-0.02, 0.02, (inner.sum(), 3)) / 3
    mesh.xyz = xyz
    aff = sum(orc.has_affine_map(lm.TET10, x) for x in mesh.xyz[mesh.conn])
    assert aff < mesh.n_elem // 2
    check_parity(mesh, dm, lm.ELASTICITY, 2, 4, k, f)


def test_elasticity_hex8_and_tet4():
    mesh, dm, k, f = make_problem(3, lm.HEX8, 3, lm.ELASTICITY)
    check_parity(mesh, dm, lm.ELASTICITY, 1, 2, k, f, nu=0.25)
    mesh, dm, k, f = make_problem(3, lm.TET4, 3, lm.ELASTICITY, jitter=0.2)
    check_parity(mesh, dm, lm.ELASTICITY, 1, 2, k, f)


@pytest.mark.parametrize("jit", [0.0, 0.2])
def test_elasticity_prism6(jit):
    """PRISM6 (build_cube, two prisms per cell): affine when unjittered, the
    per-quadrature-point map once interior nodes move."""
    mesh, dm, k, f = make_problem(3, lm.PRISM6, 3, lm.ELASTICITY, jitter=jit)
    aff = sum(orc.has_affine_map(lm.PRISM6, x) for x in mesh.xyz[mesh.conn])
    assert (aff == mesh.n_elem) == (jit == 0.0)
    check_parity(mesh, dm, lm.ELASTICITY, 1, 3, k, f)


def test_repeat_is_bitwise_deterministic():
    mesh, dm, k, f = make_problem(6, lm.TET10, 3, lm.ELASTICITY, jitter=0.2)
    asm, rp, col = gpu_system(mesh, dm, lm.ELASTICITY, 2, 4, k, f)
    K1, F1 = asm.assemble()
    for _ in range(3):
        K2, F2 = asm.assemble()
        assert np.array_equal(K1, K2) and np.array_equal(F1, F2)
    # refreshing the inputs re-assembles the new problem
    asm.update_inputs(elem_coef=2 * k)
    K3, _ = asm.assemble()
    c = dm.constrained.astype(bool)
    rows = np.repeat(np.arange(dm.n_dofs), np.diff(rp))
    free = ~c[rows] & ~c[col]
    np.testing.assert_allclose(K3[free], 2 * K1[free], rtol=1e-14, atol=1e-14 * abs(K1).max())
    asm.close()


def test_degenerate_element_raises():
    mesh, dm, k, f = make_problem(3, lm.HEX8, 1, lm.POISSON, bids=[])
    xyz = mesh.xyz.copy()
    c = mesh.conn[5]
    xyz[c[6]] = xyz[c[0]]
    mesh.xyz = xyz
    asm = lm.GpuAssembly(lm.POISSON, 1, 2)
    asm.init(mesh, dm)
    with pytest.raises(lm.DegenerateMap) as ei:
        asm.assemble()
    assert ei.value.elem >= 0
    asm.close()


def test_c2_full_size_properties():
    """TET10 elasticity on build_cube 48^3 split 6 tets per hex (no clamp, f = 1):
    sizes, sparsity size, rigid-body modes in the kernel of K, sampled symmetry
    and the load sum (the full problem is beyond the oracle's time budget; the
    medium case below is compared entry by entry)."""
    mesh, dm, k, f = make_problem(48, lm.TET10, 3, lm.ELASTICITY, jitter=0.2, seed=1, bids=[])
    assert (mesh.n_elem, dm.n_dofs) == (663552, 2738019)
    ones = np.ones((mesh.n_nodes, 3))
    asm, rp, col = gpu_system(mesh, dm, lm.ELASTICITY, 2, 4, k, ones)
    assert len(col) == 231797385
    # the device block graph against the host compute_sparsity restatement
    import ctypes
    from libmesh_gb300._capi import lib, ptr
    nnz = ctypes.c_int64()
    rph = np.empty(dm.n_dofs + 1, np.int32)
    colh = np.empty(len(col), np.int32)
    assert lib().lmg_host_sparsity(mesh.n_elem, 10, 3, dm.n_dofs, ptr(dm.elem_dofs), nnz, ptr(rph), ptr(colh)) == 0
    assert nnz.value == len(col) and np.array_equal(rp, rph) and np.array_equal(col, colh)
    del rph, colh
    K, F = asm.assemble()
    asm.close()
    assert abs(F.sum() - 3.0) < 1e-10  # f = 1 per component integrates to the unit volume
    import scipy.sparse as sp
    A = sp.csr_matrix((K, col, rp), shape=(dm.n_dofs, dm.n_dofs))
    npe = 10
    node_of = np.empty(dm.n_dofs, np.int64)
    comp = np.empty(dm.n_dofs, np.int64)
    for v in range(3):
        node_of[dm.elem_dofs[:, v * npe:(v + 1) * npe].ravel()] = mesh.conn.ravel()
        comp[dm.elem_dofs[:, v * npe:(v + 1) * npe].ravel()] = v
    x = mesh.xyz[node_of]
    scale = np.abs(K).max()
    for v in range(3):
        assert np.abs(A @ (comp == v).astype(float)).max() < 1e-11 * scale
    u = np.zeros(dm.n_dofs)
    u[comp == 0] = -x[comp == 0, 1]
    u[comp == 1] = x[comp == 1, 0]
    assert np.abs(A @ u).max() < 1e-11 * scale
    rows = np.repeat(np.arange(dm.n_dofs, dtype=np.int64), np.diff(rp))
    keys = rows * dm.n_dofs + col
    idx = np.random.default_rng(0).integers(0, len(K), 1_000_000)
    tpos = np.searchsorted(keys, col[idx].astype(np.int64) * dm.n_dofs + rows[idx])
    assert np.array_equal(keys[tpos], col[idx].astype(np.int64) * dm.n_dofs + rows[idx])
    assert np.abs(K[idx] - K[tpos]).max() < 1e-14 * scale


def test_c2_medium_parity():
    mesh, dm, k, f = make_problem(10, lm.TET10, 3, lm.ELASTICITY, jitter=0.2, seed=1)
    check_parity(mesh, dm, lm.ELASTICITY, 2, 4, k, f)


@pytest.mark.parametrize("precision", [lm.FP64, lm.MIXED])
def test_chunked_host_output_equals_device_output(precision):
    """Host outputs above 64 MB are inserted in row chunks, each copied to the
    host while the next is inserted; the result equals the device-resident
    assembly (one insertion launch, one copy afterwards) bit for bit."""
    mesh, dm, k, f = make_problem(20, lm.TET10, 3, lm.ELASTICITY, jitter=0.2, seed=5)
    asm, rp, col = gpu_system(mesh, dm, lm.ELASTICITY, 2, 4, k, f)
    assert asm.nnz * 8 > 64 << 20
    n0 = asm.launch_count()
    asm.assemble_device(precision)
    asm.synchronize()
    n1 = asm.launch_count()
    Kd, Fd = asm.result()
    K, F = asm.assemble(precision)
    n2 = asm.launch_count()
    assert n2 - n1 > n1 - n0                  # the insertion ran in several launches
    assert np.array_equal(K, Kd) and np.array_equal(F, Fd)
    asm.close()
