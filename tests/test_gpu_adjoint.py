"""Adjoint sensitivities with respect to per-element coefficients (GPU VJP)
against the oracle's restatement of ImplicitSystem::adjoint_qoi_parameter_sensitivity
(central differences of the residual) and against central differences of the
QoI itself (device solves).  Bar: relative agreement <= 1e-6."""
import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from helpers import make_problem

pytestmark = pytest.mark.gpu


def centroid_x(mesh):
    return mesh.xyz[mesh.conn][:, :, 0].mean(1)


@pytest.mark.parametrize("et,nv,form,fo,qo,n,jit", [(lm.HEX8, 1, lm.POISSON, 1, 2, 6, 0.0),
                                                    (lm.TET10, 3, lm.ELASTICITY, 2, 4, 3, 0.2)])
def test_vjp_matches_reference_adjoint_sensitivity(et, nv, form, fo, qo, n, jit):
    mesh, dm, k, f = make_problem(n, et, nv, form, jitter=jit, seed=4)
    region = (centroid_x(mesh) < 0.5).astype(np.uint8)
    system = lm.LinearImplicitSystem(mesh, nv)
    system.dof_map = dm
    system.attach_assemble_object(lm.GpuAssembly(form, fo, qo, elem_coef=k, nodal_f=f))
    system.init()
    Q, g = system.adjoint_qoi_parameter_sensitivity(region, rtol=1e-13)
    rng = np.random.default_rng(4)
    params = rng.choice(mesh.n_elem, 6, replace=False)
    Qr, sens = orc.adjoint_qoi_parameter_sensitivity(form, et, fo, qo, mesh.xyz, mesh.conn, nv, dm.elem_dofs,
                                                     dm.n_dofs, dm.constrained, system.row_ptr, system.col_idx,
                                                     k, f, region, params)
    assert abs(Q - Qr) <= 1e-9 * abs(Qr)
    scale = np.abs(g).max()
    np.testing.assert_allclose(g[params], sens, rtol=1e-6, atol=1e-6 * scale)
    system.assembly.close()


def test_vjp_matches_qoi_central_differences():
    """dq/dk_e against (q(k + h e_j) - q(k - h e_j)) / 2h with h = 1e-6 k_j, device solves."""
    mesh, dm, k, f = make_problem(8, lm.HEX8, 1, lm.POISSON, seed=4)
    region = (centroid_x(mesh) < 0.25).astype(np.uint8)
    asm = lm.GpuAssembly(lm.POISSON, 1, 2, elem_coef=k, nodal_f=f)
    system = lm.LinearImplicitSystem(mesh, 1)
    system.dof_map = dm
    system.attach_assemble_object(asm)
    system.init()
    Q, g = system.adjoint_qoi_parameter_sensitivity(region, rtol=1e-14)
    qv = asm.qoi_region_load(region)
    rng = np.random.default_rng(5)
    for j in rng.choice(mesh.n_elem, 8, replace=False):
        h = 1e-6 * k[j]
        vals = []
        for s in (+1, -1):
            kk = k.copy()
            kk[j] += s * h
            asm.update_inputs(elem_coef=kk)
            asm.assemble()
            u, _, _ = asm.solve(rtol=1e-14, maxit=100000)
            vals.append(qv @ u)
        fd = (vals[0] - vals[1]) / (2 * h)
        assert abs(g[j] - fd) <= 1e-6 * max(abs(fd), 1e-3 * np.abs(g).max()), (j, g[j], fd)
    asm.close()


@pytest.mark.parametrize("et,fo,qo,n,jit", [(lm.HEX8, 1, 2, 4, 0.1), (lm.TET4, 1, 2, 3, 0.15), (lm.TET10, 2, 4, 2, 0.1)])
def test_coordinate_sensitivity_matches_reference_adjoint(et, fo, qo, n, jit):
    """dq/dx (lmg_vjp_xyz, reverse mode through detJ and J^-1) against the
    oracle's restatement of adjoint_qoi_parameter_sensitivity with node
    coordinates as parameters (central differences of the residual and of the
    QoI).  Bar: relative agreement <= 1e-6."""
    mesh, dm, k, f = make_problem(n, et, 1, lm.POISSON, jitter=jit, seed=4)
    region = (centroid_x(mesh) < 0.5).astype(np.uint8)
    asm = lm.GpuAssembly(lm.POISSON, fo, qo, elem_coef=k, nodal_f=f)
    system = lm.LinearImplicitSystem(mesh, 1)
    system.dof_map = dm
    system.attach_assemble_object(asm)
    system.init()
    asm.assemble()
    u, _, _ = asm.solve(rtol=1e-14, maxit=100000)
    z, _, _ = asm.solve(rhs=asm.qoi_region_load(region), rtol=1e-14, maxit=100000)
    g = asm.vjp_xyz(u, z, region)
    x = mesh.xyz
    interior = np.nonzero(np.all((x > 1e-9) & (x < 1 - 1e-9), axis=1))[0]
    rng = np.random.default_rng(6)
    params = [(int(nd), int(d)) for nd, d in zip(rng.choice(interior, 5, replace=False), rng.integers(0, 3, 5))]
    _, ref = orc.coordinate_sensitivity(lm.POISSON, et, fo, qo, x, mesh.conn, dm.elem_dofs, dm.n_dofs,
                                        dm.constrained, system.row_ptr, system.col_idx, k, f, region, params)
    got = np.array([g[nd, d] for nd, d in params])
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6 * np.abs(g).max())
    # a rigid translation of the whole mesh leaves q unchanged: the interior-plus-boundary sum vanishes
    assert np.all(np.abs(g.sum(0)) <= 1e-9 * np.abs(g).sum(0))
    asm.close()


@pytest.mark.parametrize("et,fo,qo,n,jit", [(lm.TET10, 2, 4, 2, 0.1), (lm.HEX8, 1, 2, 3, 0.1)])
def test_elasticity_coordinate_sensitivity_matches_reference_adjoint(et, fo, qo, n, jit):
    """Elasticity: dq/dx for q = integral of the sum of u's components over the
    marked elements, against the oracle's central-difference restatement."""
    mesh, dm, k, f = make_problem(n, et, 3, lm.ELASTICITY, jitter=jit, seed=5)
    region = (centroid_x(mesh) < 0.5).astype(np.uint8)
    asm = lm.GpuAssembly(lm.ELASTICITY, fo, qo, elem_coef=k, nodal_f=f)
    system = lm.LinearImplicitSystem(mesh, 3)
    system.dof_map = dm
    system.attach_assemble_object(asm)
    system.init()
    asm.assemble()
    u, _, _ = asm.solve(rtol=1e-14, maxit=100000)
    z, _, _ = asm.solve(rhs=asm.qoi_region_load(region), rtol=1e-14, maxit=100000)
    g = asm.vjp_xyz(u, z, region)
    x = mesh.xyz
    interior = np.nonzero(np.all((x > 1e-9) & (x < 1 - 1e-9), axis=1))[0]
    rng = np.random.default_rng(7)
    params = [(int(nd), int(d)) for nd, d in zip(rng.choice(interior, 5, replace=False), rng.integers(0, 3, 5))]
    _, ref = orc.coordinate_sensitivity(lm.ELASTICITY, et, fo, qo, x, mesh.conn, dm.elem_dofs, dm.n_dofs,
                                        dm.constrained, system.row_ptr, system.col_idx, k, f, region, params,
                                        n_vars=3)
    got = np.array([g[nd, d] for nd, d in params])
    np.testing.assert_allclose(got, ref, rtol=1e-6, atol=1e-6 * np.abs(g).max())
    asm.close()
