"""Parity at the benchmark configurations' full sizes.

* Elasticity TET10 on build_cube 48^3 (663,552 elements, 231,797,385 nonzeros):
  the FP64 drop-in against the oracle entry by entry (sparsity bit-exact; K and
  F within 1e-13 of the entry or of the row's largest entry), then the mixed
  form: relative Frobenius error of K and F against the oracle and the
  relative error of the CG-solved field (rtol 1e-12) against the FP64
  drop-in's solve, <= 1e-6.
* Convection-diffusion HEX27 on build_cube 24^3 after three cycles of refining
  20 % of the active elements (356,138 elements, hanging-node and Dirichlet
  rows): FP64 against the oracle's constrain_element_matrix_and_vector
  restatement, entry by entry.
* Adjoint sensitivities of the Poisson HEX8 build_cube 128^3 problem
  (2,097,152 element coefficients): the coefficient VJP against central
  differences of the residual (h = 1e-6 max(|k|, 1e-3), the step of
  adjoint_qoi_parameter_sensitivity) on 64 random parameters, and the
  node-coordinate VJP against central differences of the QoI and residual on
  a sample of nodes; agreement <= 1e-6 relative to max(|entry|, 1e-3 of the
  gradient's largest entry).
The oracle runs on all host threads."""
import os

import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from helpers import make_problem

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def chunked_scaled_error(K, Kr, rp, chunk=1 << 20):
    """max over entries of |K - K_ref| / max(|K_ref_ij|, max_j |K_ref_ij| of the
    row), computed a block of rows at a time (the full-size arrays are large)."""
    n = len(rp) - 1
    worst = 0.0
    for r0 in range(0, n, chunk):
        r1 = min(n, r0 + chunk)
        a, b = int(rp[r0]), int(rp[r1])
        lrp = (rp[r0:r1 + 1] - a).astype(np.int64)
        kr = np.abs(Kr[a:b])
        rowmax = np.maximum.reduceat(kr, lrp[:-1])
        scale = np.maximum(kr, np.repeat(rowmax, np.diff(lrp)))
        worst = max(worst, float(np.max(np.abs(K[a:b] - Kr[a:b]) / np.maximum(scale, 1e-300))))
    return worst


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_c2_elasticity_48_fp64_and_mixed_against_oracle():
    mesh, dm, k, f = make_problem(48, lm.TET10, 3, lm.ELASTICITY, jitter=0.2, seed=1)
    assert (mesh.n_elem, dm.n_dofs) == (663552, 2738019)
    asm = lm.GpuAssembly(lm.ELASTICITY, 2, 4, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    rp, col = asm.sparsity()
    rpo, colo = orc.sparsity(dm.n_dofs, dm.elem_dofs)
    assert np.array_equal(rp, rpo) and np.array_equal(col, colo)
    del rpo, colo
    Kr, Fr, st, _ = orc.assemble(lm.ELASTICITY, lm.TET10, 2, 4, mesh.xyz, mesh.conn, 3, dm.elem_dofs, dm.n_dofs,
                                 dm.constrained, rp, col, coef=k, nodal_f=f, n_threads=THREADS)
    assert st == 0
    K, F = asm.assemble(lm.FP64)
    err = chunked_scaled_error(K, Kr, rp)
    assert err <= 1e-13, "K scaled error %.3g" % err
    ftol = 1e-13 * np.maximum(np.abs(Fr), np.abs(Fr).max())
    assert np.all(np.abs(F - Fr) <= ftol)
    u64, it64, rr64 = asm.solve(rtol=1e-12, maxit=400000)
    assert rr64 <= 1e-12
    del K
    K32, F32 = asm.assemble(lm.MIXED)
    k_err, f_err = rel(K32, Kr), rel(F32, Fr)
    del K32
    u32, it32, rr32 = asm.solve(rtol=1e-12, maxit=400000)
    assert rr32 <= 1e-12
    u_err = rel(u32, u64)
    print("C2 mixed: ||dK||/||K|| %.3g  ||dF||/||F|| %.3g  ||du||/||u|| %.3g  (CG %d / %d iterations)"
          % (k_err, f_err, u_err, it64, it32))
    assert k_err < 1e-6 and f_err < 1e-13
    assert u_err <= 1e-6
    asm.close()


def test_c3_refined_convection_diffusion_full_size_against_oracle():
    import bench
    mesh = lm.Mesh.build_refined_cube(24, lm.HEX27, 3, 0.2, 2)
    dm = lm.DofMap(mesh, 1)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    dm.create_dof_constraints()
    assert mesh.n_elem == 356138
    rng = np.random.default_rng(2)
    k = np.exp(rng.normal(0.0, 0.5, mesh.n_elem))
    f = rng.uniform(-1.0, 1.0, (mesh.n_nodes, 1))
    params = bench.cd_params()
    asm = lm.GpuAssembly(lm.ADVDIFF, 2, 5, elem_coef=k, nodal_f=f, params=params)
    asm.init(mesh, dm)
    rp, ci = asm.sparsity()
    rpo, cio = orc.sparsity_constrained(dm.n_dofs, dm.elem_dofs, dm.cons_ptr, dm.cons_col)
    assert np.array_equal(rp, rpo) and np.array_equal(ci, cio)
    del rpo, cio
    K, F = asm.assemble()
    K32, F32 = asm.assemble(lm.MIXED)
    asm.close()
    Kr, Fr, st, _ = orc.assemble(lm.ADVDIFF, mesh.elem_type, 2, 5, mesh.xyz, mesh.conn, 1, dm.elem_dofs, dm.n_dofs,
                                 dm.constrained, rp, ci, coef=k, nodal_f=f,
                                 cons_rows=(dm.cons_ptr, dm.cons_col, dm.cons_val), params=params,
                                 n_threads=THREADS)
    assert st == 0
    err = chunked_scaled_error(K, Kr, rp)
    assert err <= 1e-13, "K scaled error %.3g" % err
    ftol = 1e-13 * max(np.abs(Fr).max(), 1e-300)
    assert np.all(np.abs(F - Fr) <= np.maximum(1e-13 * np.abs(Fr), ftol))
    print("C3 FP64 worst scaled error %.3g; mixed ||dK||/||K|| %.3g ||dF||/||F|| %.3g"
          % (err, rel(K32, Kr), rel(F32, Fr)))
    assert rel(K32, Kr) < 1e-6 and rel(F32, Fr) < 1e-6


def c5_problem(n=128):
    mesh = lm.Mesh.build_cube(n, n, n, lm.HEX8)
    dm = lm.DofMap(mesh, 1)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    rng = np.random.default_rng(4)
    k = np.exp(rng.normal(0.0, 1.0, mesh.n_elem))
    f = rng.uniform(-1.0, 1.0, (mesh.n_nodes, 1))
    region = (mesh.xyz[mesh.conn][:, :, 0].mean(1) < 0.25).astype(np.uint8)
    return mesh, dm, k, f, region


def local_system(mesh, dm, elems, xyz, coef, f):
    """K and F of the elements `elems` alone (the oracle's assembly, Dirichlet
    rows applied per element as constrain_element_matrix_and_vector does) on
    their own dofs, in a dense local numbering.  Returns (global dofs, K, F)."""
    ed = dm.elem_dofs[elems]
    dofs, loc = np.unique(ed, return_inverse=True)
    nd = len(dofs)
    rp = np.arange(0, nd * nd + 1, nd, dtype=np.int32)
    col = np.tile(np.arange(nd, dtype=np.int32), nd)
    K, F, st, _ = orc.assemble(lm.POISSON, lm.HEX8, 1, 2, xyz, mesh.conn[elems], 1,
                               loc.reshape(ed.shape).astype(np.int32), nd, dm.constrained[dofs], rp, col,
                               coef=coef[elems], nodal_f=f)
    assert st == 0
    return dofs, K.reshape(nd, nd), F


def test_c5_adjoint_128_against_central_differences():
    """Central differences restate adjoint_qoi_parameter_sensitivity
    (src/systems/implicit_system.C:474-623): for a parameter p, h = 1e-6
    max(|p|, 1e-3), -dR/dp = (R(p - h) - R(p + h)) / 2h and dq/dp = (q(p + h) -
    q(p - h)) / 2h at the primal u, sensitivity = dq/dp + (-dR/dp) . z.  The
    residuals are the oracle's FP64 assembly of the elements the parameter
    touches (every other element's contribution is unchanged and cancels
    exactly in the difference), so the differences carry FP64 rounding only."""
    mesh, dm, k, f, region = c5_problem()
    assert mesh.n_elem == 2097152
    asm = lm.GpuAssembly(lm.POISSON, 1, 2, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    asm.assemble()
    u, _, rr = asm.solve(rtol=1e-12, maxit=200000)
    assert rr <= 1e-12
    qv = asm.qoi_region_load(region)
    z, _, rr = asm.solve(rhs=qv, rtol=1e-12, maxit=200000)
    assert rr <= 1e-12
    g = asm.vjp_coef(u, z)
    gscale = np.abs(g).max()
    rng = np.random.default_rng(4)
    params = rng.choice(mesh.n_elem, 64, replace=False)
    worst = 0.0
    for j in params:
        d = 1e-6 * max(abs(k[j]), 1e-3)
        res = []
        for s in (-1.0, 1.0):
            kk = k.copy()
            kk[j] += s * d
            dofs, Ke, Fe = local_system(mesh, dm, np.array([j]), mesh.xyz, kk, f)
            res.append(Ke @ u[dofs] - Fe)
        fd = ((res[0] - res[1]) / (2 * d)) @ z[dofs]
        e = abs(g[j] - fd) / max(abs(g[j]), 1e-3 * gscale)
        worst = max(worst, e)
        assert e <= 1e-6, (int(j), g[j], fd)
    print("C5 coefficient VJP vs central differences on 64 parameters: worst relative error %.3g" % worst)
    # node-coordinate sensitivities on a sample of interior nodes, some on the QoI region's edge
    gx = asm.vjp_xyz(u, z, region)
    asm.close()
    xscale = np.abs(gx).max()
    interior = np.nonzero(((mesh.xyz > 0) & (mesh.xyz < 1)).all(1))[0]
    near = interior[np.abs(mesh.xyz[interior, 0] - 0.25) < 0.02]
    nodes = np.concatenate([rng.choice(interior, 3, replace=False), rng.choice(near, 3, replace=False)])
    ones = np.ones((mesh.n_nodes, 1))
    worst = 0.0
    for node in nodes:
        elems = np.nonzero((mesh.conn == node).any(1))[0]
        reg = elems[region[elems] != 0]
        for dd in range(3):
            p = mesh.xyz[node, dd]
            h = 1e-6 * max(abs(p), 1e-3)
            parts = []
            for s in (-1.0, 1.0):
                x = mesh.xyz.copy()
                x[node, dd] += s * h
                dofs, Ke, Fe = local_system(mesh, dm, elems, x, k, f)
                q = 0.0
                if len(reg):
                    qd, _, qf = local_system(mesh, dm, reg, x, k, ones)
                    qf[dm.constrained[qd] != 0] = 0.0
                    q = qf @ u[qd]
                parts.append((Ke @ u[dofs] - Fe, q))
            fd = (parts[1][1] - parts[0][1]) / (2 * h) + ((parts[0][0] - parts[1][0]) / (2 * h)) @ z[dofs]
            e = abs(gx[node, dd] - fd) / max(abs(gx[node, dd]), 1e-3 * xscale)
            worst = max(worst, e)
            assert e <= 1e-6, (int(node), dd, gx[node, dd], fd)
    print("C5 coordinate VJP vs central differences on %d nodes x 3: worst relative error %.3g" % (len(nodes), worst))
