"""The general path's insertion plan built on the device (plan_device.cu)
against the host build (general_plan in context_general.cu): both plans drive
the same kernels, so K and F of both forms must agree bit for bit.  Covers
hanging-node constraint rows on refined HEX27 / HEX8 cubes (Poisson and
convection-diffusion), Dirichlet rows alone, no constraints, cubic
HIERARCHIC elements (64, 20 and 40 dofs; their pattern kernels mask the
Dirichlet rows themselves, so the plan has no constraint matrices) and the full-size
convection-diffusion mesh (build_cube 24^3 HEX27, three cycles of 20 %
refinement)."""
import time

import numpy as np
import pytest

import libmesh_gb300 as lm

pytestmark = pytest.mark.gpu


def cd_params(seed=3, n_modes=8, kappa=1e-2):
    rng = np.random.default_rng(seed)
    p = [kappa, n_modes]
    for _ in range(n_modes):
        p += list(rng.uniform(-1, 1, 3)) + list(2 * np.pi * rng.uniform(-1.5, 1.5, 3)) + [rng.uniform(0, 2 * np.pi)]
    return np.array(p)


def both_plans(form, m, dm, fo, qo, k, f, params=None):
    out = []
    for on_device in (True, False):
        asm = lm.GpuAssembly(form, fo, qo, elem_coef=k, nodal_f=f, params=params)
        asm.init(m, dm)
        asm.set_plan_on_device(on_device)
        t0 = time.perf_counter()
        K64, F64 = asm.assemble(lm.FP64)
        t_first = time.perf_counter() - t0
        K32, F32 = asm.assemble(lm.MIXED)
        general = asm.plan_on_device()
        asm.close()
        out.append((K64, F64, K32, F32, general, t_first))
    return out


def check(out):
    (K64d, F64d, K32d, F32d, dev_flag, td), (K64h, F64h, K32h, F32h, host_flag, th) = out
    assert dev_flag and not host_flag
    for a, b in ((K64d, K64h), (F64d, F64h), (K32d, K32h), (F32d, F32h)):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    return td, th


@pytest.mark.parametrize("form,et,n,cycles,seed,fo,qo,dirichlet,constraints", [
    (lm.POISSON, lm.HEX27, 3, 2, 2, 2, 5, True, True),
    (lm.ADVDIFF, lm.HEX27, 2, 3, 11, 2, 5, True, True),
    (lm.ADVDIFF, lm.HEX27, 3, 2, 4, 2, 5, False, True),
    (lm.POISSON, lm.HEX8, 3, 3, 5, 1, 3, True, True),
    (lm.ADVDIFF, lm.HEX27, 4, 0, 1, 2, 5, True, True),
    (lm.ADVDIFF, lm.HEX27, 3, 0, 1, 2, 5, False, False),
])
def test_device_plan_equals_host_plan(form, et, n, cycles, seed, fo, qo, dirichlet, constraints):
    m = lm.Mesh.build_refined_cube(n, et, cycles, 0.2, seed) if cycles else lm.Mesh.build_cube(n, n, n, et)
    dm = lm.DofMap(m, 1)
    if dirichlet:
        dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    if constraints:
        dm.create_dof_constraints()
    rng = np.random.default_rng(seed)
    f = rng.uniform(-1, 1, (m.n_nodes, 1))
    k = np.exp(rng.normal(0, 0.5, m.n_elem))
    check(both_plans(form, m, dm, fo, qo, k, f, cd_params() if form == lm.ADVDIFF else None))


@pytest.mark.parametrize("et,dims,qo", [(lm.HEX27, (3, 2, 3), 7), (lm.TET14, (3, 3, 3), 6),
                                        (lm.PRISM21, (2, 3, 2), 5)])
def test_device_plan_cubic_hierarchic(et, dims, qo):
    m = lm.Mesh.build_cube(*dims, et)
    dm = lm.DofMap(m, 1, fe_order=3 | lm.HIERARCHIC)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    rng = np.random.default_rng(3)
    k = rng.uniform(0.1, 10.0, m.n_elem)
    f = rng.uniform(-1.0, 1.0, (m.n_nodes, 1))
    check(both_plans(lm.POISSON, m, dm, 3 | lm.HIERARCHIC, qo, k, f))


def test_device_plan_full_size_convection_diffusion():
    m = lm.Mesh.build_refined_cube(24, lm.HEX27, 3, 0.2, 2)
    dm = lm.DofMap(m, 1)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    dm.create_dof_constraints()
    rng = np.random.default_rng(2)
    f = rng.uniform(-1, 1, (m.n_nodes, 1))
    k = np.exp(rng.normal(0, 0.5, m.n_elem))
    td, th = check(both_plans(lm.ADVDIFF, m, dm, 2, 5, k, f, cd_params()))
    print("plan and first assembly (%d elements): device %.3f s, host %.3f s" % (m.n_elem, td, th))


def test_pipelined_host_output_equals_device_output():
    """Host outputs of a large general-path system: the insertion runs in row
    ranges, each range's copy overlapping the next range's insertion; K and F
    equal the device outputs of one whole-mesh insertion bit for bit."""
    import torch
    m = lm.Mesh.build_refined_cube(16, lm.HEX27, 3, 0.2, 2)
    dm = lm.DofMap(m, 1)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    dm.create_dof_constraints()
    rng = np.random.default_rng(2)
    f = rng.uniform(-1, 1, (m.n_nodes, 1))
    k = np.exp(rng.normal(0, 0.5, m.n_elem))
    asm = lm.GpuAssembly(lm.ADVDIFF, 2, 5, elem_coef=k, nodal_f=f, params=cd_params())
    asm.init(m, dm)
    assert asm.nnz * 8 > 64 << 20   # large enough for the pipelined host output
    for prec in (lm.FP64, lm.MIXED):
        Kh, Fh = asm.assemble(prec)
        Kd = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
        Fd = torch.empty(dm.n_dofs, dtype=torch.float64, device="cuda")
        asm.assemble_device(prec, Kd.data_ptr(), Fd.data_ptr())
        asm.synchronize()
        assert np.array_equal(Kh.view(np.uint64), Kd.cpu().numpy().view(np.uint64))
        assert np.array_equal(Fh.view(np.uint64), Fd.cpu().numpy().view(np.uint64))
    asm.close()
