"""Setup on the GPU: hanging-node constraint rows (lmg_constraint_rows_device)
against the host construction (lmg_constraint_rows, itself checked against the
oracle's Newton inverse_map in tests/test_amr_host.py): the constrained set,
the row structure and every coefficient bit for bit, on refined HEX8 and
HEX27 cubes with one and three variables and at the full size of config 3;
and dof numbering (lmg_dofmap_distribute_device) against the host's."""
import time

import numpy as np
import pytest

import libmesh_gb300 as lm

pytestmark = pytest.mark.gpu


def rows(m, n_vars, dirichlet, device):
    dm = lm.DofMap(m, n_vars)
    if dirichlet:
        dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], list(range(n_vars)))
    t0 = time.perf_counter()
    dm.create_dof_constraints(device=device)
    return dm, time.perf_counter() - t0


def same(a, b):
    assert np.array_equal(a.constrained, b.constrained)
    assert np.array_equal(a.cons_ptr, b.cons_ptr)
    assert np.array_equal(a.cons_col, b.cons_col)
    assert np.array_equal(a.cons_val, b.cons_val)


@pytest.mark.parametrize("n,et,cycles,seed,n_vars,dirichlet", [
    (3, lm.HEX8, 2, 1, 1, True), (4, lm.HEX27, 3, 2, 1, True), (4, lm.HEX27, 2, 5, 3, True),
    (3, lm.HEX8, 3, 7, 3, False), (5, lm.HEX27, 3, 11, 1, False)])
def test_device_rows_equal_host_rows(n, et, cycles, seed, n_vars, dirichlet):
    m = lm.Mesh.build_refined_cube(n, et, cycles, 0.2, seed)
    host, _ = rows(m, n_vars, dirichlet, None)
    dev, _ = rows(m, n_vars, dirichlet, 0)
    assert int(host.constrained.sum()) > 0
    same(host, dev)


def test_device_rows_full_size_config3():
    """build_cube 24^3 HEX27, three cycles of 20 % refinement (the
    convection-diffusion benchmark mesh)."""
    m = lm.Mesh.build_refined_cube(24, lm.HEX27, 3, 0.2, 2)
    host, th = rows(m, 1, True, None)
    dev, td = rows(m, 1, True, 0)
    same(host, dev)
    print("config-3 constraint rows: host %.3f s, device %.3f s (%d rows)" % (th, td, int(host.constrained.sum())))


@pytest.mark.parametrize("et,n_vars,fo,dims", [
    (lm.HEX8, 1, 0, (5, 4, 3)), (lm.TET10, 3, 0, (4, 4, 4)), (lm.HEX27, 1, 0, (3, 3, 3)),
    (lm.HEX27, 1, 3 | lm.HIERARCHIC, (3, 2, 3)), (lm.TET14, 1, 3 | lm.HIERARCHIC, (3, 3, 3)),
    (lm.PRISM21, 1, 3 | lm.HIERARCHIC, (2, 3, 2)), (lm.PRISM18, 1, 2 | lm.HIERARCHIC, (3, 3, 2))])
def test_device_dof_numbering_equals_host(et, n_vars, fo, dims):
    """distribute_dofs as a scan on the device: n_dofs and every dof_indices
    list equal the host's sequential first-touch numbering."""
    m = lm.Mesh.build_cube(*dims, et)
    h = lm.DofMap(m, n_vars, fe_order=fo or None)
    d = lm.DofMap(m, n_vars, fe_order=fo or None, device=0)
    assert d.n_dofs == h.n_dofs and np.array_equal(d.elem_dofs, h.elem_dofs)


def test_device_dof_numbering_refined_and_full_size():
    """A refined HEX27 mesh (the config-3 mesh) and the 48^3 TET10 headline mesh."""
    for m, nv in ((lm.Mesh.build_refined_cube(24, lm.HEX27, 3, 0.2, 2), 1),
                  (lm.Mesh.build_cube(48, 48, 48, lm.TET10, jitter=0.2, seed=1), 3)):
        t0 = time.perf_counter()
        h = lm.DofMap(m, nv)
        th = time.perf_counter() - t0
        t0 = time.perf_counter()
        d = lm.DofMap(m, nv, device=0)
        td = time.perf_counter() - t0
        assert d.n_dofs == h.n_dofs and np.array_equal(d.elem_dofs, h.elem_dofs)
        print("dof numbering (%d elements): host %.3f s, device %.3f s" % (m.n_elem, th, td))
