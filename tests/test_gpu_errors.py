"""Error statuses of the device context through the C ABI (the reference
raises libmesh_error_msg / DegenerateMap; here every failure is a status and
lmg_last_error's message, and the context stays usable), and the smallest
meshes: one hexahedron, one cube of six tets, one cube of cubic tets."""
import ctypes as C

import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from helpers import k_tolerance, make_problem, oracle_assemble
from libmesh_gb300 import _capi
from libmesh_gb300._capi import lib, ptr

pytestmark = pytest.mark.gpu


def last_error(h):
    msg = C.create_string_buffer(512)
    eid = C.c_int64(-1)
    lib().lmg_last_error(h, C.byref(eid), msg, 512)
    return msg.value.decode(), eid.value


@pytest.fixture
def ctx():
    h = C.c_void_p()
    assert lib().lmg_context_create(C.byref(h), 0) == _capi.OK
    yield h
    assert lib().lmg_context_destroy(h) == _capi.OK


def test_calls_out_of_order_are_state_errors(ctx):
    nnz = C.c_int64()
    assert lib().lmg_sparsity_build(ctx, C.byref(nnz)) == _capi.ERR_STATE
    assert "dofmap" in last_error(ctx)[0]
    m = lm.Mesh.build_cube(2, 2, 2, lm.HEX8)
    assert lib().lmg_mesh_upload(ctx, m.n_nodes, ptr(m.xyz), m.n_elem, m.elem_type, ptr(m.conn)) == _capi.OK
    K = np.empty(1)
    F = np.empty(1)
    assert lib().lmg_assemble(ctx, lm.FP64, ptr(K), ptr(F), 0) != _capi.OK


def test_out_of_range_ids_are_bounds_errors(ctx):
    m = lm.Mesh.build_cube(2, 2, 2, lm.HEX8)
    conn = m.conn.copy()
    conn[5, 3] = m.n_nodes  # one past the last node
    st = lib().lmg_mesh_upload(ctx, m.n_nodes, ptr(m.xyz), m.n_elem, m.elem_type, ptr(conn))
    assert st == _capi.ERR_BOUNDS
    assert last_error(ctx)[1] == 5
    # the context is still usable
    assert lib().lmg_mesh_upload(ctx, m.n_nodes, ptr(m.xyz), m.n_elem, m.elem_type, ptr(m.conn)) == _capi.OK
    dm = lm.DofMap(m, 1)
    ed = dm.elem_dofs.copy()
    ed[3, 0] = -1
    assert lib().lmg_dofmap_upload(ctx, 1, dm.n_dofs, ptr(ed)) == _capi.ERR_BOUNDS
    assert last_error(ctx)[1] == 3
    assert lib().lmg_dofmap_upload(ctx, 1, dm.n_dofs, ptr(dm.elem_dofs)) == _capi.OK
    nnz = C.c_int64()
    assert lib().lmg_sparsity_build(ctx, C.byref(nnz)) == _capi.OK and nnz.value > 0


def test_unbuilt_feature_combinations_are_unsupported(ctx):
    n = C.c_int32()
    assert lib().lmg_fe_dofs_per_elem(lm.TET10, 3 | lm.HIERARCHIC, 1, C.byref(n)) == _capi.ERR_UNSUPPORTED
    assert lib().lmg_fe_dofs_per_elem(lm.TET14, 3 | lm.HIERARCHIC, 3, C.byref(n)) == _capi.ERR_UNSUPPORTED
    m = lm.Mesh.build_cube(1, 1, 1, lm.TET10)
    assert lib().lmg_mesh_upload(ctx, m.n_nodes, ptr(m.xyz), m.n_elem, m.elem_type, ptr(m.conn)) == _capi.OK
    ed = np.zeros((m.n_elem, 20), np.int32)
    assert lib().lmg_dofmap_upload_fe(ctx, 1, 3 | lm.HIERARCHIC, 20, ptr(ed)) == _capi.ERR_UNSUPPORTED
    assert "TET14" in last_error(ctx)[0]


def test_curved_cubic_tets_are_refused():
    m = lm.Mesh.build_cube(1, 1, 1, lm.TET14)
    xyz = m.xyz.copy()
    xyz[m.conn[0, 12]] += 0.01  # move a face node off its face centroid
    mc = lm.Mesh(xyz, m.conn, m.elem_type, m.side_bid)
    dm = lm.DofMap(mc, 1, fe_order=3 | lm.HIERARCHIC)
    asm = lm.GpuAssembly(lm.POISSON, 3 | lm.HIERARCHIC, 6)
    with pytest.raises(lm.LmgError, match="affine"):
        asm.init(mc, dm)
    asm.close()


def test_single_hex_matches_oracle():
    mesh, dm, k, f = make_problem(1, lm.HEX8, 1, lm.POISSON, coef=True)
    asm = lm.GpuAssembly(lm.POISSON, 1, 2, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    rp, col = asm.sparsity()
    K, F = asm.assemble()
    asm.close()
    assert len(col) == 64
    Kr, Fr, st, _ = oracle_assemble(lm.POISSON, mesh, dm, 1, 2, rp, col, k, f)
    assert st == 0 and np.all(np.abs(K - Kr) <= k_tolerance(Kr, rp))
    assert np.allclose(F, Fr, rtol=1e-13, atol=1e-13 * np.abs(Fr).max())


def test_single_cube_of_cubic_tets_matches_oracle():
    m = lm.Mesh.build_cube(1, 1, 1, lm.TET14)
    dm = lm.DofMap(m, 1, fe_order=3 | lm.HIERARCHIC)
    rng = np.random.default_rng(2)
    k = rng.uniform(0.1, 10, m.n_elem)
    f = rng.uniform(-1, 1, (m.n_nodes, 1))
    asm = lm.GpuAssembly(lm.POISSON, 3 | lm.HIERARCHIC, 6, elem_coef=k, nodal_f=f)
    asm.init(m, dm)
    rp, ci = asm.sparsity()
    K, F = asm.assemble()
    asm.close()
    Kr, Fr, st, _ = orc.assemble(lm.POISSON, m.elem_type, 3 | 0x100, 6, m.xyz, m.conn, 1, dm.elem_dofs, dm.n_dofs,
                                 dm.constrained, rp, ci, coef=k, nodal_f=f)
    assert st == 0 and np.all(np.abs(K - Kr) <= k_tolerance(Kr, rp))
