"""lmg_cg_solve_noalloc (work vectors in a fixed device array, no allocation)
against lmg_cg_solve on the same assembled systems, two calls in a row each,
through the C ABI.  Bar: |x - x_ref| <= 1e-13 max|x_ref| and the same
iteration count; the device's free memory (cudaMemGetInfo) is the same before
and after the second call, so that call allocated nothing."""
import ctypes as C

import numpy as np
import pytest

import libmesh_gb300 as lm
from libmesh_gb300 import _capi
from helpers import make_problem

pytestmark = pytest.mark.gpu


def _device_arrays(torch, asm):
    """CSR pattern and F on the device: row_ptr / col_idx uploaded by the test,
    K and F in the context's own buffers."""
    rp, ci = asm.sparsity()
    d_rp = torch.from_numpy(rp).cuda()
    d_ci = torch.from_numpy(ci).cuda()
    K, F = C.c_void_p(), C.c_void_p()
    _capi.check(_capi.lib().lmg_result_device(asm.ctx, C.byref(K), C.byref(F)), asm.ctx)
    return d_rp, d_ci, K.value, F.value


def _solve_noalloc(torch, n, d_rp, d_ci, k_ptr, f_ptr, x, rtol, maxit):
    it, rr = C.c_int32(), C.c_double()
    msg = C.create_string_buffer(256)
    st = _capi.lib().lmg_cg_solve_noalloc(n, C.c_void_p(d_rp.data_ptr()), C.c_void_p(d_ci.data_ptr()),
                                          C.c_void_p(k_ptr), C.c_void_p(f_ptr), C.c_void_p(x.data_ptr()),
                                          rtol, maxit, C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                          C.byref(it), C.byref(rr), msg, 256)
    assert st == _capi.OK, msg.value.decode()
    return x.cpu().numpy(), it.value, rr.value


@pytest.mark.parametrize("et,nv,form,fo,qo,n", [(lm.HEX8, 1, lm.POISSON, 1, 2, 10),
                                                (lm.TET10, 3, lm.ELASTICITY, 2, 4, 4)])
def test_noalloc_solve_matches_cg_solve(et, nv, form, fo, qo, n):
    torch = pytest.importorskip("torch")
    mesh, dm, k, f = make_problem(n, et, nv, form, jitter=0.1, seed=7)
    asm = lm.GpuAssembly(form, fo, qo, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    asm.assemble()
    rtol, maxit = 1e-10, 20000
    x_ref, it_ref, rr_ref = asm.solve(rtol=rtol, maxit=maxit)
    d_rp, d_ci, k_ptr, f_ptr = _device_arrays(torch, asm)
    asm.synchronize()
    scale = np.abs(x_ref).max()
    assert scale > 0
    xs_buf = [torch.full((dm.n_dofs,), np.nan, dtype=torch.float64, device="cuda") for _ in range(2)]
    torch.cuda.synchronize()
    for call, x in enumerate(xs_buf):
        free0 = torch.cuda.mem_get_info()[0]
        xs, it, rr = _solve_noalloc(torch, dm.n_dofs, d_rp, d_ci, k_ptr, f_ptr, x, rtol, maxit)
        if call == 1:  # the first call may load the library's module; the second must allocate nothing
            assert torch.cuda.mem_get_info()[0] == free0
        assert it == it_ref
        assert abs(rr - rr_ref) <= 1e-13 * max(rr_ref, 1e-300) + 1e-300
        assert np.max(np.abs(xs - x_ref)) <= 1e-13 * scale
    asm.close()


def test_noalloc_rejects_sizes_beyond_the_work_space():
    torch = pytest.importorskip("torch")
    lim = _capi.CG_NOALLOC_MAX_DOFS
    buf = torch.zeros(16, dtype=torch.float64, device="cuda")
    ibuf = torch.zeros(16, dtype=torch.int32, device="cuda")
    it, rr = C.c_int32(), C.c_double()
    msg = C.create_string_buffer(256)
    p, ip = C.c_void_p(buf.data_ptr()), C.c_void_p(ibuf.data_ptr())
    st = _capi.lib().lmg_cg_solve_noalloc(lim + 1, ip, ip, p, p, p, 1e-10, 10, None,
                                          C.byref(it), C.byref(rr), msg, 256)
    assert st == _capi.ERR_ARG
    assert b"exceeds" in msg.value and str(lim).encode() in msg.value


def test_noalloc_rejects_a_non_finite_right_hand_side():
    """NaN in the right-hand side: both solvers return LMG_ERR_ARG (no
    iterates reported as converged)."""
    torch = pytest.importorskip("torch")
    mesh, dm, k, f = make_problem(4, lm.HEX8, 1, lm.POISSON, seed=7)
    asm = lm.GpuAssembly(lm.POISSON, 1, 2, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    asm.assemble()
    d_rp, d_ci, k_ptr, _ = _device_arrays(torch, asm)
    asm.synchronize()
    rhs = np.ones(dm.n_dofs)
    rhs[3] = np.nan
    with pytest.raises(lm.LmgError) as ei:
        asm.solve(rhs=rhs, rtol=1e-10, maxit=100)
    assert ei.value.status == _capi.ERR_ARG
    d_rhs = torch.from_numpy(rhs).cuda()
    x = torch.zeros(dm.n_dofs, dtype=torch.float64, device="cuda")
    it, rr = C.c_int32(), C.c_double()
    msg = C.create_string_buffer(256)
    st = _capi.lib().lmg_cg_solve_noalloc(dm.n_dofs, C.c_void_p(d_rp.data_ptr()), C.c_void_p(d_ci.data_ptr()),
                                          C.c_void_p(k_ptr), C.c_void_p(d_rhs.data_ptr()),
                                          C.c_void_p(x.data_ptr()), 1e-10, 100,
                                          C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                          C.byref(it), C.byref(rr), msg, 256)
    assert st == _capi.ERR_ARG and b"not finite" in msg.value
    asm.close()
