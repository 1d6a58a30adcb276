"""ctypes binding of include/libmesh_gb300.h.

The native library is required: importing this module without a built
liblmg.so raises, there is no Python fallback for any entry point."""
import ctypes as C
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liblmg.so")

# status codes
OK, ERR_ARG, ERR_CUDA, ERR_STATE, ERR_DEGENERATE, ERR_BOUNDS, ERR_NEW_NONZERO, ERR_OOM, \
    ERR_UNSUPPORTED = range(9)
STATUS_NAMES = {0: "OK", 1: "ERR_ARG", 2: "ERR_CUDA", 3: "ERR_STATE", 4: "ERR_DEGENERATE",
                5: "ERR_BOUNDS", 6: "ERR_NEW_NONZERO", 7: "ERR_OOM", 8: "ERR_UNSUPPORTED"}
# element types (libMesh ElemType values)
TET4, TET10, HEX8, HEX27, PRISM6, PRISM18, TET14, PRISM21 = 8, 9, 10, 12, 13, 15, 34, 36
# forms and precisions
POISSON, ELASTICITY, ADVDIFF = 0, 1, 2
FP64, MIXED = 0, 1
# FE family flag OR'ed into fe_order
HIERARCHIC = 0x100
# work-space limit of lmg_cg_solve_noalloc
CG_NOALLOC_MAX_DOFS = 524288

_p = C.c_void_p
_i32, _i64, _u64, _f64 = C.c_int32, C.c_int64, C.c_uint64, C.c_double
_pi32, _pi64, _pf64 = C.POINTER(C.c_int32), C.POINTER(C.c_int64), C.POINTER(C.c_double)

# name -> (argtypes); every entry point returns lmg_status (int32)
SIGNATURES = {
    "lmg_mesh_cube": [_i32, _i32, _i32, _i32, _f64, _u64, C.POINTER(_p)],
    "lmg_mesh_info": [_p, _pi64, _pi64, _pi32, _pi32, _pi32],
    "lmg_mesh_copy": [_p, _p, _p, _p],
    "lmg_mesh_free": [_p],
    "lmg_dofmap_distribute": [_i64, _i64, _i32, _p, _i32, _pi64, _p],
    "lmg_dirichlet_dofs": [_i64, _i32, _i32, _p, _p, _p, _i32, _p, _i32, _i64, _p],
    "lmg_fe_dofs_per_elem": [_i32, _i32, _i32, _pi32],
    "lmg_dofmap_distribute_fe": [_i64, _i64, _i32, _p, _i32, _i32, _pi64, _p],
    "lmg_dofmap_distribute_device": [_i32, _i64, _i64, _i32, _p, _i32, _i32, _pi64, _p],
    "lmg_dirichlet_dofs_fe": [_i64, _i32, _i32, _i32, _p, _p, _p, _i32, _p, _i32, _i64, _p],
    "lmg_host_sparsity": [_i64, _i32, _i32, _i64, _p, _pi64, _p, _p],
    "lmg_mesh_refine": [_p, _i32, _f64, _u64],
    "lmg_mesh_tree": [_p, _pi64, _p, _p, _p, _p],
    "lmg_constraint_rows": [_p, _i32, _p, _i64, _p, _p, _p, _p, _p, _i64],
    "lmg_constraint_rows_device": [_p, _i32, _i32, _p, _i64, _p, _p, _p, _p, _p, _i64],
    "lmg_host_sparsity_constrained": [_i64, _i32, _i64, _p, _p, _p, _pi64, _p, _p],
    "lmg_context_create": [C.POINTER(_p), _i32],
    "lmg_context_destroy": [_p],
    "lmg_context_set_stream": [_p, _p],
    "lmg_mesh_upload": [_p, _i64, _p, _i64, _i32, _p],
    "lmg_dofmap_upload": [_p, _i32, _i64, _p],
    "lmg_dofmap_upload_fe": [_p, _i32, _i32, _i64, _p],
    "lmg_constraints_upload": [_p, _p],
    "lmg_constraint_rows_upload": [_p, _p, _p, _p, _p],
    "lmg_sparsity_build": [_p, _pi64],
    "lmg_sparsity_copy": [_p, _p, _p],
    "lmg_sparsity_on_device": [_p, _pi32],
    "lmg_context_set_plan_on_device": [_p, _i32],
    "lmg_plan_on_device": [_p, _pi32],
    "lmg_form_set": [_p, _i32, _i32, _i32, _p, _i32, _p, _p],
    "lmg_inputs_update": [_p, _p, _p, _p],
    "lmg_assemble": [_p, _i32, _p, _p, _i32],
    "lmg_result_device": [_p, C.POINTER(_p), C.POINTER(_p)],
    "lmg_synchronize": [_p],
    "lmg_result_copy": [_p, _p, _p],
    "lmg_last_error": [_p, _pi64, C.c_char_p, _i32],
    "lmg_cg_solve": [_p, _p, _p, _f64, _i32, _pi32, _pf64],
    "lmg_cg_solve_noalloc": [_i64, _p, _p, _p, _p, _p, _f64, _i32, _p, _pi32, _pf64, C.c_char_p, _i32],
    "lmg_qoi_region_load": [_p, _p, _p],
    "lmg_vjp_coef": [_p, _p, _p, _p],
    "lmg_residual": [_p, _p, _p, _i32],
    "lmg_vjp_xyz": [_p, _p, _p, _p, _p],
    "lmg_context_set_tensor_cores": [_p, _i32],
    "lmg_perflog_enable": [_p, _i32],
    "lmg_perflog_read": [_p, _pf64, _pf64, _pi64],
    "lmg_launch_count": [_p, _pi64],
    "lmg_context_set_grid": [_p, _i32],
    "lmg_batch_create": [C.POINTER(_p), _i32],
    "lmg_batch_destroy": [_p],
    "lmg_batch_add": [_p, _p],
    "lmg_batch_tune": [_p, _i32, _i32],
    "lmg_batch_assemble": [_p, _i32],
    "lmg_batch_synchronize": [_p, _pi64],
    "lmg_batch_info": [_p, C.POINTER(_p), _pi64, _p, _i32],
    "lmg_batch_set_persistent": [_p, _i32],
    "lmg_batch_last_error": [_p, C.c_char_p, _i32],
    "lmg_batch_persistent_info": [_p, _pi32, _pi32, _pi64],
    "lmg_probe_fp64": [_i32, _pf64],
    "lmg_probe_fp64_tensor": [_i32, _pf64],
    "lmg_probe_f2d": [_i32, _i64, _p, _p],
}

_lib = None


def lib():
    """Load liblmg.so (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "libmesh_gb300 native library missing (%s): run "
                "`python -c 'import __graft_entry__ as g; g.build()'`" % LIB_PATH)
        l = C.CDLL(LIB_PATH)
        for name, args in SIGNATURES.items():
            f = getattr(l, name)
            f.argtypes = args
            f.restype = C.c_int32
        _lib = l
    return _lib


class LmgError(RuntimeError):
    def __init__(self, status, msg="", elem=-1):
        self.status = status
        self.elem = elem
        super().__init__("%s (%d)%s%s" % (STATUS_NAMES.get(status, "?"), status,
                                          ": " + msg if msg else "",
                                          " [element %d]" % elem if elem >= 0 else ""))


class DegenerateMap(LmgError):
    """Mirror of libMesh::DegenerateMap: a Jacobian at or under tolerance."""


def check(status, ctx=None):
    if status == OK:
        return
    msg, elem = "", -1
    if ctx is not None:
        buf = C.create_string_buffer(512)
        e = C.c_int64(-1)
        lib().lmg_last_error(ctx, C.byref(e), buf, 512)
        msg, elem = buf.value.decode(errors="replace"), e.value
    cls = DegenerateMap if status == ERR_DEGENERATE else LmgError
    raise cls(status, msg, elem)


def ptr(a):
    """Raw data pointer of a contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)
