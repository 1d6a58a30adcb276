"""Mixed form on non-affine elements: the per-point B^T D B products as Gram
products E^T E on the tensor cores (tcgen05, BF16 three-way split, FP32
accumulation in tensor memory), against the FP64 drop-in, the CUDA-core mixed
path and the oracle.

Bar (the benchmark spec's tolerance for the mixed form): relative error of the
CG-solved field <= 1e-6 and relative Frobenius error of K <= 1e-6; F equals
the FP64 drop-in's bit for bit; repeated assemblies are bitwise identical."""
import numpy as np
import pytest

import libmesh_gb300 as lm
import oracle as orc
from helpers import make_problem

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def curved(n, et, nv, form, seed=1):
    """build_cube tets or hexes with every element non-affine: TET10 mid-edge
    nodes moved off their edges, or interior hex vertices jittered."""
    mesh, dm, k, f = make_problem(n, et, nv, form, jitter=0.2, seed=seed)
    if et == lm.TET10:
        rng = np.random.default_rng(seed + 10)
        mid = np.unique(mesh.conn[:, 4:])
        xyz = mesh.xyz.copy()
        inner = ~((xyz[mid] == 0) | (xyz[mid] == 1)).any(1)
        xyz[mid[inner]] += rng.uniform(-0.02, 0.02, (inner.sum(), 3)) / n
        mesh.xyz = xyz
    return mesh, dm, k, f


@pytest.mark.parametrize("et,nv,form,fo,qo,n", [(lm.TET10, 3, lm.ELASTICITY, 2, 4, 6),
                                                (lm.TET10, 1, lm.POISSON, 2, 4, 5),
                                                (lm.HEX8, 1, lm.POISSON, 1, 2, 8),
                                                (lm.TET4, 3, lm.ELASTICITY, 1, 2, 6)])
def test_tensor_core_mixed_form(et, nv, form, fo, qo, n):
    mesh, dm, k, f = curved(n, et, nv, form)
    aff = sum(orc.has_affine_map(et, x) for x in mesh.xyz[mesh.conn])
    assert et == lm.TET4 or aff < mesh.n_elem // 4
    asm = lm.GpuAssembly(form, fo, qo, elem_coef=k, nodal_f=f)
    asm.init(mesh, dm)
    rp, col = asm.sparsity()
    K64, F64 = asm.assemble(lm.FP64)
    u64, _, rr = asm.solve(rtol=1e-13, maxit=200000)
    K32, F32 = asm.assemble(lm.MIXED)
    K32b, F32b = asm.assemble(lm.MIXED)
    u32, _, rr32 = asm.solve(rtol=1e-13, maxit=200000)
    asm.set_tensor_cores(False)
    Kcc, Fcc = asm.assemble(lm.MIXED)
    asm.close()
    assert np.array_equal(K32, K32b) and np.array_equal(F32, F32b)
    assert np.array_equal(F32, F64)
    print("tensor-core mixed %d/%d: ||dK||/||K|| %.3g (CUDA-core mixed %.3g)  ||du||/||u|| %.3g"
          % (et, form, rel(K32, K64), rel(Kcc, K64), rel(u32, u64)))
    assert rel(K32, K64) < 1e-6
    assert rel(u32, u64) <= 1e-6
    # entry by entry: FP32-level agreement with the CUDA-core mixed path
    scale = np.maximum.reduceat(np.abs(K64), rp[:-1])[np.repeat(np.arange(dm.n_dofs), np.diff(rp))]
    assert np.max(np.abs(K32 - Kcc) / scale) < 1e-5
