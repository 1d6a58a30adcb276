"""Shared helpers for the parity tests."""
import numpy as np

import libmesh_gb300 as lm
import oracle as orc


def csr_rows(row_ptr):
    return np.repeat(np.arange(len(row_ptr) - 1), np.diff(row_ptr))


def k_tolerance(Kr, row_ptr, rel=1e-13):
    """Per-entry bound: rel * max(|K_ref_ij|, max_j |K_ref_ij| of the row).  The
    row-scale floor covers entries that vanish in exact arithmetic and come out
    as cancellation residue (~1e-17 of the row scale) in both codes."""
    rowmax = np.maximum.reduceat(np.abs(Kr), row_ptr[:-1]) if len(Kr) else np.zeros(0)
    return rel * np.maximum(np.abs(Kr), rowmax[csr_rows(row_ptr)])


def max_scaled_err(K, Kr, row_ptr):
    tol = k_tolerance(Kr, row_ptr, 1.0)
    return float(np.max(np.abs(K - Kr) / np.maximum(tol, 1e-300))) if len(K) else 0.0


def make_problem(n, et, nv, form, jitter=0.0, seed=1, bids=None, coef=True, load=True):
    mesh = lm.Mesh.build_cube(n, n, n, et, jitter=jitter, seed=seed)
    dm = lm.DofMap(mesh, nv)
    if bids is None:
        bids = [0, 1, 2, 3, 4, 5] if form == lm.POISSON else [4]
    if len(bids):
        dm.add_dirichlet_boundary(bids, list(range(nv)))
    rng = np.random.default_rng(seed)
    f = rng.uniform(-1, 1, (mesh.n_nodes, nv)) if load else None
    k = (np.exp(rng.normal(0, 0.5, mesh.n_elem)) if coef else None)
    return mesh, dm, k, f


def oracle_assemble(form, mesh, dm, fe_order, q_order, row_ptr, col, k, f, nu=0.3, n_threads=1):
    return orc.assemble(form, mesh.elem_type, fe_order, q_order, mesh.xyz, mesh.conn, dm.n_vars,
                        dm.elem_dofs, dm.n_dofs, dm.constrained, row_ptr, col, coef=k, nodal_f=f,
                        nu=nu, n_threads=n_threads)
