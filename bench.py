"""Headline benchmark: finite-element assembly throughput (Melem/s) of 3-D linear
elasticity, QUADRATIC LAGRANGE TET10, QGauss FOURTH (Keast 11 points), on
build_cube 48^3 split into 6 tets per hex (663,552 elements, 2,738,019 dofs,
231,797,385 nonzeros), interior vertices jittered +-0.2h (seed 1), E_e ~
lognormal(0, 0.5), nu = 0.3, nodal body force ~ U[-1, 1], clamp on x = 0.

One step = one full assembly of K (CSR values) and F from zero through the C ABI.
`value` has the inputs resident on the device; `e2e` refreshes the per-step
inputs (E_e, f) from pinned host memory and copies K and F back to pinned host
memory inside the timed region.  `--impl reference` times the CPU restatement of
the reference's threaded assembly (FEMSystem-style element ranges, mutex-guarded
insertion) on the host cores.  Under torchrun every rank assembles its own
replica (assembly needs no exchange on one box): scaling "weak"."""
import argparse
import gc
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Melem/s assembled (FP64 drop-in vs mixed/batched at <=1e-6 rel err), % roofline"
N_CUBE = 48


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def build_problem(n=N_CUBE):
    import libmesh_gb300 as lm
    mesh = lm.Mesh.build_cube(n, n, n, lm.TET10, jitter=0.2, seed=1)
    dm = lm.DofMap(mesh, 3)
    dm.add_dirichlet_boundary([4], [0, 1, 2])
    rng = np.random.default_rng(1)
    E = np.exp(rng.normal(0.0, 0.5, mesh.n_elem))
    f = rng.uniform(-1.0, 1.0, (mesh.n_nodes, 3))
    return mesh, dm, E, f


def algorithmic(mesh, dm, nnz):
    """Unique bytes of one assembly, and flops per element (FMA = 2) of the
    reference's B^T D B form and of the affine reference-tensor form the FP64
    element kernel executes."""
    n_geo, n, q = 10, 10, 11
    B = 24 * mesh.n_nodes + 4 * mesh.n_elem * n_geo + 8 * dm.n_dofs + 8 * mesh.n_elem + 8 * nnz + 8 * dm.n_dofs
    ref_form = q * (2 * (6 * 6 * 3 * n + 3 * n * 3 * n * 6) + 18 * n) + q * (18 * n_geo + 60)
    blocks = n * (n + 1) // 2                      # diagonal + strictly upper 3x3 blocks
    ours = (2 * blocks * 9 * 9                     # K^{ik}_{ab} = sum_mn A^{ik}_{mn} S^{mn}_{ab}
            + 2 * 3 * n * n                        # Fe = detJ M f
            + 2 * 81 * 3 + 2 * 27                  # element tensor A (81 entries) and G G^T
            + 2 * n_geo * 9 + 60)                  # Jacobian at qp 0, det, inverse
    return B, ref_form, ours


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev):
        self.dev, self.proc, self.path = dev, None, None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        time.sleep(0.25)
        self.proc.terminate()
        self.proc.wait()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        os.unlink(self.path)
        if sm:
            out = {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                   "samples": len(sm)}
        return out


def cpu_sample(xyz, conn, elem_dofs, n_dofs, constrained, E, f, rp, col, threads, budget_s=12.0, n=None):
    """Times the oracle (restated reference assembly: FE::reinit per element,
    dense Ke, constrain_element_matrix_and_vector, CSR insertion by per-row
    binary search under one mutex) on elements [0, n) of the mesh.  Without n,
    a probe sizes the sample to about budget_s seconds.  Returns (Melem/s, n,
    seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    elasticity, tet10 = 1, 9            # LMG_ELASTICITY, libMesh TET10
    t = {}
    if n is None:
        probe = max(threads * 4, 64)
        orc.assemble(elasticity, tet10, 2, 4, xyz, conn, 3, elem_dofs, n_dofs, constrained, rp, col, coef=E,
                     nodal_f=f, n_threads=threads, e_range=(0, probe), timing=t)
        rate = probe / max(t["seconds"], 1e-6)
        n = int(min(conn.shape[0], max(probe, rate * budget_s)))
    orc.assemble(elasticity, tet10, 2, 4, xyz, conn, 3, elem_dofs, n_dofs, constrained, rp, col, coef=E,
                 nodal_f=f, n_threads=threads, e_range=(0, n), timing=t)
    return n / t["seconds"] / 1e6, n, t["seconds"]


def oracle_problem(n=N_CUBE):
    """The headline problem built by the oracle alone (restated build_cube ->
    jitter -> all_tri -> all_second_order, dof numbering, Dirichlet set and
    compute_sparsity), with the same seeded E_e and f as build_problem."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as orc
    tet10 = 9
    xyz, conn, side_bid = orc.mesh_cube(n, tet10, 0.2, 1)
    elem_dofs, n_dofs = orc.distribute_dofs(xyz.shape[0], conn, 3)
    constrained = orc.dirichlet(tet10, 3, elem_dofs, side_bid, [4], [0, 1, 2], n_dofs)
    rp, col = orc.sparsity(n_dofs, elem_dofs)
    rng = np.random.default_rng(1)
    E = np.exp(rng.normal(0.0, 0.5, conn.shape[0]))
    f = rng.uniform(-1.0, 1.0, (xyz.shape[0], 3))
    return xyz, conn, elem_dofs, n_dofs, constrained, rp, col, E, f


def run_reference(args, rank):
    """The reference arm: the CPU restatement of libMesh's threaded assembly
    (the reference itself cannot be built here) on all host cores.  Mesh, dof
    map, constraints and sparsity come from the oracle too, so nothing of the
    product is loaded.  One step assembles a contiguous element sample of the
    headline mesh sized to about 2 s; ms_per_step is that sample's measured
    time and value the best of the timed steps (Melem/s, the same metric and
    config as the GPU arm).  A 1-thread rate on a smaller sample is reported
    beside it."""
    if rank != 0:
        return
    prob = oracle_problem(args.n)
    xyz, conn, elem_dofs, n_dofs, constrained, rp, col, E, f = prob
    cores = os.cpu_count() or 1
    budget = max(0.5, min(2.0, 100.0 / max(1, args.steps + args.warmup)))
    _, n, _ = cpu_sample(*prob[:5], E, f, rp, col, cores, budget_s=budget)
    rates, secs = [], []
    for i in range(args.warmup + args.steps):
        v, _, sec = cpu_sample(xyz, conn, elem_dofs, n_dofs, constrained, E, f, rp, col, cores, n=n)
        if i >= args.warmup:
            rates.append(v)
            secs.append(sec)
    v1, n1, s1 = cpu_sample(xyz, conn, elem_dofs, n_dofs, constrained, E, f, rp, col, 1, budget_s=budget)
    best, ms = float(max(rates)), float(np.median(secs)) * 1e3
    sample = ("elements [0, %d) of the %d-element mesh per step (%.2f s), %d threads; value = best of %d steps"
              % (n, conn.shape[0], ms * 1e-3, cores, len(rates)))
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": best, "unit": "Melem/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded mesh jitter, E_e, f)",
        "config": {"workload": "elasticity TET10 build_cube %d^3 x6 tets, QGauss FOURTH" % args.n,
                   "n_elem": int(conn.shape[0]), "n_dofs": int(n_dofs), "nnz": int(len(col))},
        "cpu_baseline": {"value": best, "unit": "Melem/s", "cores": cores, "kind": "port", "sample": sample,
                         "median": float(np.median(rates)),
                         "one_thread": {"value": v1, "unit": "Melem/s", "cores": 1,
                                        "sample": "elements [0, %d), %.2f s" % (n1, s1)}},
        "e2e": {"value": best, "unit": "Melem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def cd_params(seed=3, n_modes=8, kappa=1e-2):
    """Convection-diffusion data: kappa and the modes of the streamfunction
    psi = sum_m a_m sin(k_m . x + phase_m), b = curl psi (divergence-free)."""
    rng = np.random.default_rng(seed)
    p = [kappa, n_modes]
    for _ in range(n_modes):
        p += list(rng.uniform(-1, 1, 3)) + list(2 * np.pi * rng.uniform(-1.5, 1.5, 3)) + [rng.uniform(0, 2 * np.pi)]
    return np.array(p)


def run_amr(args, local):
    """Secondary workload: steady convection-diffusion, SECOND LAGRANGE HEX27,
    QGauss FIFTH, on build_cube(n^3, HEX27) after 3 cycles of refining 20% of
    the active elements (level-one rule), hanging-node and Dirichlet
    constraints applied through C^T K C.  Same JSON keys as the headline."""
    import torch
    import libmesh_gb300 as lm
    torch.cuda.set_device(local)
    t0 = time.perf_counter()
    n = 24 if args.n == N_CUBE else args.n      # build_cube 24^3 HEX27 unless --n is given
    mesh = lm.Mesh.build_refined_cube(n, lm.HEX27, 3, 0.2, 2)
    t_mesh = time.perf_counter() - t0
    t1 = time.perf_counter()
    dm = lm.DofMap(mesh, 1)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    t_dofmap = time.perf_counter() - t1
    dm_host = lm.DofMap(mesh, 1)
    dm_host.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    t1 = time.perf_counter()
    dm_host.create_dof_constraints()            # hanging-node rows on the host (timed for comparison)
    t_rows_host = time.perf_counter() - t1
    t1 = time.perf_counter()
    dm.create_dof_constraints(device=local)     # the same rows formed on the GPU
    t_rows_dev = time.perf_counter() - t1
    del dm_host
    t0 += t_rows_host
    rng = np.random.default_rng(2)
    k = np.exp(rng.normal(0.0, 0.5, mesh.n_elem))
    f = rng.uniform(-1.0, 1.0, (mesh.n_nodes, 1))
    asm = lm.GpuAssembly(lm.ADVDIFF, 2, 5, elem_coef=k, nodal_f=f, params=cd_params(), device=local)
    t1 = time.perf_counter()
    asm.init(mesh, dm)                  # uploads, constrained sparsity on the device
    t_init = time.perf_counter() - t1
    stream = torch.cuda.current_stream()
    asm.set_stream(stream.cuda_stream)
    t1 = time.perf_counter()
    asm.assemble_device(lm.FP64)        # builds the slot plan
    asm.synchronize()
    t_first = time.perf_counter() - t1
    setup_s = time.perf_counter() - t0
    for _ in range(max(3, args.warmup)):
        asm.assemble_device(lm.FP64)
    asm.synchronize()
    clocks = Clocks(local)
    clocks.start()
    torch.cuda.synchronize()
    l0 = asm.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        asm.assemble_device(lm.FP64)
    ev1.record(stream)
    ev1.synchronize()
    asm.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = asm.launch_count() - l0
    clk = clocks.stop()
    asm.perflog_enable(True)
    for _ in range(5):
        asm.assemble_device(lm.FP64)
    el_ms, ga_ms, calls = asm.perflog_read()
    asm.perflog_enable(False)
    # the mixed form (FP32 contraction and constraint products, FP64 map and sums), same inputs
    asm.assemble_device(lm.MIXED)
    asm.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        asm.assemble_device(lm.MIXED)
    ev1.record(stream)
    ev1.synchronize()
    asm.synchronize()
    ms32 = ev0.elapsed_time(ev1) / args.steps
    K32 = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
    K64 = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
    F32 = torch.empty(dm.n_dofs, dtype=torch.float64, device="cuda")
    F64 = torch.empty(dm.n_dofs, dtype=torch.float64, device="cuda")
    asm.assemble_device(lm.MIXED, K32.data_ptr(), F32.data_ptr())
    asm.assemble_device(lm.FP64, K64.data_ptr(), F64.data_ptr())
    asm.synchronize()
    mixed = {"form": "mixed (FP32 contraction and constraint products, FP64 map and global sums)",
             "value": mesh.n_elem / (ms32 * 1e-3) / 1e6, "unit": "Melem/s", "ms_per_step": ms32,
             "speedup_vs_fp64": ms / ms32,
             "k_rel_frobenius_vs_fp64": float(torch.linalg.norm(K32 - K64) / torch.linalg.norm(K64)),
             "f_rel_vs_fp64": float(torch.linalg.norm(F32 - F64) / torch.linalg.norm(F64))}
    del K32, K64, F32, F64
    Kh = torch.empty(asm.nnz, dtype=torch.float64, pin_memory=True)
    Fh = torch.empty(dm.n_dofs, dtype=torch.float64, pin_memory=True)
    kh = torch.from_numpy(k).pin_memory()
    t1 = time.perf_counter()
    n_e2e = max(3, min(args.steps, 5))
    for _ in range(n_e2e):
        asm.update_inputs(elem_coef=kh.numpy())
        asm.assemble_into(Kh.data_ptr(), Fh.data_ptr(), lm.FP64)
    e2e_s = (time.perf_counter() - t1) / n_e2e
    asm.close()
    n_cons = int(dm.constrained[dm.elem_dofs].any(1).sum())
    print(json.dumps({
        "metric": METRIC, "value": mesh.n_elem / (ms * 1e-3) / 1e6, "unit": "Melem/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded refinement, k_e, f, b)",
        "setup_breakdown_s": {"refined_mesh": t_mesh, "dof_map": t_dofmap, "constraint_rows_host": t_rows_host,
                              "constraint_rows_device": t_rows_dev, "init_uploads_sparsity": t_init,
                              "slot_plan_and_first_assembly": t_first},
        "config": {"workload": "convection-diffusion HEX27 build_cube %d^3, 3 cycles x 20%% h-refinement, "
                               "QGauss FIFTH, hanging-node + Dirichlet constraints" % n,
                   "n_elem": mesh.n_elem, "n_dofs": dm.n_dofs, "nnz": asm.nnz, "constrained_elements": n_cons,
                   "setup_s": setup_s, "l2": "inputs larger than L2"},
        "e2e": {"value": mesh.n_elem / e2e_s / 1e6, "unit": "Melem/s", "h2d_bytes_per_step": 8 * mesh.n_elem,
                "d2h_bytes_per_step": 8 * (asm.nnz + dm.n_dofs)},
        "gpu_launches": launches, "clocks": clk, "mixed": mixed,
        "stages_ms": {"elements_and_constraints": el_ms / calls, "insertion": ga_ms / calls}}))


BATCH_KINDS = [  # (element, HIERARCHIC order, QGauss order, elements per grid cell)
    (10, 1, 3, 1),   # HEX8   FIRST
    (12, 2, 5, 1),   # HEX27  SECOND
    (12, 3, 7, 1),   # HEX27  THIRD
    (8, 1, 2, 6),    # TET4   FIRST
    (9, 2, 4, 6),    # TET10  SECOND
    (13, 1, 3, 2),   # PRISM6 FIRST
    (15, 2, 4, 2),   # PRISM18 SECOND
    (36, 3, 5, 2),   # PRISM21 THIRD
    (34, 3, 6, 6),   # TET14  THIRD
]


def batch_members(n_meshes, seed=3, lo=1e3, hi=5e4):
    """The config-4 mix, scaled: meshes with log-uniform element counts in
    [lo, hi], cycling through HIERARCHIC hexes (p = 1, 2, 3), tets (p = 1, 2, 3)
    and prisms (p = 1), Poisson with k_e ~ U[0.1, 10], Dirichlet on every side."""
    import libmesh_gb300 as lm
    rng = np.random.default_rng(seed)
    sizes = np.exp(rng.uniform(np.log(lo), np.log(hi), n_meshes))
    out = []
    for i, s in enumerate(sizes):
        et, p, qo, per_cell = BATCH_KINDS[i % len(BATCH_KINDS)]
        n = max(2, int(round((s / per_cell) ** (1.0 / 3.0))))
        mesh = lm.Mesh.build_cube(n, n, n, et)
        fo = p | lm.HIERARCHIC
        dm = lm.DofMap(mesh, 1, fe_order=fo)
        dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
        k = rng.uniform(0.1, 10.0, mesh.n_elem)
        f = rng.uniform(-1.0, 1.0, (mesh.n_nodes, 1))
        a = lm.GpuAssembly(lm.POISSON, fo, qo, elem_coef=k, nodal_f=f)
        a.init(mesh, dm)
        out.append((a, mesh.n_elem))
    return out


def run_batch(args, local):
    """Secondary workload: many independent systems of mixed element types,
    forms and FE families, assembled (a) through the C ABI, each system on its
    own stream, (b) as one tuned CUDA graph (lmg_batch_*), and (c) one system
    after another on one stream."""
    import torch
    import libmesh_gb300 as lm
    torch.cuda.set_device(local)
    n_meshes = args.meshes
    t0 = time.perf_counter()
    mem = batch_members(n_meshes, hi=args.max_elems)
    setup_s = time.perf_counter() - t0
    total = sum(e for _, e in mem)
    # (a) one after another, default grids
    for a, _ in mem:
        a.assemble_device(lm.FP64)
    for a, _ in mem:
        a.synchronize()
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(args.steps):
        for a, _ in mem:
            a.assemble_device(lm.FP64)
        for a, _ in mem:
            a.synchronize()
    seq_ms = (time.perf_counter() - t1) * 1e3 / args.steps
    # (b) one graph, tuned grids
    b = lm.Batch(local)
    for a, _ in mem:
        b.add(a)
    t2 = time.perf_counter()
    b.tune(lm.FP64, reps=2)
    tune_s = time.perf_counter() - t2
    for _ in range(max(3, args.warmup)):
        b.assemble(lm.FP64)
    b.synchronize()
    sptr, launches, grids = b.info()
    stream = torch.cuda.ExternalStream(sptr)
    clocks = Clocks(local)
    clocks.start()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        b.assemble(lm.FP64)
    ev1.record(stream)
    ev1.synchronize()
    b.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    clk = clocks.stop()
    # the mixed form through the same graph machinery, tuned for it
    b.tune(lm.MIXED, reps=2)
    for _ in range(max(3, args.warmup)):
        b.assemble(lm.MIXED)
    b.synchronize()
    ev0.record(stream)
    for _ in range(args.steps):
        b.assemble(lm.MIXED)
    ev1.record(stream)
    ev1.synchronize()
    b.synchronize()
    ms32 = ev0.elapsed_time(ev1) / args.steps
    persist, hybrid = None, None
    if not args.no_persistent:
        # one persistent launch per replay (every member's tiles and insertion from one queue)
        persist = {}
        b.set_persistent(True)
        for prec, key in ((lm.FP64, "fp64"), (lm.MIXED, "mixed")):
            b.tune(prec, reps=2)
            for _ in range(max(3, args.warmup)):
                b.assemble(prec)
            b.synchronize()
            ev0.record(stream)
            for _ in range(args.steps):
                b.assemble(prec)
            ev1.record(stream)
            ev1.synchronize()
            b.synchronize()
            tile, ctas, items = b.persistent_info()
            pms = ev0.elapsed_time(ev1) / args.steps
            persist[key] = {"ms_per_step": pms, "value": total / (pms * 1e-3) / 1e6, "unit": "Melem/s",
                            "tile_elements_per_cta": tile, "ctas_per_sm": ctas or "occupancy", "work_items": items}
        persist["launches_per_replay"] = 1
        persist["mixed_speedup_vs_fp64"] = persist["fp64"]["ms_per_step"] / persist["mixed"]["ms_per_step"]
        # hybrid: one persistent launch over the per-pattern members, the others' own kernels beside it
        hybrid = {}
        b.set_persistent(True, hybrid=True)
        for prec, key in ((lm.FP64, "fp64"), (lm.MIXED, "mixed")):
            b.tune(prec, reps=2)
            for _ in range(max(3, args.warmup)):
                b.assemble(prec)
            b.synchronize()
            ev0.record(stream)
            for _ in range(args.steps):
                b.assemble(prec)
            ev1.record(stream)
            ev1.synchronize()
            b.synchronize()
            hms = ev0.elapsed_time(ev1) / args.steps
            _, hl, _ = b.info()
            hybrid[key] = {"ms_per_step": hms, "value": total / (hms * 1e-3) / 1e6, "unit": "Melem/s",
                           "launches_per_replay": hl}
        hybrid["mixed_speedup_vs_fp64"] = hybrid["fp64"]["ms_per_step"] / hybrid["mixed"]["ms_per_step"]
        hybrid["vs_graph"] = ms / hybrid["fp64"]["ms_per_step"]
    b.close()
    # (c) one system after another on one stream, as System::assemble is
    # called for each system in turn (the tuned grids of the graph)
    one = torch.cuda.Stream()
    for a, _ in mem:
        a.set_stream(one.cuda_stream)
    for _ in range(max(3, args.warmup)):
        for a, _ in mem:
            a.assemble_device(lm.FP64)
    one.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(one)
    for _ in range(args.steps):
        for a, _ in mem:
            a.assemble_device(lm.FP64)
    ev1.record(one)
    ev1.synchronize()
    serial_ms = ev0.elapsed_time(ev1) / args.steps
    n_dofs_total = sum(a.dof_map.n_dofs for a, _ in mem)
    for a, _ in mem:
        a.close()
    print(json.dumps({
        "metric": METRIC, "value": total / (ms * 1e-3) / 1e6, "unit": "Melem/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "double-float (FP32 pairs) contraction, FP64 geometry, FP64 / double-float sums",
        "data": "synthetic (seeded sizes, coefficients, loads)",
        "config": {"workload": "batch of %d systems (config-4 mix), element counts log-uniform in "
                               "[1e3, %.0e]: HIERARCHIC Poisson on HEX8 p1, HEX27 p2, HEX27 p3, TET4 p1, TET10 p2, "
                               "PRISM6 p1, PRISM18 p2, PRISM21 p3, TET14 p3, k_e ~ U[0.1, 10]" % (n_meshes, args.max_elems),
                   "total_elements": total, "total_dofs": n_dofs_total,
                   "setup_s": setup_s, "tune_s": tune_s},
        "sequential": {"ms_per_step": seq_ms, "value": total / (seq_ms * 1e-3) / 1e6, "unit": "Melem/s",
                       "how": "lmg_assemble per system on its own stream, host loop, default grids"},
        "serial_one_stream": {"ms_per_step": serial_ms, "value": total / (serial_ms * 1e-3) / 1e6,
                              "unit": "Melem/s", "graph_speedup": serial_ms / ms,
                              "how": "lmg_assemble per system in turn on one stream (System::assemble one "
                                     "after another), tuned grids"},
        "mixed": {"ms_per_step": ms32, "value": total / (ms32 * 1e-3) / 1e6, "unit": "Melem/s",
                  "speedup_vs_fp64": ms / ms32},
        "persistent": persist,
        "persistent_hybrid": hybrid,
        "graph_speedup": seq_ms / ms, "gpu_launches": launches * args.steps, "launches_per_replay": launches,
        "tuned_ctas_per_sm": {str(g): int((grids == g).sum()) for g in sorted(set(grids.tolist()))},
        "clocks": clk}))


def run_adjoint(args, local):
    """Secondary workload: adjoint sensitivities of q(u) = integral of u over
    x < 0.25 to all element coefficients, Poisson on build_cube 128^3 HEX8
    (2,097,152 elements), k_e = exp(N(0,1)): assembly, primal and adjoint CG
    (Jacobi, rtol 1e-10), QoI load, one VJP pass.  The reference perturbs each
    parameter and assembles the residual twice per parameter."""
    import torch
    import libmesh_gb300 as lm
    torch.cuda.set_device(local)
    n = 128 if args.n == N_CUBE else args.n
    mesh = lm.Mesh.build_cube(n, n, n, lm.HEX8)
    dm = lm.DofMap(mesh, 1)
    dm.add_dirichlet_boundary([0, 1, 2, 3, 4, 5], [0])
    rng = np.random.default_rng(4)
    k = np.exp(rng.normal(0.0, 1.0, mesh.n_elem))
    f = rng.uniform(-1.0, 1.0, (mesh.n_nodes, 1))
    region = (mesh.xyz[mesh.conn][:, :, 0].mean(1) < 0.25).astype(np.uint8)
    asm = lm.GpuAssembly(lm.POISSON, 1, 2, elem_coef=k, nodal_f=f, device=local)
    asm.init(mesh, dm)
    asm.assemble()
    t = {}
    t0 = time.perf_counter()
    asm.assemble_device(lm.FP64)
    asm.synchronize()
    t["assemble_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    u, it_u, rr_u = asm.solve(rtol=1e-10, maxit=100000)
    t["primal_solve_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    qv = asm.qoi_region_load(region)
    t["qoi_load_s"] = time.perf_counter() - t0
    t0 = time.perf_counter()
    z, it_z, rr_z = asm.solve(rhs=qv, rtol=1e-10, maxit=100000)
    t["adjoint_solve_s"] = time.perf_counter() - t0
    asm.vjp_coef(u, z)
    vj = []
    for _ in range(max(1, args.steps)):
        t0 = time.perf_counter()
        g = asm.vjp_coef(u, z)
        vj.append(time.perf_counter() - t0)
    t["vjp_s"] = float(np.median(vj))
    t0 = time.perf_counter()
    gx = asm.vjp_xyz(u, z, region)
    t["vjp_xyz_s"] = time.perf_counter() - t0
    asm.close()
    total = sum(t.values())
    print(json.dumps({
        "metric": "element-coefficient sensitivities per second (adjoint VJP)", "value": mesh.n_elem / total,
        "unit": "params/s", "n_gpus": 1, "steps": args.steps, "warmup": 1, "ms_per_step": total * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded k_e, f)",
        "config": {"workload": "adjoint_qoi_parameter_sensitivity, Poisson HEX8 build_cube %d^3, QoI = int_{x<0.25} u"
                               % n, "n_elem": mesh.n_elem, "n_dofs": dm.n_dofs, "nnz": asm.nnz,
                   "cg_iterations": [it_u, it_z], "relres": [rr_u, rr_z]},
        "stages_s": t, "vjp_melem_per_s": mesh.n_elem / t["vjp_s"] / 1e6,
        "q": float(qv @ u), "grad_norm": float(np.linalg.norm(g)), "coord_grad_norm": float(np.linalg.norm(gx)),
        "e2e_note": "host timers around the public calls; u, z, q and the gradient cross the host boundary"}))


def run_curved(args, local):
    """Secondary workload: the headline elasticity problem with every TET10
    non-affine (mid-edge nodes moved off their edges by up to 0.005 h), so every
    element takes the reference's per-point form.  Times the FP64 drop-in and
    the mixed form with the per-point Gram products on the tensor cores and on
    the CUDA cores."""
    import torch
    import libmesh_gb300 as lm
    torch.cuda.set_device(local)
    mesh, dm, E, f = build_problem(args.n)
    rng = np.random.default_rng(11)
    mid = np.unique(mesh.conn[:, 4:])
    xyz = mesh.xyz.copy()
    inner = ~((xyz[mid] == 0) | (xyz[mid] == 1)).any(1)
    xyz[mid[inner]] += rng.uniform(-0.005, 0.005, (inner.sum(), 3)) / args.n
    mesh.xyz = xyz
    asm = lm.GpuAssembly(lm.ELASTICITY, 2, 4, elem_coef=E, nodal_f=f, nu=0.3, device=local)
    asm.init(mesh, dm)
    stream = torch.cuda.current_stream()
    asm.set_stream(stream.cuda_stream)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(prec, tc=True):
        asm.set_tensor_cores(tc)
        for _ in range(max(3, args.warmup)):
            asm.assemble_device(prec)
        asm.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            asm.assemble_device(prec)
        ev1.record(stream)
        ev1.synchronize()
        asm.synchronize()
        return ev0.elapsed_time(ev1) / args.steps

    clocks = Clocks(local)
    clocks.start()
    ms64 = timed(lm.FP64)
    clk = clocks.stop()
    ms_tc = timed(lm.MIXED, True)
    ms_cc = timed(lm.MIXED, False)
    Ks = {}
    for name, prec, tc in (("fp64", lm.FP64, True), ("tc", lm.MIXED, True), ("cc", lm.MIXED, False)):
        asm.set_tensor_cores(tc)
        Kd = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
        Fd = torch.empty(dm.n_dofs, dtype=torch.float64, device="cuda")
        asm.assemble_device(prec, Kd.data_ptr(), Fd.data_ptr())
        asm.synchronize()
        Ks[name] = Kd
    asm.perflog_enable(True)
    asm.set_tensor_cores(True)
    for _ in range(5):
        asm.assemble_device(lm.MIXED)
    el_ms, ga_ms, calls = asm.perflog_read()
    asm.close()
    n_el = mesh.n_elem
    rk = lambda a: float(torch.linalg.norm(Ks[a] - Ks["fp64"]) / torch.linalg.norm(Ks["fp64"]))  # noqa: E731
    print(json.dumps({
        "metric": METRIC, "value": n_el / (ms64 * 1e-3) / 1e6, "unit": "Melem/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms64, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded mesh jitter, mid-edge offsets, E_e, f)",
        "config": {"workload": "elasticity TET10 build_cube %d^3 x6 tets, mid-edge nodes moved (every element "
                               "non-affine), QGauss FOURTH" % args.n, "n_elem": n_el, "n_dofs": dm.n_dofs},
        "clocks": clk,
        "mixed_tensor_cores": {"ms_per_step": ms_tc, "value": n_el / (ms_tc * 1e-3) / 1e6,
                               "speedup_vs_fp64": ms64 / ms_tc, "k_rel_frobenius_vs_fp64": rk("tc"),
                               "stages_ms": {"elements": el_ms / calls, "insertion": ga_ms / calls}},
        "mixed_cuda_cores": {"ms_per_step": ms_cc, "value": n_el / (ms_cc * 1e-3) / 1e6,
                             "speedup_vs_fp64": ms64 / ms_cc, "k_rel_frobenius_vs_fp64": rk("cc")}}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the cpu_baseline leg")
    ap.add_argument("--n", type=int, default=N_CUBE, help="cube divisions (48 = the headline mesh)")
    ap.add_argument("--no-mixed", action="store_true", help="skip timing the mixed form beside FP64")
    ap.add_argument("--no-persistent", action="store_true",
                    help="batch workload: skip the persistent-launch legs (e.g. for a launch list of the graph)")
    ap.add_argument("--workload", default="elasticity",
                    choices=["elasticity", "amr-cd", "batch", "adjoint", "curved"],
                    help="elasticity = the headline; amr-cd = refined HEX27 convection-diffusion; "
                         "batch = many mixed systems as one CUDA graph; adjoint = 128^3 sensitivities; "
                         "curved = the headline mesh with every element non-affine")
    ap.add_argument("--meshes", type=int, default=64, help="systems in the batch workload")
    ap.add_argument("--max-elems", type=float, default=5e4,
                    help="largest system of the batch workload (2e5 with --meshes 256 is the full config-4 mix)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if args.impl == "reference":
        return run_reference(args, rank)
    if args.workload in ("amr-cd", "batch", "adjoint", "curved"):
        from libmesh_gb300 import _build
        _build.build()
        return {"amr-cd": run_amr, "batch": run_batch, "adjoint": run_adjoint,
                "curved": run_curved}[args.workload](args, local)

    import torch
    import libmesh_gb300 as lm
    from libmesh_gb300 import _build
    _build.build()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    prec = lm.FP64 if args.precision == "fp64" else lm.MIXED
    setup = {}
    t0 = time.perf_counter()
    mesh, dm, E, f = build_problem(args.n)
    setup["mesh_dofmap_s"] = time.perf_counter() - t0
    asm = lm.GpuAssembly(lm.ELASTICITY, 2, 4, elem_coef=E, nodal_f=f, nu=0.3, device=local)
    t0 = time.perf_counter()
    asm.init(mesh, dm)                  # upload, sparsity (device block graph), reference tensors
    setup["init_s"] = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    asm.set_stream(stream.cuda_stream)
    t0 = time.perf_counter()
    asm.assemble_device(prec)           # the first call builds the slot plan
    asm.synchronize()
    setup["first_assembly_s"] = time.perf_counter() - t0
    # the timed legs below run without the harness's garbage collector (a
    # collection pause on the host would stall the launch queue)
    gc.collect()
    gc.disable()
    for _ in range(max(3, args.warmup)):
        asm.assemble_device(prec)
    asm.synchronize()

    clocks = Clocks(local)
    clocks.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    l0 = asm.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        asm.assemble_device(prec)
    ev1.record(stream)
    ev1.synchronize()
    asm.synchronize()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / args.steps
    launches = asm.launch_count() - l0
    clk = clocks.stop()
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = world * mesh.n_elem / (ms * 1e-3) / 1e6

    # the other form, timed the same way on the same inputs
    other = None
    if not args.no_mixed and prec == lm.FP64:
        asm.assemble_device(lm.MIXED)
        asm.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            asm.assemble_device(lm.MIXED)
        ev1.record(stream)
        ev1.synchronize()
        asm.synchronize()
        ms32 = ev0.elapsed_time(ev1) / args.steps
        K32 = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
        K64 = torch.empty(asm.nnz, dtype=torch.float64, device="cuda")
        F32 = torch.empty(dm.n_dofs, dtype=torch.float64, device="cuda")
        F64 = torch.empty(dm.n_dofs, dtype=torch.float64, device="cuda")
        asm.assemble_device(lm.MIXED, K32.data_ptr(), F32.data_ptr())
        asm.assemble_device(lm.FP64, K64.data_ptr(), F64.data_ptr())
        asm.synchronize()
        krel = float(torch.linalg.norm(K32 - K64) / torch.linalg.norm(K64))
        frel = float(torch.linalg.norm(F32 - F64) / torch.linalg.norm(F64))
        del K32, K64, F32, F64
        other = {"form": "mixed (FP32 contraction, FP64 Jacobian/diagonal/accumulation)",
                 "value": world * mesh.n_elem / (ms32 * 1e-3) / 1e6, "unit": "Melem/s", "ms_per_step": ms32,
                 "speedup_vs_fp64": ms / ms32, "k_rel_frobenius_vs_fp64": krel, "f_rel_vs_fp64": frel,
                 "solved_field": "relative error of the CG-solved field against the FP64 solve: "
                                 "tests/test_gpu_full_size.py (C2 at full size, bar 1e-6)"}

    # matrix-free residual R = K u - F (no K), against assembling K and one product
    resid = None
    if prec == lm.FP64:
        ud = torch.randn(dm.n_dofs, dtype=torch.float64, device="cuda")
        Rd = torch.empty(dm.n_dofs, dtype=torch.float64, device="cuda")
        for _ in range(2):
            asm.residual_device(ud.data_ptr(), Rd.data_ptr())
        asm.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            asm.residual_device(ud.data_ptr(), Rd.data_ptr())
        ev1.record(stream)
        ev1.synchronize()
        asm.synchronize()
        rms = ev0.elapsed_time(ev1) / args.steps
        resid = {"what": "R = K u - F without forming K (lmg_residual, device vectors)", "ms_per_step": rms,
                 "value": world * mesh.n_elem / (rms * 1e-3) / 1e6, "unit": "Melem/s",
                 "vs_assembly": ms / rms}
        del ud, Rd

    # per-stage times (PerfLog events) for the roofline
    asm.perflog_enable(True)
    for _ in range(5):
        asm.assemble_device(prec)
    el_ms, ga_ms, calls = asm.perflog_read()
    asm.perflog_enable(False)
    el_ms, ga_ms = el_ms / calls, ga_ms / calls

    # end to end through the C ABI with host buffers
    Kh = torch.empty(asm.nnz, dtype=torch.float64, pin_memory=True)
    Fh = torch.empty(dm.n_dofs, dtype=torch.float64, pin_memory=True)
    Eh = torch.from_numpy(E).pin_memory()
    fh = torch.from_numpy(np.ascontiguousarray(f)).pin_memory()
    e2e_steps = max(3, min(args.steps, 10))
    for _ in range(2):
        asm.update_inputs(elem_coef=Eh.numpy(), nodal_f=fh.numpy())
        asm.assemble_into(Kh.data_ptr(), Fh.data_ptr(), prec)
    if dist:
        dist.barrier()
    # host timers around the C-ABI calls (still without the garbage collector)
    t0 = time.perf_counter()
    e2e_ms = []
    for _ in range(e2e_steps):
        t1 = time.perf_counter()
        asm.update_inputs(elem_coef=Eh.numpy(), nodal_f=fh.numpy())
        asm.assemble_into(Kh.data_ptr(), Fh.data_ptr(), prec)
        e2e_ms.append(1e3 * (time.perf_counter() - t1))
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if dist:
        t = torch.tensor([e2e_s], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e = world * mesh.n_elem / e2e_s / 1e6
    # the device-to-host link alone: plain copies of K's size into the same
    # pinned buffer, the fastest of five (one copy disturbed by other work on
    # the shared host would otherwise set the floor)
    Kd = torch.empty(asm.nnz, dtype=torch.float64, device=local)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    copy_ms = []
    for r in range(5):
        ev0.record()
        Kh.copy_(Kd, non_blocking=True)
        ev1.record()
        ev1.synchronize()
        copy_ms.append(ev0.elapsed_time(ev1))
    link_gbs = 8 * asm.nnz / (min(copy_ms) * 1e-3) / 1e9
    del Kd

    B, ref_flops, our_flops = algorithmic(mesh, dm, asm.nnz)
    hbm, hbm_src = peaks()
    fp64 = lm.probe_fp64(local)
    fp64_tc = lm.probe_fp64_tensor(local)
    if el_ms >= ga_ms:
        dom = {"kernel": "k_elem_affine<ELASTICITY,10,3,double>", "bound": "fp64", "unit": "TFLOP/s",
               "achieved": our_flops * mesh.n_elem / (el_ms * 1e-3) / 1e12, "peak": fp64,
               "peak_source": "measured FP64 DFMA probe (lmg_probe_fp64) in this run",
               "flops_per_elem": our_flops, "reference_form_flops_per_elem": ref_flops}
    else:
        # algorithmic bytes the insertion owns: the K and F it writes (8 B per
        # nonzero and per dof); the element blocks it reads are implementation
        # traffic of the two-pass design and are reported beside it
        no = 45
        gbytes = 8 * asm.nnz + 8 * dm.n_dofs
        impl = 8 * mesh.n_elem * (10 * 9 + no * 9) + 8 * mesh.n_elem * 30 + 4 * mesh.n_elem * 100
        dom = {"kernel": "k_gather<double,3> + k_load_vec<3>", "bound": "hbm", "unit": "GB/s",
               "achieved": gbytes / (ga_ms * 1e-3) / 1e9, "peak": hbm, "peak_source": hbm_src,
               "bytes_per_launch": gbytes, "implementation_bytes_per_launch": impl}
    dom["frac"] = dom["achieved"] / dom["peak"]
    # DRAM bytes of one launch from ncu on the 24^3 case (profiles/elasticity_tet10_24_kernels.md),
    # scaled by the element count; traffic grows in proportion to the mesh.
    per24 = {"k_gather<double,3> + k_load_vec<3>": 644832256 + 213843712 + 23702016,
             "k_elem_affine<ELASTICITY,10,3,double>": 20240128 + 296399360}
    dom["traffic"] = per24[dom["kernel"]] * mesh.n_elem / 82944.0 if args.n == N_CUBE else None
    dom["traffic_source"] = "ncu dram__bytes_read+write on build_cube 24^3, scaled x%.1f" % (mesh.n_elem / 82944.0)
    dom["stages_ms"] = {"elements": el_ms, "insertion": ga_ms}
    dom["step_hbm"] = {"achieved_gbs": B / (ms * 1e-3) / 1e9, "peak_gbs": hbm, "frac": B / (ms * 1e-3) / 1e9 / hbm,
                       "algorithmic_bytes": B}

    gc.enable()
    cpu = None
    if rank == 0 and not args.no_cpu:
        rp, col = asm.sparsity()
        cores = os.cpu_count() or 1
        v, n, s = cpu_sample(mesh.xyz, mesh.conn, dm.elem_dofs, dm.n_dofs, dm.constrained, E, f, rp, col, cores,
                             budget_s=10.0)
        cpu = {"value": v, "unit": "Melem/s", "cores": cores, "kind": "port",
               "sample": "elements [0, %d) of the mesh, %.1f s, %d threads" % (n, s, cores)}
    asm.close()
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "Melem/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": ("double-float (FP32 pairs) contraction and sums, FP64 geometry" if prec == lm.FP64
                      else "f32 contraction, FP64 geometry, double-float sums"),
            "data": "synthetic (seeded mesh jitter, E_e, f)",
            "config": {"workload": "elasticity TET10 build_cube %d^3 x6 tets, QGauss FOURTH" % args.n,
                       "n_elem": mesh.n_elem, "n_dofs": dm.n_dofs, "nnz": asm.nnz,
                       "precision": args.precision, "l2": "inputs larger than L2 (2.6 GB element buffer)",
                       "parallelism": "replica per GPU", "setup": setup},
            "mdofs_per_s": value * dm.n_dofs / mesh.n_elem,
            "e2e": {"value": e2e, "unit": "Melem/s", "h2d_bytes_per_step": 8 * (mesh.n_elem + 3 * mesh.n_nodes),
                    "d2h_bytes_per_step": 8 * (asm.nnz + dm.n_dofs), "d2h_link_gbs": link_gbs,
                    "copy_floor_melem_s": mesh.n_elem / (8 * (asm.nnz + dm.n_dofs) / (link_gbs * 1e9)) / 1e6,
                    "step_ms": [round(x, 2) for x in e2e_ms],
                    "median_step_ms": float(np.median(e2e_ms))},
            "gpu_launches": launches, "clocks": clk, "roofline": dom, "cpu_baseline": cpu,
            "mixed": other, "residual": resid,
            "fp64_probe_tflops": {"dfma": fp64, "dmma_m8n8k4": fp64_tc,
                                  "note": "measured in this run; the drop-in contracts in double-float on the "
                                          "FP32 pipe instead"}}))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
