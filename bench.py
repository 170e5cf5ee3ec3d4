"""Benchmark of the GB300 CG assembly + Krylov path.

Workload (the plain-FP64-at-scale configuration): the P1 pressure-Poisson
system on the 128^3 six-tet unit cube (12,582,912 tets, 2,146,689 nodes,
31,802,497 CSR entries), interior vertices jittered +-0.2h (splitmix64 seed
20261204), source f = sin(pi x) sin(pi y) sin(pi z), Dirichlet 0 on the
boundary, degree-2 quadrature.

* step   = one assembly of that system (zero + coloured element loop + rhs),
           inputs resident in HBM; metric = elements assembled per second.
* e2e    = the same assembly through the host-pointer C-ABI call
           (fl_gpu_assemble_advdif_cg) with pinned host buffers: H2D of the
           source field, D2H of val and rhs inside the timed region.
* solve  = CG + Jacobi to rtol 1e-10 on the assembled system, plain FP64 and
           mixed precision (FP32 inner CG inside FP64 refinement).

``--impl reference`` times the CPU restatement of the reference algorithm
(OpenMP over colours, full quadrature loops, bisection addto) on all host
cores for the same metric.

Multi-GPU: replicas only -- each rank assembles its own copy of the workload;
``value`` is the elements of all ranks divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Melem/s assembly (P1 Poisson 128^3); Poisson time-to-1e-10"


def algorithmic_bytes(E, N, nnz):
    """Compulsory HBM bytes of one P1 assembly: connectivity, coordinates,
    source, CSR pattern read once, values and rhs written once."""
    return 16 * E + 24 * N + 8 * N + 4 * (N + 1) + 12 * nnz + 8 * N


def cg_iteration_bytes(N, nnz):
    """Compulsory bytes of one fused FP64 PCG iteration (matrix + vectors)."""
    return 12 * nnz + 4 * (N + 1) + 104 * N


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(key):
    """DRAM bytes per launch recorded from an ncu capture (profiles/ncu_traffic.txt)."""
    p = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        with open(p) as fh:
            for line in fh:
                f = line.split()
                if f and not f[0].startswith("#") and f[0] == key:
                    return float(f[1])
    except Exception:
        return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 5.0:  # first sample before timing
                time.sleep(0.01)
            self.lines.clear()
        except Exception:
            self.proc = None
        self.t_start = time.time()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def hold(self, step, min_s=1.0):
        """Keep running `step` (the timed region's own work) until the sampler
        has covered at least `min_s` seconds since the timed region began, so a
        timed region shorter than the sampling interval still gets samples
        taken under the same load."""
        import torch
        while time.time() - self.t_start < min_s:
            for _ in range(8):
                step()
            torch.cuda.synchronize()

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, dist, device):
    """The largest x over all ranks (the slowest rank's time); x itself
    without a process group."""
    if not dist:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        if args.impl != "reference":
            torch.cuda.set_device(local)
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
        return rank, ws, dist
    return 0, 1, None


def workload_name(n):
    """The headline workload's name, the same string in both arms."""
    return f"P1 Poisson assembly, {n}^3 six-tet cube, jitter 0.2h"


def row_scaled_err(a, b, findrm):
    """max over entries of |a - b| / max_j |b(i, j)| (row-scaled relative error)."""
    findrm = np.asarray(findrm, dtype=np.int64)
    lens = np.diff(findrm)
    ab = np.abs(b)
    rowmax = np.zeros(lens.size)
    nz = lens > 0
    rowmax[nz] = np.maximum.reduceat(ab, findrm[:-1][nz])
    rowmax[rowmax == 0] = 1.0
    return float(np.max(np.abs(a - b) / np.repeat(rowmax, lens))) if a.size else 0.0


def rel_err(a, b):
    """max |a - b| / max |b|."""
    sc = float(np.abs(b).max()) or 1.0
    return float(np.abs(a - b).max() / sc)


def sig(x, d=4):
    """x rounded to d significant digits (compact summary values)."""
    if x is None or isinstance(x, (bool, str)):
        return x
    if isinstance(x, (list, tuple)):
        return [sig(v, d) for v in x]
    if isinstance(x, dict):
        return {k: sig(v, d) for k, v in x.items()}
    if isinstance(x, int):
        return x
    x = float(x)
    return 0.0 if x == 0 else float(f"{x:.{d}g}")


def workload(n):
    from fluidity_gb300 import meshgen as M
    nd, X = M.cube_mesh(n)
    return nd, X, M.poisson_source(X), M.boundary_nodes(X)


def cpu_assembly_rate(nd, X, src, colours=None, findrm=None, colm=None, reps=1, nthreads=0):
    """Oracle assembly of the whole workload on all host cores; (Melem/s, threads, s)."""
    from oracle import oracle as O
    if findrm is None:
        findrm, colm, _ = O.make_sparsity(nd)
    if colours is None:
        ocol, ncol = O.colour_cg1(nd)
        colours = O.colour_sets(ocol, ncol)
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        _, _, st = O.assemble_advdif(ndglno_t=nd, nt=X.shape[0], ndglno_x=nd, coords=X,
                                     findrm=findrm, colm=colm, diffusivity=1.0, source=src,
                                     colours=colours, nthreads=nthreads)
        dt = time.perf_counter() - t0
        assert st == 0
        best = dt if best is None else min(best, dt)
    return nd.shape[0] / best / 1e6, nthreads or O.num_threads(), best


def cpu_advdif_steps(n=16, nsteps=10, nthreads=0):
    """The oracle's restatement of the 10-step advection-diffusion workload on
    the host cores (assembly, Dirichlet, GMRES(30) + Jacobi); ms per step."""
    from fluidity_gb300 import meshgen as M
    from oracle import oracle as O
    nd, X = M.cube_mesh(n)
    findrm, colm, _ = O.make_sparsity(nd)
    ocol, ncol = O.colour_cg1(nd)
    cs = O.colour_sets(ocol, ncol)
    u = M.advdif_velocity(X)
    bn = M.boundary_nodes(X)
    T = M.gaussian_tracer(X)
    t0 = time.perf_counter()
    its, Ts = [], []
    for _ in range(nsteps):
        val, rhs, st = O.assemble_advdif(ndglno_t=nd, nt=X.shape[0], ndglno_x=nd, coords=X,
                                         findrm=findrm, colm=colm, theta=0.5, dt=0.01,
                                         have_mass=True, velocity=u, T=T, diffusivity=1e-3,
                                         colours=cs, nthreads=nthreads)
        assert st == 0
        ina = np.zeros(X.shape[0], dtype=np.uint8)
        O.apply_dirichlet(bn, np.zeros(bn.size), T, 0.01, rhs, ina)
        dx, it, reason, _ = O.petsc_solve(findrm.astype(np.int64), colm, val, ina, rhs,
                                          ksp="gmres", restart=30, rtol=1e-10)
        its.append(int(it))
        T = T + 0.01 * dx
        Ts.append(T)
    return (time.perf_counter() - t0) / nsteps * 1e3, its, Ts


def run_reference(args, rank, ws, dist):
    if rank != 0:
        return
    from oracle import oracle as O
    nd, X, src, bn = workload(args.n)
    t0 = time.perf_counter()
    findrm, colm, _ = O.make_sparsity(nd)
    ocol, ncol = O.colour_cg1(nd)
    colours = O.colour_sets(ocol, ncol)
    setup = time.perf_counter() - t0
    times = []
    for k in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, _, st = O.assemble_advdif(ndglno_t=nd, nt=X.shape[0], ndglno_x=nd, coords=X,
                                     findrm=findrm, colm=colm, diffusivity=1.0, source=src,
                                     colours=colours)
        dt = time.perf_counter() - t0
        assert st == 0
        if k >= args.warmup:
            times.append(dt)
    t = float(np.mean(times))
    E = nd.shape[0]
    value = E / t / 1e6
    thr = O.num_threads()
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "Melem/s",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": workload_name(args.n), "elements": E,
                   "nodes": int(X.shape[0]), "nnz": int(colm.size), "cpu_setup_s": setup},
        "cpu_baseline": {"value": value, "unit": "Melem/s", "cores": thr, "kind": "port",
                         "sample": f"full {args.n}^3 assembly per step, OpenMP over "
                                   f"{ncol} colours"},
        "e2e": {"value": value, "unit": "Melem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def bench_batch(args, dev, stream):
    """Batched steps: 32 tracers on one 64^3 mesh (GMRES) beside 8 Poisson
    meshes of uneven size (CG), all as one set of CUDA graphs, against the
    same members run one after another through the unbatched entry points."""
    import torch

    from fluidity_gb300 import femtools as ft
    from fluidity_gb300 import meshgen as M

    nt = args.batch_fields
    kap, sc = M.batch_tracer_params(nt)
    nd, X = M.cube_mesh(64)
    shared = ft.Mesh(nd, X)
    T0 = torch.from_numpy(M.gaussian_tracer(X)).to(dev)
    u0 = M.advdif_velocity(X)
    bn = M.boundary_nodes(X)
    members = []
    for k in range(nt):
        p = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True,
                             diffusivity=float(kap[k]))
        members.append((shared, p, ft.solver_options(ksp="gmres", restart=30, rtol=1e-10,
                                                     max_its=10000),
                        bn, {"t": T0, "velocity": torch.from_numpy(sc[k] * u0).to(dev)}))
    pois = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
    meshes = []
    for i, n in enumerate(M.BATCH_MESH_SIDES):
        ndi, Xi = M.batch_mesh(i)
        mi = ft.Mesh(ndi, Xi)
        meshes.append(mi)
        members.append((mi, pois, ft.solver_options(ksp="cg", rtol=1e-10, max_its=20000),
                        M.boundary_nodes(Xi), {"source": torch.from_numpy(M.poisson_source(Xi)).to(dev)}))
    elements = sum(m.E for m, *_ in members)
    b = ft.Batch()
    regs = [b.add(m, p, o, bc_nodes=bnd, bc_values=np.zeros(bnd.size), **f)
            for m, p, o, bnd, f in members]

    def reset():
        for r in regs:
            r["x"].zero_()

    t0 = time.perf_counter()
    reset()
    b.run(stream=stream)  # autotune, graph build, first execution
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    reps_n = max(2, min(args.steps, 5))
    l0 = ft.kernel_launch_count()
    times = []
    for _ in range(reps_n):
        reset()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        reps = b.run(stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    launches = (ft.kernel_launch_count() - l0) // reps_n
    batch_ms = float(np.median(times))
    xb = [r["x"].clone() for r in regs]

    # the same members one by one through fl_dev_assemble / apply_dirichlet / petsc_solve
    seq_times = []
    for _ in range(2):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        srep = []
        xs = []
        for (m, p, o, bnd, f), r in zip(members, regs):
            val, rhs = ft.assemble_advection_diffusion_cg(m, p, val=r["val"], rhs=r["rhs"],
                                                          stream=stream, **{k: f.get(k) for k in
                                                                            ("t", "velocity", "source")})
            r["inactive"].zero_()
            nodes = torch.from_numpy(bnd).to(dev)
            ft.apply_dirichlet_conditions(m, rhs, r["inactive"], nodes,
                                          torch.zeros(bnd.size, dtype=torch.float64, device=dev),
                                          t=f.get("t"), dt=p.dt, stream=stream)
            x = torch.zeros(m.N, dtype=torch.float64, device=dev)
            srep.append(ft.petsc_solve(m, x, val, rhs, o, inactive=r["inactive"], stream=stream))
            xs.append(x)
        e1.record(stream)
        torch.cuda.synchronize()
        seq_times.append(e0.elapsed_time(e1))
    seq_ms = float(min(seq_times))
    identical = all(torch.equal(a, c) for a, c in zip(xb, xs))
    its = [r["iterations"] for r in reps]
    keep = {}
    for k, (mm, pp, oo, bnd, ff) in ((0, members[0]), (nt, members[nt])):
        r = regs[k]
        keep[k] = {"val": r["val"].cpu().numpy(), "rhs": r["rhs"].cpu().numpy(),
                   "inactive": r["inactive"].cpu().numpy(), "x": xb[k].cpu().numpy(),
                   "iterations": reps[k]["iterations"]}
    out = {
        "workload": f"{nt} tracers (GMRES(30), rtol 1e-10) on one 64^3 mesh + 8 Poisson meshes "
                    f"n={list(M.BATCH_MESH_SIDES)} (CG, rtol 1e-10), one step each",
        "members": len(members), "elements_assembled": int(elements),
        "batch_ms": batch_ms, "sequential_ms": seq_ms, "speedup_vs_sequential": seq_ms / batch_ms,
        "steps_per_s": len(members) / (batch_ms * 1e-3),
        "melem_per_s_incl_solve": elements / (batch_ms * 1e-3) / 1e6,
        "iterations_tracers": [min(its[:nt]), max(its[:nt])], "iterations_meshes": its[nt:],
        "max_true_rel_residual": max(r["true_rel_residual"] for r in reps),
        "all_converged": all(r["reason"] > 0 for r in reps),
        "identical_to_sequential": bool(identical),
        "kernel_launches_per_run": int(launches), "build_and_first_run_s": build_s,
        "tiles": {f"n={n}": list(t) for n, t in zip([64] + list(M.BATCH_MESH_SIDES),
                                                      [(shared.tiles())] + [mm.tiles() for mm in meshes])},
    }
    b.close()
    return out, keep


def p2_algorithmic_bytes(E, N1, N2, nnz):
    """Compulsory HBM bytes of one P2 assembly (P2 and P1 connectivity,
    coordinates, source, pattern read once, values and rhs written once)."""
    return 40 * E + 16 * E + 24 * N1 + 8 * N2 + 4 * (N2 + 1) + 12 * nnz + 8 * N2


def bench_p2(args, dev, stream, n=64):
    """P2 Poisson on the n^3 six-tet cube (degree-4 quadrature): assembly
    throughput against its algorithmic bytes, then CG + Jacobi to 1e-10."""
    import ctypes as C

    import torch

    from fluidity_gb300 import femtools as ft
    from fluidity_gb300 import meshgen as M

    nd, X = M.cube_mesh(n)
    nd2, n2 = ft.make_global_numbering_p2(nd)
    X2 = M.p2_coordinates(nd, nd2, X, M.P2_COUNTS)
    m = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    p = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=4)
    src = torch.from_numpy(M.poisson_source(X2)).to(dev)
    val = torch.empty(m.nnz, dtype=torch.float64, device=dev)
    rhs = torch.empty(m.N, dtype=torch.float64, device=dev)
    step = lambda: ft.assemble_advection_diffusion_cg(m, p, source=src, val=val, rhs=rhs, stream=stream)
    for _ in range(3):
        step()
    reps = max(3, min(20, args.steps))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(reps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    m.lib.fl_set_kernel_timing(m.handle, 1)
    kms = []
    for _ in range(reps):
        step()
        f = C.c_float()
        ft.check(m.lib.fl_last_assembly_kernel_ms(m.handle, C.byref(f)), "timing")
        kms.append(f.value)
    m.lib.fl_set_kernel_timing(m.handle, 0)
    kernel_ms = float(np.median(kms))
    alg = p2_algorithmic_bytes(m.E, X.shape[0], m.N, m.nnz)
    peak, _ = measured_peak_hbm()
    achieved = alg / (kernel_ms * 1e-3) / 1e9
    sp2 = m.sparsity()
    host = {"nd": nd, "X": X, "nd2": nd2, "n2": n2, "src": M.poisson_source(X2), "val": val.cpu().numpy(),
            "rhs": rhs.cpu().numpy(), "findrm": sp2.findrm, "colm": sp2.colm, "centrm": sp2.centrm}
    ina = torch.zeros(m.N, dtype=torch.uint8, device=dev)
    bn = M.boundary_nodes(X2)
    step()
    ft.apply_dirichlet_conditions(m, rhs, ina, torch.from_numpy(bn).to(dev),
                                  torch.zeros(bn.size, dtype=torch.float64, device=dev), dt=1.0,
                                  stream=stream)
    solve = {}
    for prec in ("fp64", "reliable"):
        x = torch.zeros(m.N, dtype=torch.float64, device=dev)
        opts = ft.solver_options(ksp="cg", rtol=1e-10, max_its=50000, precision=prec, norm="unpreconditioned")
        torch.cuda.synchronize()
        e0.record(stream)
        rep = ft.petsc_solve(m, x, val, rhs, opts, inactive=ina, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        solve[prec] = {"ms": e0.elapsed_time(e1), "iterations": rep["iterations"],
                       "reason": rep["reason_name"], "true_rel_residual": rep["true_rel_residual"]}
    it_bytes = cg_iteration_bytes(m.N, m.nnz)
    f64 = solve["fp64"]
    f64["achieved_gbs"] = it_bytes * f64["iterations"] / (f64["ms"] * 1e-3) / 1e9
    f64["frac_of_hbm"] = f64["achieved_gbs"] / peak
    xa = torch.from_numpy(M.poisson_source(X2) / (3 * np.pi ** 2)).to(dev)
    return {
        "workload": f"P2 Poisson, {n}^3 six-tet cube, degree-4 quadrature (11 points)",
        "elements": m.E, "nodes": m.N, "nnz": m.nnz, "ms_per_assembly": ms,
        "melem_per_s": m.E / (ms * 1e-3) / 1e6, "kernel_ms": kernel_ms,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "algorithmic_bytes": alg},
        "solve": solve, "max_err_vs_analytic": float((x - xa).abs().max()),
    }, host


def bench_taylor_hood(args, dev, stream, n=64):
    """The Taylor-Hood pair (P2 velocity, P1 pressure) on the n^3 six-tet
    cube: the divergence element terms (by parts) and surface loop, the P2
    lumped velocity mass and C M_l^-1 C^T on its product pattern, by CUDA
    events on the stream; and, as a size-independent check, the by-parts
    matrix with every face's terms against the direct form (integration by
    parts, exact at these rules), row-scaled."""
    import torch

    from fluidity_gb300 import femtools as ft
    from fluidity_gb300 import meshgen as M
    from fluidity_gb300 import projection as PR

    nd, X = M.cube_mesh(n)
    nd2, n2 = ft.make_global_numbering_p2(nd)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m = ft.Mesh(nd2, X, x_ndglno=nd, nodes=n2)
    pat = PR.TaylorHoodPattern(m)
    prod = PR.TaylorHoodProductPattern(pat)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    faces6, xf, fe = M.boundary_faces_p2(nd, nd2)
    dfaces = torch.from_numpy(xf.astype(np.int32)).to(dev)
    dv = torch.from_numpy(faces6.astype(np.int32)).to(dev)
    dfe = torch.from_numpy(fe.astype(np.int32)).to(dev)
    ct = torch.empty((3, pat.nnz), dtype=torch.float64, device=dev)
    ml = torch.empty(m.N, dtype=torch.float64, device=dev)
    cmc = torch.empty(prod.nnz, dtype=torch.float64, device=dev)
    reps = max(3, min(10, args.steps))

    def timed(fn):
        for _ in range(2):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    def elem():
        PR.assemble_divergence_matrix_p2p1(m, pat, integrate_by_parts=True, ct=ct, stream=stream)

    def faces():
        PR.assemble_divergence_faces_p2p1(m, pat, ct, faces=dfaces, vfaces=dv, face_ele=dfe, stream=stream)

    def lumped():
        PR.compute_lumped_mass(m, out=ml, stream=stream)

    elem_ms, faces_ms, lumped_ms = timed(elem), timed(faces), timed(lumped)
    w = torch.stack([1.0 / ml] * 3, dim=1).reshape(-1).contiguous()

    def cmcf():
        PR.mult_div_vector_div_T(prod, ct, w, ct, out=cmc, stream=stream)

    cmc_ms = timed(cmcf)
    # by parts + every face (type 0) against the direct form
    elem()
    faces()
    direct = PR.assemble_divergence_matrix_p2p1(m, pat, integrate_by_parts=False, stream=stream)
    torch.cuda.synchronize()
    f = pat.sparsity().findrm
    rows = torch.from_numpy(np.repeat(np.arange(pat.N), np.diff(f))).to(dev)
    err = 0.0
    for d in range(3):
        rowmax = torch.zeros(pat.N, dtype=torch.float64, device=dev).scatter_reduce(
            0, rows, direct[d].abs(), reduce="amax")
        diff = (ct[d] - direct[d]).abs() / rowmax[rows].clamp_min(1e-300)
        err = max(err, float(diff.max()))
    out = {"workload": f"Taylor-Hood pair on the {n}^3 six-tet cube (P2 velocity, P1 pressure)",
           "elements": m.E, "velocity_nodes": m.N, "pressure_nodes": pat.N, "faces": int(xf.shape[0]),
           "nnz_divergence": pat.nnz, "nnz_cmc": prod.nnz, "pattern_setup_s": setup_s,
           "divergence_elements_ms": elem_ms, "divergence_faces_ms": faces_ms, "lumped_mass_ms": lumped_ms,
           "cmc_product_ms": cmc_ms, "by_parts_identity_max_row_scaled_err": err}
    prod.close()
    pat.close()
    m.close()
    return out


def bench_projection(args, dev, stream, m, X, n):
    """P1-P1 pressure projection on the mesh of the headline workload: the
    divergence matrix C^T, the second-order pattern, C M_l^-1 C^T, the KMK
    stabilisation, the projection rhs, CG + Jacobi on CMC + KMK to 1e-10 and
    the velocity correction; kernel times by CUDA events on the stream, and
    the oracle's serial restatement timed on a 32^3 sample."""
    import torch

    from fluidity_gb300 import femtools as ft
    from fluidity_gb300 import meshgen as M
    from fluidity_gb300 import projection as PR

    E, N, nnz = m.E, m.N, m.nnz
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    so = PR.get_csr_sparsity_secondorder(m)
    torch.cuda.synchronize()
    so_setup = time.perf_counter() - t0
    nnz2 = so.nnz
    ct = torch.empty((3, nnz), dtype=torch.float64, device=dev)
    outs = {k: torch.empty(N, dtype=torch.float64, device=dev) for k in ("ct_rhs", "dml", "gml")}
    cmc = torch.empty(nnz2, dtype=torch.float64, device=dev)
    kmk = torch.empty(nnz2, dtype=torch.float64, device=dev)
    kt = torch.empty(nnz, dtype=torch.float64, device=dev)
    bn = M.boundary_nodes(X)

    def div():
        PR.assemble_divergence_matrix_cg(m, ct=ct, ct_rhs=outs["ct_rhs"], div_mass_lumped=outs["dml"],
                                         grad_mass_lumped=outs["gml"], stream=stream)

    div()
    inv = PR.inverse_lumped_mass(outs["gml"], bn)
    pml = outs["dml"]

    def prod():
        PR.assemble_masslumped_cmc(so, ct, inv, ct, out=cmc, stream=stream)

    def kmkf():
        PR.assemble_kmk_matrix(m, so, pml, theta_pg=1.0, kmk=kmk, kt=kt, stream=stream)

    reps = max(3, min(10, args.steps))

    def timed(fn):
        for _ in range(2):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    div_ms, prod_ms, kmk_ms = timed(div), timed(prod), timed(kmkf)
    peak, _ = measured_peak_hbm()
    div_bytes = 16 * E + 24 * N + 4 * (N + 1) + 4 * nnz + 24 * nnz + 16 * N
    prod_bytes = 12 * nnz2 + 4 * (N + 1) + 24 * nnz + 8 * nnz + 4 * (N + 1) + 24 * N
    # the projection: rhs = -C u*, CG on CMC + KMK (one reference node), correction
    bubble = 64.0 * np.prod(X * (1.0 - X), axis=1)
    u = torch.from_numpy(M.advdif_velocity(X) * bubble[:, None]).to(dev).contiguous()
    prod()
    kmkf()
    PR.add_kmk_matrix(so, cmc, kmk, stream=stream)
    rhs = PR.assemble_masslumped_poisson_rhs(m, ct, None, None, None, u, dt=1.0, theta_pg=1.0, stream=stream)
    ina = torch.zeros(N, dtype=torch.uint8, device=dev)
    ina[N // 2] = 1
    rhs[N // 2] = 0.0
    dp = torch.zeros(N, dtype=torch.float64, device=dev)
    opts = ft.solver_options(ksp="cg", rtol=1e-10, max_its=50000, norm="unpreconditioned")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    rep = ft.petsc_solve(so, dp, cmc, rhs, opts, inactive=ina, stream=stream)
    PR.correct_masslumped_velocity(m, ct, inv, dp, u, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    solve_ms = e0.elapsed_time(e1)
    it_bytes = cg_iteration_bytes(N, nnz2)
    # the same projection solve with the AMG preconditioner (FP32 V-cycle,
    # unpreconditioned-norm test: rtol bounds the true residual)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    amg = ft.AmgPreconditioner(so, cmc, ina, stream=stream, unpreconditioned_norm=True)
    amg.set_precision(True)
    torch.cuda.synchronize()
    amg_setup_ms = (time.perf_counter() - t0) * 1e3
    dpa = torch.zeros(N, dtype=torch.float64, device=dev)
    amg.solve(dpa, rhs, opts, stream=stream)
    dpa.zero_()
    torch.cuda.synchronize()
    e0.record(stream)
    rep_amg = amg.solve(dpa, rhs, opts, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    amg_ms = e0.elapsed_time(e1)
    amg_levels = amg.levels()
    amg.close()
    cpu = None
    if not args.no_cpu:
        from oracle import oracle as O
        nd32, X32 = M.cube_mesh(32)
        f32, c32, _ = O.make_sparsity(nd32)
        t0 = time.perf_counter()
        ct32, _, _, gml32 = O.assemble_divergence_p1(nd32, X32, f32, c32)
        t_div = time.perf_counter() - t0
        t0 = time.perf_counter()
        sf, sc = O.sparsity_secondorder(f32, c32)
        t_so = time.perf_counter() - t0
        w32 = np.repeat((1.0 / gml32)[:, None], 3, axis=1)
        t0 = time.perf_counter()
        O.mult_div_vector_div_T(f32, c32, ct32, w32, ct32, sf, sc)
        t_prod = time.perf_counter() - t0
        cpu = {"kind": "port", "cores": 1, "sample": "32^3 six-tet cube (196,608 elements), serial oracle",
               "divergence_melem_per_s": nd32.shape[0] / t_div / 1e6, "secondorder_pattern_s": t_so,
               "cmc_product_mentries_per_s": len(sc) / t_prod / 1e6}
    so.close()
    return {
        "workload": f"P1-P1 pressure projection, {n}^3 six-tet cube",
        "elements": E, "nodes": N, "nnz_first_order": nnz, "nnz_second_order": nnz2,
        "secondorder_pattern_setup_s": so_setup,
        "divergence": {"ms": div_ms, "melem_per_s": E / (div_ms * 1e-3) / 1e6,
                       "roofline": {"bound": "hbm", "achieved": div_bytes / (div_ms * 1e-3) / 1e9,
                                    "peak": peak, "unit": "GB/s",
                                    "frac": div_bytes / (div_ms * 1e-3) / 1e9 / peak,
                                    "algorithmic_bytes": div_bytes}},
        "cmc_product": {"ms": prod_ms, "mentries_per_s": nnz2 / (prod_ms * 1e-3) / 1e6,
                        "roofline": {"bound": "hbm", "achieved": prod_bytes / (prod_ms * 1e-3) / 1e9,
                                     "peak": peak, "unit": "GB/s",
                                     "frac": prod_bytes / (prod_ms * 1e-3) / 1e9 / peak,
                                     "algorithmic_bytes": prod_bytes}},
        "kmk_ms": kmk_ms,
        "projection_solve": {"ms": solve_ms, "iterations": rep["iterations"], "reason": rep["reason_name"],
                             "true_rel_residual": rep["true_rel_residual"],
                             "cg_iteration_gbs": it_bytes * rep["iterations"] / (solve_ms * 1e-3) / 1e9},
        "projection_solve_amg": {"ms": amg_ms, "setup_ms": amg_setup_ms, "iterations": rep_amg["iterations"],
                                 "reason": rep_amg["reason_name"], "true_rel_residual": rep_amg["true_rel_residual"],
                                 "levels": amg_levels, "cycle": "fp32",
                                 "norm": "unpreconditioned ||r|| / ||b||"},
        "cpu_baseline": cpu,
    }


def bench_advdif_steps(args, dev, stream, n=16, nsteps=10):
    """The CPU-runnable workload: 10 advection-diffusion steps (theta 0.5,
    dt 0.01, GMRES(30) + Jacobi to 1e-10) on the 16^3 mesh, through
    solve_field_equation_cg's device path, timed per step."""
    import torch

    from fluidity_gb300 import femtools as ft
    from fluidity_gb300 import meshgen as M

    nd, X = M.cube_mesh(n)
    m = ft.Mesh(nd, X)
    p = ft.advdif_params(theta=0.5, dt=0.01, have_mass=True, have_advection=True, diffusivity=1e-3)
    u = torch.from_numpy(M.advdif_velocity(X)).to(dev)
    bn = M.boundary_nodes(X)
    nodes = torch.from_numpy(bn).to(dev)
    g = torch.zeros(bn.size, dtype=torch.float64, device=dev)

    def run(schedule="auto"):
        # one fl_dev_solve_field_equation_cg call per step: assembly, strong
        # Dirichlet conditions in rate-of-change form, GMRES from zero change
        # and t + dt delta, one error check per step
        opts = ft.solver_options(ksp="gmres", restart=30, rtol=1e-10, max_its=10000, schedule=schedule)
        t = torch.from_numpy(M.gaussian_tracer(X)).to(dev)
        its, ts = [], []
        for _ in range(nsteps):
            t, rep = ft.solve_field_equation_cg_device(m, t, p, opts, bc_nodes=nodes, bc_values=g, velocity=u,
                                                       stream=stream)
            its.append(rep["iterations"])
            ts.append(t)
        return t, its, ts

    def timed(schedule):
        run(schedule)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res = run(schedule)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / nsteps, res

    # the default schedule solves this 4,913-row system in one cooperative
    # launch; the launch-per-phase schedule (graph-replayed cycles) beside it
    ms_graph, _ = timed("graph")
    ms, (t, its, ts) = timed("auto")
    out = {"workload": f"advection-diffusion, {n}^3 six-tet cube, {nsteps} steps, GMRES(30)+Jacobi rtol 1e-10",
           "ms_per_step": ms, "ms_per_step_graph_schedule": ms_graph, "iterations": its,
           "tracer_max_final": float(t.max())}
    return out, [v.cpu().numpy() for v in ts]


def bench_learned(args, dev, stream, n, epochs, nsteps=240, ntrain=200):
    """Learned warm start on the rotating-source Poisson sequence: generate the
    plain solves, train the network on steps 2..ntrain-1 on the GPU, then time
    the held-out steps' solves to rtol 1e-10 from the zero, previous-step and
    learned guesses (FP64 CG and reliable-update mixed CG), each timed from the
    guess construction (the network's prediction included) to the solution."""
    import torch

    from fluidity_gb300 import femtools as ft
    from fluidity_gb300 import meshgen as M
    from fluidity_gb300 import warmstart as WS

    nd, X = M.cube_mesh(n)
    m = ft.Mesh(nd, X)
    seq = WS.PoissonSequence(m, X, M.boundary_nodes(X), stream=stream)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ps, bs = WS.pressure_sequence(seq, nsteps)
    torch.cuda.synchronize()
    gen_s = time.perf_counter() - t0
    net = WS.PressureGuessNet(m)
    t0 = time.perf_counter()
    kval = seq.val if getattr(args, "energy_loss", True) else None
    losses = WS.train(net, ps, bs, seq.mask, seq.nact, range(2, ntrain), epochs=epochs, stream=stream,
                      kval=kval)
    torch.cuda.synchronize()
    train_s = time.perf_counter() - t0
    ntrain_steps = epochs * (ntrain - 2)
    # network forward time alone
    out = torch.empty_like(ps[0])
    for _ in range(3):
        net.predict(ps[ntrain - 1], ps[ntrain - 2], bs[ntrain], out=out, stream=stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(20):
        net.predict(ps[ntrain - 1], ps[ntrain - 2], bs[ntrain], out=out, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    predict_ms = e0.elapsed_time(e1) / 20

    variants = {
        "fp64_zero": ("fp64", "zero"), "fp64_previous": ("fp64", "previous"),
        "fp64_learned": ("fp64", "learned"), "fp64_projection": ("fp64", "projection"),
        "fp64_learned_projection": ("fp64", "learned_projection"),
        "mixed_previous": ("reliable", "previous"), "mixed_learned": ("reliable", "learned"),
        "mixed_zero": ("reliable", "zero"), "mixed_projection": ("reliable", "projection"),
        "mixed_learned_projection": ("reliable", "learned_projection"),
        "amg_zero": ("amg", "zero"), "amg_previous": ("amg", "previous"), "amg_learned": ("amg", "learned"),
        "amg_projection": ("amg", "projection"), "amg_learned_projection": ("amg", "learned_projection"),
    }
    nproj = 6  # earlier solutions in the projection basis (Fischer's method)
    # one AMG hierarchy serves the whole sequence (the matrix does not change)
    seq.system(ntrain)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    amg = ft.AmgPreconditioner(m, seq.val, seq.ina, stream=stream, unpreconditioned_norm=True)
    amg.set_precision(True)  # FP32 V-cycle inside the FP64 CG
    torch.cuda.synchronize()
    amg_setup_ms = (time.perf_counter() - t0) * 1e3
    res = {k: {"ms": [], "iterations": [], "err": [], "true_rel_residual": []} for k in variants}
    pred = torch.empty_like(ps[0])
    tight = ft.solver_options(ksp="cg", rtol=1e-13, max_its=50000, norm="unpreconditioned")
    x = torch.empty_like(ps[0])
    for t in range(ntrain, nsteps):
        val, rhs, ina = seq.system(t)
        ref = ps[t].clone()
        ft.petsc_solve(m, ref, val, rhs, tight, inactive=ina, stream=stream)
        scale = ref.abs().max()
        for k, (prec, guess) in variants.items():
            opts = ft.solver_options(ksp="cg", rtol=1e-10, max_its=50000,
                                     precision="fp64" if prec == "amg" else prec, norm="unpreconditioned")
            torch.cuda.synchronize()
            e0.record(stream)
            if guess == "zero":
                x.zero_()
            elif guess == "previous":
                x.copy_(ps[t - 1])
            elif guess == "learned":
                net.predict(ps[t - 1], ps[t - 2], bs[t], out=x, stream=stream)
            else:
                basis = [ps[t - j] for j in range(1, nproj + 1)]
                if guess == "learned_projection":
                    net.predict(ps[t - 1], ps[t - 2], bs[t], out=pred, stream=stream)
                    basis = basis + [pred]
                ft.projected_guess(m, val, rhs, basis, inactive=ina, out=x, stream=stream)
            if prec == "amg":
                rep = amg.solve(x, rhs, ft.solver_options(ksp="cg", rtol=1e-10, max_its=50000), stream=stream)
            else:
                rep = ft.petsc_solve(m, x, val, rhs, opts, inactive=ina, stream=stream)
            e1.record(stream)
            torch.cuda.synchronize()
            r = res[k]
            r["ms"].append(e0.elapsed_time(e1))
            r["iterations"].append(rep["iterations"])
            r["true_rel_residual"].append(rep["true_rel_residual"])
            r["err"].append(float((x - ref).abs().max() / scale))
            assert rep["reason"] > 0, (k, t, rep)
    summary = {}
    for k, r in res.items():
        summary[k] = {"mean_ms": float(np.mean(r["ms"])), "mean_iterations": float(np.mean(r["iterations"])),
                      "max_err_vs_fp64_tight": float(np.max(r["err"])),
                      "max_true_rel_residual": float(np.max(r["true_rel_residual"]))}
    amg.close()
    base = summary["fp64_zero"]["mean_ms"]
    return {
        "amg_setup_ms": amg_setup_ms,
        "workload": f"{nsteps}-step rotating-source Poisson sequence on the {n}^3 P1 mesh; "
                    f"train on steps 2..{ntrain - 1}, CG to rtol 1e-10 on the {nsteps - ntrain} held-out steps",
        "nodes": m.N, "epochs": epochs, "train_steps": ntrain_steps, "train_s": train_s,
        "train_ms_per_step": train_s / ntrain_steps * 1e3, "loss_first_epoch": float(losses[0]),
        "loss_last_epoch": float(losses[-1]), "generate_s": gen_s, "predict_ms": predict_ms,
        "variants": summary,
        "speedup_mixed_learned_vs_fp64_zero": base / summary["mixed_learned"]["mean_ms"],
        "speedup_mixed_learned_vs_fp64_previous": summary["fp64_previous"]["mean_ms"]
        / summary["mixed_learned"]["mean_ms"],
        "speedup_fp64_learned_vs_fp64_previous": summary["fp64_previous"]["mean_ms"]
        / summary["fp64_learned"]["mean_ms"],
        "projection": f"Fischer's projection onto the {nproj} previous solutions (learned_projection: the same "
                      f"and the network's prediction), A-norm optimal, timed with the guess",
    }


def bench_solves(args, dev, stream, m, val, rhs, ina, xa, peak, kappa_name):
    """CG + Jacobi to rtol 1e-10 on one assembled Poisson system: FP64, the
    two mixed-precision forms and AMG, every one with the unpreconditioned
    test (rtol bounds the true relative residual); plus FP64 with PETSc's
    default preconditioned-norm test, and an FP64 solve to rtol 1e-13 as the
    reference of every solution's error."""
    import torch

    from fluidity_gb300 import femtools as ft

    N = m.N
    out = {}
    xs = {}

    def timed(opts):
        x = torch.zeros(N, dtype=torch.float64, device=dev)
        ft.petsc_solve(m, x, val, rhs, opts, inactive=ina, stream=stream)  # warm-up
        x.zero_()
        torch.cuda.synchronize()
        s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record(stream)
        rep = ft.petsc_solve(m, x, val, rhs, opts, inactive=ina, stream=stream)
        s1.record(stream)
        torch.cuda.synchronize()
        return x, rep, s0.elapsed_time(s1)

    xt = torch.zeros(N, dtype=torch.float64, device=dev)
    ft.petsc_solve(m, xt, val, rhs, ft.solver_options(ksp="cg", rtol=1e-13, max_its=100000,
                                                       norm="unpreconditioned", start_from_zero=True),
                   inactive=ina, stream=stream)
    scale = float(xt.abs().max())
    variants = (("fp64", "fp64", "unpreconditioned"), ("fp64_pc_norm", "fp64", "preconditioned"),
                ("mixed", "mixed", "unpreconditioned"), ("reliable", "reliable", "unpreconditioned"))
    for key, prec, norm in variants:
        opts = ft.solver_options(ksp="cg", rtol=1e-10, max_its=100000, precision=prec, norm=norm,
                                 start_from_zero=True)
        x, rep, sms = timed(opts)
        xs[key] = x
        out[key] = {"ms": sms, "iterations": rep["iterations"], "reason": rep["reason_name"],
                    "outer": rep["outer_iterations"], "norm": norm,
                    "true_rel_residual": rep["true_rel_residual"],
                    "err_vs_fp64_tight": float((x - xt).abs().max()) / scale}
    if not getattr(args, "no_amg", False):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        amg = ft.AmgPreconditioner(m, val, ina, stream=stream, unpreconditioned_norm=True)
        torch.cuda.synchronize()
        amg_setup = time.perf_counter() - t0
        opts = ft.solver_options(ksp="cg", rtol=1e-10, max_its=20000, start_from_zero=True)
        for key, fp32 in (("amg", False), ("amg_fp32_cycle", True)):
            amg.set_precision(fp32)
            xg = torch.zeros(N, dtype=torch.float64, device=dev)
            amg.solve(xg, rhs, opts, stream=stream)
            xg.zero_()
            torch.cuda.synchronize()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            rep = amg.solve(xg, rhs, opts, stream=stream)
            s1.record(stream)
            torch.cuda.synchronize()
            out[key] = {"ms": s0.elapsed_time(s1), "setup_ms": amg_setup * 1e3, "iterations": rep["iterations"],
                        "reason": rep["reason_name"], "levels": amg.levels(), "norm": "unpreconditioned",
                        "cycle": "fp32" if fp32 else "fp64", "true_rel_residual": rep["true_rel_residual"],
                        "err_vs_fp64_tight": float((xg - xt).abs().max()) / scale}
        amg.close()
    it_bytes = cg_iteration_bytes(N, m.nnz)
    f64 = out["fp64"]
    f64["achieved_gbs"] = it_bytes * f64["iterations"] / (f64["ms"] * 1e-3) / 1e9
    f64["frac_of_hbm"] = f64["achieved_gbs"] / peak
    if xa is not None:
        f64["max_err_vs_analytic"] = float((xs["fp64"] - xa).abs().max())
    for k in list(out):
        if k != "fp64" and isinstance(out[k], dict):
            out[f"speedup_{k}_vs_fp64"] = f64["ms"] / out[k]["ms"]
    out["max_true_rel_residual_unpreconditioned"] = max(
        v["true_rel_residual"] for k, v in out.items() if isinstance(v, dict) and v.get("norm") == "unpreconditioned")
    out["diffusivity"] = kappa_name
    return out


def cpu_legs(args, m, nd, X, src, gpu):
    """The oracle on the host cores (rank 0, one GPU): the timed CPU baselines
    of this run, and the checker of this run's GPU outputs at the benchmark
    sizes (integer arrays bit for bit; assembled entries row-scaled)."""
    from fluidity_gb300 import meshgen as M
    from oracle import oracle as O

    ncores = len(os.sched_getaffinity(0))
    par = {}
    # 128^3 P1: the oracle's own pattern and colouring against the GPU's
    t0 = time.perf_counter()
    f, c, ce = O.make_sparsity(nd)
    ocol, ncol = O.colour_cg1(nd)
    cs = O.colour_sets(ocol, ncol)
    setup_s = time.perf_counter() - t0
    s = m.sparsity()
    col, ptr, el = m.colouring()
    par["p1_sparsity_bit_exact"] = bool(np.array_equal(s.findrm, f) and np.array_equal(s.colm, c)
                                        and np.array_equal(s.centrm, ce))
    par["p1_colouring_bit_exact"] = bool(m.ncolours == ncol and np.array_equal(col, ocol)
                                         and np.array_equal(ptr, cs[0]) and np.array_equal(el, cs[1]))

    def oracle_asm(nthreads, **kw):
        t0 = time.perf_counter()
        v, r, st = O.assemble_advdif(ndglno_t=nd, nt=X.shape[0], ndglno_x=nd, coords=X, findrm=f, colm=c,
                                     source=src, colours=cs, nthreads=nthreads, **kw)
        assert st == 0
        return v, r, time.perf_counter() - t0

    oval, orhs, secs = oracle_asm(ncores, diffusivity=1.0)
    _, _, secs1 = oracle_asm(1, diffusivity=1.0)
    E = nd.shape[0]
    par["p1_max_row_scaled_err"] = row_scaled_err(gpu["val"], oval, f)
    par["p1_rhs_rel_err"] = rel_err(gpu["rhs"], orhs)
    del oval, orhs
    if gpu.get("aniso_val") is not None:
        aval, arhs, _ = oracle_asm(ncores, diffusivity=np.diag([1.0, 1.0, 1e-3]))
        par["p1_aniso_max_row_scaled_err"] = row_scaled_err(gpu["aniso_val"], aval, f)
        par["p1_aniso_rhs_rel_err"] = rel_err(gpu["aniso_rhs"], arhs)
        del aval, arhs
    cpu = {"value": E / secs / 1e6, "unit": "Melem/s", "cores": ncores, "kind": "port",
           "sample": f"one full {args.n}^3 assembly ({secs:.2f} s), OpenMP over {ncol} colours, oracle "
                     f"restatement of the reference loop",
           "value_1_core": E / secs1 / 1e6, "sample_1_core": f"one full {args.n}^3 assembly ({secs1:.2f} s)",
           "oracle_sparsity_and_colouring_s": setup_s}
    # 64^3 P2
    p2 = gpu.get("p2")
    if p2 is not None:
        ond2, on2 = O.make_global_numbering_p2(p2["nd"])
        par["p2_numbering_bit_exact"] = bool(on2 == p2["n2"] and np.array_equal(ond2, p2["nd2"]))
        f2, c2, ce2 = O.make_sparsity(ond2, on2)
        par["p2_sparsity_bit_exact"] = bool(np.array_equal(f2, p2["findrm"]) and np.array_equal(c2, p2["colm"])
                                            and np.array_equal(ce2, p2["centrm"]))
        pc, pn = O.colour_cg1(p2["nd"])
        t0 = time.perf_counter()
        v2, r2, st = O.assemble_advdif(ndglno_t=ond2, nt=on2, ndglno_x=p2["nd"], coords=p2["X"], findrm=f2,
                                       colm=c2, diffusivity=1.0, source=p2["src"], colours=O.colour_sets(pc, pn),
                                       quad_degree=4, t_degree=2, nthreads=ncores)
        p2s = time.perf_counter() - t0
        assert st == 0
        par["p2_max_row_scaled_err"] = row_scaled_err(p2["val"], v2, f2)
        par["p2_rhs_rel_err"] = rel_err(p2["rhs"], r2)
        cpu["p2_64_melem_per_s"] = p2["nd"].shape[0] / p2s / 1e6
        del v2, r2
    # the 16^3 advection-diffusion workload, ten steps
    adv_ms, adv_its, adv_T = cpu_advdif_steps(nthreads=ncores)
    cpu["advdif_16_ten_steps_ms_per_step"] = adv_ms
    cpu["advdif_16_ten_steps_iterations"] = adv_its
    st16 = gpu.get("steps16")
    if st16 is not None:
        gT, gits = st16
        par["advdif16_max_step_rel_diff"] = max(rel_err(a, b) for a, b in zip(gT, adv_T))
        par["advdif16_max_iteration_diff"] = int(max(abs(a - b) for a, b in zip(gits, adv_its)))
    # batch members: the first tracer on the 64^3 mesh and the Poisson member on the n=24 mesh
    bk = gpu.get("batch")
    if bk is not None:
        kap, sc = M.batch_tracer_params(args.batch_fields)
        worst = {"val": 0.0, "rhs": 0.0, "x": 0.0, "its": 0, "inactive_equal": True}
        for k, (ndm, Xm) in bk["meshes"].items():
            fm, cm, _ = O.make_sparsity(ndm)
            cc, cn = O.colour_cg1(ndm)
            bn = M.boundary_nodes(Xm)
            if k == 0:
                T0 = M.gaussian_tracer(Xm)
                kw = dict(theta=0.5, dt=0.01, have_mass=True, velocity=sc[0] * M.advdif_velocity(Xm), T=T0,
                          diffusivity=float(kap[0]))
                ksp = "gmres"
            else:
                T0 = None
                kw = dict(diffusivity=1.0, source=M.poisson_source(Xm))
                ksp = "cg"
            ov, orr, st = O.assemble_advdif(ndglno_t=ndm, nt=Xm.shape[0], ndglno_x=ndm, coords=Xm, findrm=fm,
                                            colm=cm, colours=O.colour_sets(cc, cn), nthreads=ncores, **kw)
            assert st == 0
            oina = np.zeros(Xm.shape[0], dtype=np.uint8)
            O.apply_dirichlet(bn, np.zeros(bn.size), T0, kw.get("dt", 1.0), orr, oina)
            ox, oits, oreason, _ = O.petsc_solve(fm, cm, ov, oina, orr, ksp=ksp, restart=30, rtol=1e-10,
                                                 max_its=20000, nthreads=ncores)
            g = bk["members"][k]
            worst["val"] = max(worst["val"], row_scaled_err(g["val"], ov, fm))
            worst["rhs"] = max(worst["rhs"], rel_err(g["rhs"], orr))
            worst["x"] = max(worst["x"], rel_err(g["x"], ox))
            worst["its"] = max(worst["its"], abs(g["iterations"] - oits))
            worst["inactive_equal"] = worst["inactive_equal"] and bool(np.array_equal(g["inactive"], oina))
        par["batch_members"] = "tracer 0 on 64^3 (GMRES) and the n=24 Poisson mesh (CG)"
        par["batch_max_row_scaled_err"] = worst["val"]
        par["batch_rhs_rel_err"] = worst["rhs"]
        par["batch_solution_rel_err"] = worst["x"]
        par["batch_max_iteration_diff"] = int(worst["its"])
        par["batch_dirichlet_rows_equal"] = worst["inactive_equal"]
    par["tolerances"] = ("integer arrays equal; entries <= 1e-12 row-scaled; rhs <= 1e-12 of max; "
                         "solutions at rtol 1e-10 <= 1e-7 of max; iterations +-1")
    par["pass"] = bool(par["p1_sparsity_bit_exact"] and par["p1_colouring_bit_exact"]
                       and par["p1_max_row_scaled_err"] <= 1e-12 and par["p1_rhs_rel_err"] <= 1e-12
                       and par.get("p1_aniso_max_row_scaled_err", 0) <= 1e-12
                       and par.get("p2_numbering_bit_exact", True) and par.get("p2_sparsity_bit_exact", True)
                       and par.get("p2_max_row_scaled_err", 0) <= 1e-12
                       and par.get("advdif16_max_step_rel_diff", 0) <= 1e-9
                       and par.get("advdif16_max_iteration_diff", 0) <= 1
                       and par.get("batch_max_row_scaled_err", 0) <= 1e-12
                       and par.get("batch_solution_rel_err", 0) <= 1e-7
                       and par.get("batch_max_iteration_diff", 0) <= 1
                       and par.get("batch_dirichlet_rows_equal", True))
    return cpu, par


def run_ours(args, rank, ws, dist):
    import torch

    from fluidity_gb300 import femtools as ft
    from fluidity_gb300 import meshgen as M

    dev = torch.device("cuda", torch.cuda.current_device())
    nd, X, src, bn = workload(args.n)
    E, N = nd.shape[0], X.shape[0]
    t0 = time.perf_counter()
    m = ft.Mesh(nd, X)
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    nnz = m.nnz
    lib = m.lib
    stream = torch.cuda.current_stream()
    p = ft.advdif_params(diffusivity=1.0, have_source=True, quad_degree=2)
    dsrc = torch.from_numpy(src).to(dev)
    val = torch.empty(nnz, dtype=torch.float64, device=dev)
    rhs = torch.empty(N, dtype=torch.float64, device=dev)

    def step():
        ft.assemble_advection_diffusion_cg(m, p, source=dsrc, val=val, rhs=rhs, stream=stream)

    # tile choice by the project's autotuner (results do not depend on it),
    # or fixed tiles (a profiler changes the autotuner's timings)
    if args.tiles:
        tiles = tuple(int(v) for v in args.tiles.split(","))
        ft.set_assembly_tiles(m, *tiles)
    else:
        _, _, tiles = ft.autotune_assembly(m, p, source=dsrc, val=val, rhs=rhs, stream=stream)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    l0 = ft.kernel_launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        torch.cuda.synchronize()
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
        launches = ft.kernel_launch_count() - l0
        clk.hold(step, min_s=1.0)
    ms = max_over_ranks(ev0.elapsed_time(ev1) / args.steps, dist, dev)
    clocks = clk.summary()
    clocks["window"] = "the timed region, then untimed repeats of the same step to 1 s in all"

    # element-loop device time (all colours) per assembly, CUDA events on the stream
    import ctypes as C
    lib.fl_set_kernel_timing(m.handle, 1)
    kms = []
    for _ in range(max(3, min(50, args.steps // 2))):
        step()
        f = C.c_float()
        ft.check(lib.fl_last_assembly_kernel_ms(m.handle, C.byref(f)), "timing")
        kms.append(f.value)
    lib.fl_set_kernel_timing(m.handle, 0)
    kernel_ms = float(np.median(kms))
    alg = algorithmic_bytes(E, N, nnz)
    peak, peak_kind = measured_peak_hbm()
    achieved = alg / (kernel_ms * 1e-3) / 1e9

    # e2e through the host-pointer C-ABI with pinned buffers
    hsrc = torch.from_numpy(src).pin_memory()
    hval = torch.empty(nnz, dtype=torch.float64).pin_memory()
    hrhs = torch.empty(N, dtype=torch.float64).pin_memory()
    hsrc_np, hval_np, hrhs_np = hsrc.numpy(), hval.numpy(), hrhs.numpy()
    for _ in range(2):
        ft.assemble_advection_diffusion_cg(m, p, source=hsrc_np, val=hval_np, rhs=hrhs_np)
    t0 = time.perf_counter()
    e2e_steps = max(3, min(50, args.steps // 2))
    for _ in range(e2e_steps):
        ft.assemble_advection_diffusion_cg(m, p, source=hsrc_np, val=hval_np, rhs=hrhs_np)
    e2e_ms = max_over_ranks((time.perf_counter() - t0) / e2e_steps * 1e3, dist, dev)
    gpu = {"val": val.cpu().numpy(), "rhs": rhs.cpu().numpy()}
    assert np.array_equal(hval_np, gpu["val"]), "host and device paths differ"
    # device time of one host-pointer call (chunked uploads, passes and copies
    # overlap: the element passes' start to the last row pass's end)
    lib.fl_set_kernel_timing(m.handle, 1)
    ft.assemble_advection_diffusion_cg(m, p, source=hsrc_np, val=hval_np, rhs=hrhs_np)
    f = C.c_float()
    ft.check(lib.fl_last_assembly_kernel_ms(m.handle, C.byref(f)), "timing")
    e2e_compute_ms = f.value
    lib.fl_set_kernel_timing(m.handle, 0)
    # the host link alone: val and rhs copied device -> pinned host
    link = []
    for _ in range(3):
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record()
        hval.copy_(val, non_blocking=True)
        hrhs.copy_(rhs, non_blocking=True)
        c1.record()
        c1.synchronize()
        link.append(c0.elapsed_time(c1))
    link_ms = min(link)

    # solves: Dirichlet + CG to 1e-10 (fp64, mixed, AMG), isotropic and anisotropic
    solve = aniso = None
    if not args.no_solve:
        ina = torch.zeros(N, dtype=torch.uint8, device=dev)
        dbn = torch.from_numpy(bn).to(dev)
        dg = torch.zeros(bn.size, dtype=torch.float64, device=dev)
        step()
        ft.apply_dirichlet_conditions(m, rhs, ina, dbn, dg, dt=1.0, stream=stream)
        xa = torch.from_numpy(src / (3 * np.pi ** 2)).to(dev)
        solve = bench_solves(args, dev, stream, m, val, rhs, ina, xa, peak, "1 (isotropic)")
        # the anisotropic variant kappa = diag(1, 1, 1e-3)
        pa = ft.advdif_params(diffusivity=np.diag([1.0, 1.0, 1e-3]), have_source=True, quad_degree=2)
        aval = torch.empty(nnz, dtype=torch.float64, device=dev)
        arhs = torch.empty(N, dtype=torch.float64, device=dev)
        ft.assemble_advection_diffusion_cg(m, pa, source=dsrc, val=aval, rhs=arhs, stream=stream)
        torch.cuda.synchronize()
        gpu["aniso_val"], gpu["aniso_rhs"] = aval.cpu().numpy(), arhs.cpu().numpy()
        ina.zero_()
        ft.apply_dirichlet_conditions(m, arhs, ina, dbn, dg, dt=1.0, stream=stream)
        aniso = bench_solves(args, dev, stream, m, aval, arhs, ina, None, peak, "diag(1, 1, 1e-3)")
        del aval, arhs

    p2 = None
    if not args.no_p2:
        p2, gpu["p2"] = bench_p2(args, dev, stream)
    projection = None if args.no_projection else bench_projection(args, dev, stream, m, X, args.n)
    if projection is not None and not args.no_p2:
        projection["taylor_hood_64"] = bench_taylor_hood(args, dev, stream, 64)
    steps16, ts16 = bench_advdif_steps(args, dev, stream)
    gpu["steps16"] = (ts16, steps16["iterations"])
    batch = None
    if not args.no_batch:
        batch, keep = bench_batch(args, dev, stream)
        gpu["batch"] = {"members": keep, "meshes": {0: M.cube_mesh(64), args.batch_fields: M.batch_mesh(0)}}
    learned = None
    if not args.no_learned:
        sizes = [int(v) for v in args.learned_sizes.split(",") if v]
        learned = {f"n{k}": bench_learned(args, dev, stream, k,
                                          epochs=args.epochs if k <= 64 else max(4, args.epochs // 3))
                   for k in sizes}

    if rank != 0:
        return
    cpu = parity = None
    if not args.no_cpu and ws == 1:
        cpu, parity = cpu_legs(args, m, nd, X, src, gpu)
    value = E * ws / (ms * 1e-3) / 1e6
    e2e = {"value": E * ws / (e2e_ms * 1e-3) / 1e6, "unit": "Melem/s",
           "h2d_bytes_per_step": 8 * N, "d2h_bytes_per_step": 8 * nnz + 8 * N,
           "ms_per_step": e2e_ms, "assembly_ms_within": e2e_compute_ms, "d2h_copy_ms": link_ms}
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": ncu_traffic(f"assembly_p1_poisson_{args.n}"),
                "peak_kind": peak_kind,
                "kernel": "assembly: k_asm_p1_diffusion_df + k_rows_pull_df",
                "kernel_ms": kernel_ms, "algorithmic_bytes": alg}
    line = {
        "metric": METRIC, "value": value, "unit": "Melem/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64 (double-float element arithmetic)", "data": "synthetic",
        "config": {"workload": workload_name(args.n),
                   "elements": E, "nodes": N, "nnz": nnz, "colours": m.ncolours,
                   "parallelism": f"replicas{ws}", "l2": "inputs larger than L2 (no flush)",
                   "assembly_tiles": list(tiles),
                   "gpu_setup_s (sparsity+colouring)": setup_s},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "parity": parity,
        "solve": solve,
        "solve_anisotropic": aniso,
        "p2": p2,
        "projection": projection,
        "advdif_16_ten_steps": steps16,
        "batch": batch,
        "learned": learned,
    }
    line["summary"] = compact_summary(line)
    print(json.dumps(line), flush=True)


def compact_summary(line):
    """The headline numbers of every section in a few hundred bytes, last in the
    line so a truncated log still holds them."""
    def pick(d, *keys):
        return {k: sig(d[k]) for k in keys if d and k in d}

    out = {"assembly_p1_melem_s": sig(line["value"]), "e2e_melem_s": sig(line["e2e"]["value"]),
           "roofline_frac": sig(line["roofline"]["frac"]), "kernel_ms": sig(line["roofline"]["kernel_ms"])}
    par = line.get("parity")
    if par:
        out["parity"] = {k: sig(v, 2) for k, v in par.items() if k not in ("tolerances", "batch_members")}
    for key in ("solve", "solve_anisotropic"):
        sv = line.get(key)
        if sv:
            out[key] = {k: [sig(sv[k]["ms"]), sv[k]["iterations"], sig(sv[k]["true_rel_residual"], 3)]
                        for k in ("fp64", "fp64_pc_norm", "mixed", "reliable", "amg_fp32_cycle") if k in sv}
            out[key]["fields"] = "ms, iterations, true relative residual"
    p2 = line.get("p2")
    if p2:
        out["p2_64"] = {"melem_s": sig(p2["melem_per_s"]), "frac": sig(p2["roofline"]["frac"]),
                        "cg_fp64_ms": sig(p2["solve"]["fp64"]["ms"]), "cg_reliable_ms": sig(p2["solve"]["reliable"]["ms"])}
    st = line.get("advdif_16_ten_steps")
    if st:
        out["advdif16_ms_per_step"] = sig(st["ms_per_step"])
        if "ms_per_step_graph_schedule" in st:
            out["advdif16_ms_per_step_graph_schedule"] = sig(st["ms_per_step_graph_schedule"])
    b = line.get("batch")
    if b:
        out["batch"] = pick(b, "batch_ms", "sequential_ms", "speedup_vs_sequential")
    pr = line.get("projection")
    if pr:
        out["projection_128"] = {"div_ms": sig(pr["divergence"]["ms"]), "cmc_ms": sig(pr["cmc_product"]["ms"]),
                                 "kmk_ms": sig(pr["kmk_ms"]), "solve_ms": sig(pr["projection_solve"]["ms"]),
                                 "amg_solve_ms": sig(pr["projection_solve_amg"]["ms"])}
        th = pr.get("taylor_hood_64")
        if th:
            out["taylor_hood_64"] = {"div_ms": sig(th["divergence_elements_ms"]), "faces_ms": sig(th["divergence_faces_ms"]),
                                     "cmc_ms": sig(th["cmc_product_ms"]),
                                     "identity_err": sig(th["by_parts_identity_max_row_scaled_err"], 2)}
    ln = line.get("learned")
    if ln:
        for k, v in ln.items():
            vs = v["variants"]
            out[f"learned_{k}"] = {name: [sig(vs[name]["mean_ms"]), sig(vs[name]["mean_iterations"], 3)] for name in
                                  ("fp64_zero", "fp64_previous", "fp64_learned", "fp64_projection",
                                   "fp64_learned_projection", "mixed_previous", "mixed_learned",
                                   "mixed_projection", "mixed_learned_projection", "amg_previous",
                                   "amg_projection", "amg_learned_projection") if name in vs}
            out[f"learned_{k}"]["fields"] = "mean ms, mean iterations"
            out[f"learned_{k}"]["predict_ms"] = sig(v["predict_ms"])
            out[f"learned_{k}"]["max_true_rel_residual"] = sig(max(x["max_true_rel_residual"] for x in vs.values()), 3)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", "--hexes", dest="n", type=int, default=128, help="hexes per side")
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--no-p2", action="store_true")
    ap.add_argument("--no-learned", action="store_true")
    ap.add_argument("--no-projection", action="store_true")
    ap.add_argument("--tiles", default="",
                    help="fixed assembly tiles 'elem_block,elem_blocks_per_sm,row_tile' instead of the autotuner")
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--learned-sizes", default="64,128",
                    help="mesh sides of the learned-warm-start sequences")
    ap.add_argument("--batch-fields", type=int, default=32)
    args = ap.parse_args()
    rank, ws, dist = dist_setup(args)
    try:
        if args.impl == "reference":
            run_reference(args, rank, ws, dist)
        else:
            run_ours(args, rank, ws, dist)
    finally:
        if dist:
            dist.destroy_process_group()


if __name__ == "__main__":
    main()
