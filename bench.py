"""Benchmark of the FreeFEM assemble-and-solve path on one GB300.

Workload (default): 3D linear elasticity on the unit cube, cube(64,64,64) split into 6 tets per
hexahedron (1,572,864 tets), [P2,P2,P2] (6,440,067 DOFs), E=1, nu=0.3, clamped on the face x=0
(label 4), body force (0,0,-1), FP64, Jacobi-PCG to FreeFEM's eps=1e-10.  A step is one full
pass of the path from the mesh + DOF table to the solution:
    space setup (node->element incidence) + matrix A = a(Vh,Vh) (pattern, values, tgv)
    + b = a(0,Vh) (same pass) + u[] = A^-1*b (CG)
value: inputs (coordinates, elements, DOF table) resident in HBM before the timed region.
e2e:   the same through the public API from host (numpy) arrays, host<->device copies timed.
The matrix (~6 GB) is larger than L2 (129 MB), so no flush is needed between steps.

--impl reference times the oracle port of FreeFEM's CPU path (oracle/ffo.c) on the host cores,
one single-threaded instance per core (FreeFEM's core is single-threaded), on a bounded sample
of the same workload family.
"""
from __future__ import annotations

import argparse
import dataclasses
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "freefem-sources_gb300"))

METRIC = "assemble+solve DOFs/s: FP64 plain vs mixed/adjoint/batched, at 1e-8 rel err"
UNIT = "DOFs/s"
ITMAX = 20000   # iteration cap of the timed solves (CG needs a few thousand here)

CONFIGS = {
    "elasticity_p2_cube64": dict(mesh=("cube", 64), kind="P2vec", form="elasticity", on=(4,),
                                 eps=1e-10),
    "poisson_p1_square256": dict(mesh=("square", 256), kind="P1", form="diffusion",
                                 on=(1, 2, 3, 4), eps=1e-10),
    # 3D scalar diffusion, kappa P0 with ln kappa ~ N(0,1) i.i.d. per tet (seed 3)
    "diffusion_p1_cube160": dict(mesh=("cube", 160), kind="P1", form="diffusion",
                                 on=(1, 2, 3, 4, 5, 6), eps=1e-10, kappa_seed=3),
    # 1024 independent jittered squares, N ~ U{16..128}, FP32 inner / FP64 refinement to 1e-8
    "batched_p1_1024": dict(batch=True, nprob=1024, nmin=16, nmax=128, eps=1e-8, seed=0),
    # 2D inverse diffusion on square(512): dL/dkappa by the adjoint at kappa = 1, with
    # ln kappa_true a Gaussian field (squared-exponential, length 0.1, sigma 1), 1% noise;
    # heat variant: 200 implicit-Euler steps, dt 1e-3, checkpoints every 20 steps
    "inverse_diffusion_p1_square512": dict(adjoint=True, mesh=("square", 512), kind="P1",
                                           form="diffusion", on=(1, 2, 3, 4), eps=1e-12, seed=4,
                                           ell=0.1, sigma=1.0, noise=0.01, nfd=64,
                                           heat_steps=200, heat_dt=1e-3, heat_checkpoint=20),
}
SAMPLE = {"elasticity_p2_cube64": ("cube", 12), "poisson_p1_square256": ("square", 256),
          "diffusion_p1_cube160": ("cube", 40), "batched_p1_1024": ("square", 64),
          "inverse_diffusion_p1_square512": ("square", 256)}


def gaussian_field(n, ell, sigma, seed):
    """A stationary Gaussian field on the n x n cell centres of the unit square, covariance
    sigma^2 exp(-r^2 / (2 ell^2)), sampled by circulant embedding (Dietrich & Newsam 1997) on
    the 2n x 2n periodic grid of spacing 1/n.  Returns field[i + j*n] for cell (i, j)."""
    import numpy as np
    m = 2 * n
    d = np.minimum(np.arange(m), m - np.arange(m)) / n
    cov = sigma ** 2 * np.exp(-(d[:, None] ** 2 + d[None, :] ** 2) / (2 * ell ** 2))
    lam = np.maximum(np.fft.fft2(cov).real, 0.0)
    rng = np.random.Generator(np.random.PCG64(seed))
    xi = rng.standard_normal((m, m)) + 1j * rng.standard_normal((m, m))
    z = np.fft.fft2(np.sqrt(lam / (m * m)) * xi).real[:n, :n]   # z[j, i]: row j = y index
    return np.ascontiguousarray(z).ravel()


def build_problem(cfg, size=None):
    import numpy as np
    import ffgpu
    from ffgpu.fespace import FESpace
    kind_mesh, n = cfg["mesh"] if size is None else size
    Th = ffgpu.cube(n) if kind_mesh == "cube" else ffgpu.square(n)
    Vh = FESpace(Th, cfg["kind"])
    if cfg["form"] == "elasticity":
        a = ffgpu.varf_elasticity(E=1.0, nu=0.3, f=(0.0, 0.0, -1.0), on=cfg["on"])
    else:
        kappa = None
        if "kappa_seed" in cfg:
            kappa = np.exp(np.random.Generator(np.random.PCG64(cfg["kappa_seed"])).standard_normal(Th.nt))
        a = ffgpu.varf_diffusion(kappa=kappa, f=1.0, on=cfg["on"])
    return Th, Vh, a, np


# ------------------------------------------------------------------ CPU: the oracle port
def _oracle_adjoint_run(cfg, size):
    """CPU gradient of the inverse problem: forward CG, transpose CG, P0 sensitivities."""
    import numpy as np
    import ffgpu
    import ffo
    from ffgpu.fespace import FESpace
    Th = ffgpu.square(size[1])
    Vh = FESpace(Th, "P1")
    u_obs = np.zeros(Vh.ndof)
    M = ffo.assemble(Th, Vh, mass=1.0, c_stiff=0.0)     # the loss's mass matrix, set up once
    t0 = time.perf_counter()
    A = ffo.assemble(Th, Vh, kappa=np.ones(Th.nt))
    b = ffo.rhs(Th, Vh, f=1.0)
    on = Vh.on(cfg["on"])
    ffo.setbc(A, b, on)
    u, it, _, _ = ffo.cg(A, b, eps=cfg["eps"])
    r = u - u_obs
    Mr = M.matmul(r)
    lam, it2, _, _ = ffo.cg(A, Mr, eps=cfg["eps"], trans=True)
    # dL/dkappa_e = -lam_e' K_e u_e (K_e = |K| G G'), the varf FreeFEM scripts use for it
    X = Th.coords[Th.elems]
    e1, e2 = X[:, 1] - X[:, 0], X[:, 2] - X[:, 0]
    area = 0.5 * (e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0])
    gu = np.zeros((Th.nt, 2))
    gl = np.zeros((Th.nt, 2))
    for i in range(3):
        p1, p2 = X[:, (i + 1) % 3], X[:, (i + 2) % 3]
        G = np.stack([-(p2[:, 1] - p1[:, 1]), p2[:, 0] - p1[:, 0]], axis=1) / (2 * area[:, None])
        gu += G * u[Th.elems[:, i], None]
        gl += G * lam[Th.elems[:, i], None]
    gk = -area * (gu * gl).sum(axis=1)
    dt = time.perf_counter() - t0
    del gk
    return Vh.ndof, dt, it + it2


def _oracle_run(args):
    cfgname, size = args
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ffo
    cfg = CONFIGS[cfgname]
    if cfg.get("adjoint"):
        return _oracle_adjoint_run(cfg, size)
    Th, Vh, a, np = build_problem(cfg, size)
    t0 = time.perf_counter()
    quad = None if cfg["kind"] != "P1" or Th.dim == 3 else "qf2pT"
    A = ffo.assemble(Th, Vh, form=cfg["form"], quad=quad, kappa=a.kappa)
    b = ffo.rhs(Th, Vh, f=(0.0, 0.0, -1.0) if cfg["form"] == "elasticity" else 1.0, quad=quad)
    ffo.setbc(A, b, Vh.on(cfg["on"]))
    u, it, r, _ = ffo.cg(A, b, eps=cfg["eps"])
    dt = time.perf_counter() - t0
    return Vh.ndof, dt, it


def cpu_baseline(cfgname, procs=1, reps=1):
    """DOFs/s of the oracle on the sample problem, `procs` concurrent single-core instances."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ffo
    ffo.build()
    size = SAMPLE[cfgname]
    jobs = [(cfgname, size)] * (procs * reps)
    t0 = time.perf_counter()
    if procs == 1:
        res = [_oracle_run(j) for j in jobs]
    else:
        with mp.get_context("spawn").Pool(procs) as pool:
            res = pool.map(_oracle_run, jobs)
    wall = time.perf_counter() - t0
    ndof = res[0][0]
    per = statistics.median(r[1] for r in res)
    value = ndof * len(res) / wall if procs > 1 else ndof / per
    what = ("forward CG + transpose CG + P0 sensitivities" if CONFIGS[cfgname].get("adjoint")
            else "full assemble+rhs+CG")
    return dict(value=value, unit=UNIT, cores=procs, kind="port",
                sample=f"{size[0]}({size[1]}) same varf, {what} (eps={CONFIGS[cfgname]['eps']}), "
                       f"{len(res)} run(s), {res[0][2]} CG iterations, single-threaded oracle "
                       f"(oracle/ffo.c) per core"), wall


# ------------------------------------------------------------------ clocks
class ClockSampler:
    def __init__(self):
        self.p = None
        self.path = os.path.join(tempfile.gettempdir(), "ffgpu_clocks_%d.csv" % os.getpid())

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
            return
        # nvidia-smi's start-up (NVML initialisation) stalls CUDA calls of this process for tens of
        # milliseconds: the timed region starts once the sampler has written its first line
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 5.0 and self.p.poll() is None:
            try:
                if os.path.getsize(self.path) > 0:
                    break
            except OSError:
                pass
            time.sleep(0.01)

    def stop(self):
        if not self.p:
            return None
        self.p.terminate()
        try:
            self.p.wait(5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            t = [x.strip() for x in line.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1])); mx.append(float(t[2]))
            except ValueError:
                continue
            for nm, v in zip(names, t[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ GPU arm
# ------------------------------------------------------------------ replicas across ranks
# One process per GPU (torchrun); no data-path collective: every rank assembles and solves its
# own problem(s), the timings are bracketed by barriers and reduced by MAX, and the value counts
# the DOFs of all ranks.
def dist_max(values, world, device):
    """Element-wise max over ranks of a list of timings (identity on one rank)."""
    if world <= 1:
        return list(values)
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return t.tolist()


def dist_sum(values, world, device):
    """Element-wise sum over ranks (the units all ranks processed)."""
    if world <= 1:
        return list(values)
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.SUM)
    return t.tolist()


def rank_device(rank, world):
    return 0 if world == 1 else int(os.environ.get("LOCAL_RANK", rank))


def run_gpu(args, rank, world):
    import numpy as np
    import torch
    import ffgpu
    from ffgpu.build import build
    build()
    cfgname = args.config
    cfg = CONFIGS[cfgname]
    dev = rank_device(rank, world)
    torch.cuda.set_device(dev)
    Th, Vh, a, _ = build_problem(cfg)
    ctx = ffgpu.context(dev)
    stream = torch.cuda.ExternalStream(ffgpu.stream_handle(dev), device=dev)
    X = torch.from_numpy(Th.coords).cuda(dev)
    E = torch.from_numpy(np.ascontiguousarray(Th.elems)).cuda(dev)
    D = torch.from_numpy(np.ascontiguousarray(Vh.dof)).cuda(dev)
    BE = torch.from_numpy(np.ascontiguousarray(Th.belems)).cuda(dev)
    BL = torch.from_numpy(np.ascontiguousarray(Th.blabel)).cuda(dev)
    onbc = Vh.on(cfg["on"])
    a.on = cfg["on"]
    # the device-resident step reads the P0 coefficient from HBM like the mesh; e2e passes it
    # from host memory
    a_host = a
    if a.kappa is not None:
        a = dataclasses.replace(a, kappa=torch.from_numpy(np.ascontiguousarray(a.kappa)).to(dev))
    b = torch.empty(Vh.ndof, dtype=torch.float64, device=dev)
    phase = {"space": [], "assemble": [], "solve": []}

    def step_device():
        t = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        t[0].record(stream)
        S = ffgpu.DeviceSpace(Vh, device=dev, coords=X, elems=E, dof=D if Vh.kind != "P1" else None,
                              belems=BE, blabel=BL)
        t[1].record(stream)
        A = ffgpu.matrix(a, S, eps=cfg["eps"], itmax=ITMAX, rhs_out=b, device=dev)
        t[2].record(stream)
        u = A.solve(b)
        t[3].record(stream)
        t[3].synchronize()
        phase["space"].append(t[0].elapsed_time(t[1]))
        phase["assemble"].append(t[1].elapsed_time(t[2]))
        phase["solve"].append(t[2].elapsed_time(t[3]))
        return S, A, u

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()

    # warm-up
    for _ in range(args.warmup):
        S, A, u = step_device()
        it_warm = A.stats.iterations
        del A, S
    barrier()
    clocks = ClockSampler()
    clocks.start()
    l0 = ffgpu.kernel_launches(dev)
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    times, iters, asm_ms = [], [], []
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    barrier()
    ev0.record(stream)
    evs[0].record(stream)
    for k in range(args.steps):
        S, A, u = step_device()
        evs[k + 1].record(stream)
        evs[k + 1].synchronize()
        times.append(evs[k].elapsed_time(evs[k + 1]))
        iters.append(A.stats.iterations)
        keep = (S, A, u)
    ev1.record(stream)
    barrier()
    total_ms = ev0.elapsed_time(ev1)
    launches = ffgpu.kernel_launches(dev) - l0
    clk = clocks.stop()
    S, A, u = keep
    # accuracy: relative residual of the solution on non-tgv rows
    ub = u
    r = A.mult(ub)
    rh = (b - r).cpu().numpy()
    mask = onbc.astype(bool)
    rel_res = float(np.linalg.norm(rh[~mask]) / np.linalg.norm(b.cpu().numpy()[~mask]))
    # dominant kernel: the SpMV of the CG (K_a, with its fused dot), in the layout the tuner
    # chose, launched back to back on the library stream and timed there with CUDA events
    # (each launch streams the whole matrix, larger than L2)
    spmv_avg = A.time_spmv(0, 20)
    n, nnz, bs = A.n, A.nnz, A.block_size
    nnzb = nnz // (bs * bs)
    nb = n // bs
    layout = A.spmv_layout(0)
    # algorithmic bytes of one SpMV (CSR with FP64 values and int32 columns, x read once, y
    # written): 12 nnz + 4 (n+1) + 8 n + 8 n; the bytes the chosen layout actually streams
    # (one column index per 3x3 block, 16-bit column differences, SELL padding) beside it
    spmv_bytes = 12 * nnz + 4 * (n + 1) + 8 * n + 8 * n
    if (layout or "").startswith("sell32"):
        lib = ffgpu.lib()
        col_bytes = 2 if lib.ffgpu_matrix_spmv_layout(A.h, 3) else 4
        ent = lib.ffgpu_matrix_spmv_layout(A.h, 4)
        ent = ent if ent > 0 else nnzb
        # per stored block entry: values + column; per row: permutation; x read, y written
        stored = ent * (8 * bs * bs + col_bytes) + 4 * nb + 8 * n + 8 * n
    else:
        stored = 8 * nnz + 4 * nnzb + 4 * (nb + 1) + 8 * n + 8 * n
    achieved = spmv_bytes / (spmv_avg * 1e-3) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    traffic = None
    try:
        tr = json.load(open(os.path.join(REPO, "profiles", "traffic.json")))
        traffic = tr.get(cfgname, {}).get("spmv_bytes_per_launch")
    except Exception:
        pass
    # variants on the same workload: the double-float SpMV CG and the mixed-precision IR,
    # each with its error against this run's FP64 solution
    u_ref = u.clone()
    variants = {}

    def timed_variant(fn, reps):
        out, ms = None, []
        for r in range(reps + 1):
            e0v = torch.cuda.Event(enable_timing=True)
            e1v = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(dev)
            e0v.record(stream)
            out = fn()
            e1v.record(stream)
            e1v.synchronize()
            if r > 0:
                ms.append(e0v.elapsed_time(e1v))
        return out, statistics.median(ms)

    if not args.no_variants:
        def run_df():
            S2 = ffgpu.DeviceSpace(Vh, device=dev, coords=X, elems=E, dof=D, belems=BE, blabel=BL)
            A2 = ffgpu.matrix(a, S2, eps=cfg["eps"], itmax=ITMAX, rhs_out=b, device=dev)
            return A2.solve(b, spmv_mode=1), A2.stats.iterations, A2.spmv_layout(1), A2
        (udf, itdf, lay, Adf), msdf = timed_variant(run_df, 2)
        variants["fp64_values_doublefloat_spmv"] = {
            "value": Vh.ndof / (msdf * 1e-3), "ms_per_step": msdf, "cg_iterations": itdf,
            "spmv_layout": lay, "spmv_ms": Adf.time_spmv(1, 10),
            "rel_err_vs_fp64": float(torch.linalg.norm(udf - u_ref) / torch.linalg.norm(u_ref))}
        del Adf

        def run_ir():
            S2 = ffgpu.DeviceSpace(Vh, device=dev, coords=X, elems=E, dof=D, belems=BE, blabel=BL)
            A2 = ffgpu.matrix(a, S2, eps=cfg["eps"], itmax=ITMAX, rhs_out=b, device=dev)
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            ur = A2.solve_mixed(b, eps=cfg["eps"])
            t1.record(stream)
            t1.synchronize()
            return (ur, A2.stats.iterations, A2.stats.outer_iterations, A2.spmv_layout(2), t0.elapsed_time(t1),
                    A2)
        (uir, itir, outir, lay32, solve_ir_ms, Air), msir = timed_variant(run_ir, 1)
        variants["mixed_fp32_inner_fp64_refinement"] = {
            "value": Vh.ndof / (msir * 1e-3), "ms_per_step": msir, "inner_iterations": itir,
            "outer_iterations": outir, "spmv_layout": lay32, "spmv_ms": Air.time_spmv(2, 10),
            "solve_ms": solve_ir_ms,
            "solve_speedup_vs_fp64": statistics.median(phase["solve"][-args.steps:]) / solve_ir_ms,
            "rel_err_vs_fp64": float(torch.linalg.norm(uir - u_ref) / torch.linalg.norm(u_ref))}
        del Air
    # e2e: public API from host arrays (H2D of mesh/DOF table/BC mask, D2H of b and u)
    e2e_times = []
    bh = np.zeros(Vh.ndof)
    bh.fill(0.0)   # pages mapped before the timed region, as a caller's reused buffer is
    for s in range(max(1, args.warmup // 3) + args.steps):
        barrier()
        t0 = time.perf_counter()
        Ah = ffgpu.matrix(a_host, Vh, eps=cfg["eps"], itmax=ITMAX, rhs_out=bh, device=dev)
        uh = Ah.solve(bh)
        t1 = time.perf_counter()
        if s >= max(1, args.warmup // 3):
            e2e_times.append((t1 - t0) * 1e3)
        del Ah
    # P1 crosses no DOF table (its DOFs are the vertices); the P0 coefficient does cross
    h2d = (Th.coords.nbytes + Th.elems.nbytes + (0 if Vh.kind == "P1" else Vh.dof.nbytes) + Th.belems.nbytes
           + Th.blabel.nbytes + bh.nbytes + (a_host.kappa.nbytes if a_host.kappa is not None else 0))
    d2h = bh.nbytes + uh.nbytes
    # max over ranks
    t_step = total_ms / args.steps
    t_e2e = sum(e2e_times) / len(e2e_times)
    t_step, t_e2e = dist_max([t_step, t_e2e], world, torch.device("cuda", dev))
    value = world * Vh.ndof / (t_step * 1e-3)
    e2e_value = world * Vh.ndof / (t_e2e * 1e-3)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": cfgname, "mesh": f"{cfg['mesh'][0]}({cfg['mesh'][1]})",
                   "fe": cfg["kind"], "ndof": Vh.ndof, "nnz": nnz, "nt": Th.nt,
                   "solver": "Jacobi-PCG", "eps": cfg["eps"], "cg_iterations": iters[-1],
                   "l2": "inputs larger than L2 (matrix %.1f GB)" % (nnz * 8 / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "space_ms": statistics.median(phase["space"][-args.steps:]),
                   "assemble_ms": statistics.median(phase["assemble"][-args.steps:]),
                   "solve_ms": statistics.median(phase["solve"][-args.steps:]),
                   "ms_per_cg_iteration": statistics.median(phase["solve"][-args.steps:]) / max(1, iters[-1]),
                   "spmv_layout": layout,
                   "rel_residual": rel_res},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": t_e2e},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": f"FP64 SpMV of the CG (K_a), layout {layout}, block size {bs}",
                     "bytes_per_launch": spmv_bytes, "ms_per_launch": spmv_avg,
                     "stored_bytes_per_launch": stored,
                     "frac_of_stored_bytes": stored / (spmv_avg * 1e-3) / 1e9 / peak,
                     "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"},
        "assembly_roofline": assembly_roofline(Th, Vh, cfg, statistics.median(phase["assemble"][-args.steps:]), peak),
        "clocks": clk,
        "variants": variants,
    }
    return out


def assembly_roofline(Th, Vh, cfg, ms, peak):
    """The assembly (pattern + values + RHS + on()) against the algorithmic bytes of an
    element-scatter assembly, per element with k local DOFs: connectivity 4k, coordinates
    8 d (d+1), coefficient 8, element -> nonzero map 4 k^2, values 8 k^2, plus the RHS 8 n."""
    d = Th.dim
    k = Vh.ndofK
    bytes_ = Th.nt * (4 * k + 8 * d * (d + 1) + 8 + 12 * k * k) + 8 * Vh.ndof
    gbs = bytes_ / (ms * 1e-3) / 1e9
    return {"bound": "fp64 / latency (per-row gather, no scatter)", "achieved": gbs, "peak": peak, "unit": "GB/s",
            "frac": gbs / peak, "bytes": int(bytes_), "ms": ms,
            "note": "the device writes each nonzero once (row gather), not once per element contribution: "
                    "the scatter formula's bytes are not what it moves"}


def profile_case(kind, n, iters, spmv_mode):
    """Small case for ncu: space + assembly + a fixed number of CG iterations, twice."""
    import numpy as np
    import torch
    import ffgpu
    from ffgpu.build import build
    from ffgpu.fespace import FESpace
    build()
    if kind == "elasticity":
        Th = ffgpu.cube(n); Vh = FESpace(Th, "P2vec"); a = ffgpu.varf_elasticity(f=(0, 0, -1.0), on=(4,))
    elif kind == "diffusion3d":
        Th = ffgpu.cube(n); Vh = FESpace(Th, "P1")
        kap = np.exp(np.random.Generator(np.random.PCG64(1)).standard_normal(Th.nt))
        a = ffgpu.varf_diffusion(kappa=kap, f=1.0, on=(1, 2, 3, 4, 5, 6))
    else:
        Th = ffgpu.square(n); Vh = FESpace(Th, "P1"); a = ffgpu.varf_diffusion(f=1.0, on=(1, 2, 3, 4))
    dev = torch.device("cuda", 0)
    X = torch.from_numpy(Th.coords).to(dev); E = torch.from_numpy(np.ascontiguousarray(Th.elems)).to(dev)
    D = torch.from_numpy(Vh.dof).to(dev)
    BE = torch.from_numpy(np.ascontiguousarray(Th.belems)).to(dev)
    BL = torch.from_numpy(np.ascontiguousarray(Th.blabel)).to(dev)
    b = torch.empty(Vh.ndof, dtype=torch.float64, device=dev)
    for rep in range(2):
        S = ffgpu.DeviceSpace(Vh, coords=X, elems=E, dof=D, belems=BE, blabel=BL)
        A = ffgpu.matrix(a, S, eps=1e-10, itmax=iters, rhs_out=b)
        try:
            if spmv_mode == 2:      # mixed precision: one refinement step of `iters` FP32 iterations
                A.solve_mixed(b, eps=1e-10, eps_inner=1e-30, itmax_inner=iters, max_outer=1)
            else:
                A.solve(b, spmv_mode=spmv_mode)
        except ffgpu.FFGPUError as e:
            if e.code != -3:
                raise
        torch.cuda.synchronize()
        print(f"profile case {kind}({n}): ndof {Vh.ndof} nnz {A.nnz} iterations {A.stats.iterations} "
              f"device {A.stats.elapsed_ms:.2f} ms")
        del A, S


def run_adjoint(args, rank=0, world=1):
    """dL/dkappa by the adjoint (forward CG, transpose CG, sensitivity kernel) on the device;
    the heat variant with checkpoint-and-recompute; FD check on seeded elements.  A step is one
    gradient evaluation (L, dL/dkappa, dL/df at kappa = 1, its forward solve included); on N
    ranks every rank evaluates its own replica (weak scaling, no collective on the data path)."""
    import numpy as np
    import torch
    import ffgpu
    from ffgpu import adjoint
    from ffgpu.build import build
    from ffgpu.fespace import FESpace
    build()
    cfg = CONFIGS[args.config]
    n = cfg["mesh"][1]
    Th = ffgpu.square(n)
    Vh = FESpace(Th, "P1")
    di = rank_device(rank, world)
    dev = torch.device("cuda", di)
    torch.cuda.set_device(dev)
    ffgpu.context(di)
    stream = torch.cuda.ExternalStream(ffgpu.stream_handle(di), device=dev)
    cells = gaussian_field(n, cfg["ell"], cfg["sigma"], cfg["seed"])
    k_true = torch.from_numpy(np.exp(np.repeat(cells, 2))).to(dev)      # both triangles of a cell
    ones = torch.ones(Th.nt, dtype=torch.float64, device=dev)
    P = adjoint.DiffusionProblem(Vh, on=cfg["on"], eps=cfg["eps"], device=di)
    u_true = P.solve(k_true, 1.0)
    rng = np.random.Generator(np.random.PCG64(cfg["seed"] + 1))
    rms = float(torch.sqrt(torch.mean(u_true * u_true)))
    u_obs = u_true + cfg["noise"] * rms * torch.from_numpy(rng.standard_normal(Vh.ndof)).to(dev)
    kappa = ones

    def ev():
        return torch.cuda.Event(enable_timing=True)

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        P.value_and_grad(kappa, 1.0, u_obs)
    # the timed steps: K gradient evaluations between barriers
    barrier()
    l0 = ffgpu.kernel_launches(di)
    clocks = ClockSampler()
    clocks.start()
    e0, e1 = ev(), ev()
    e0.record(stream)
    for _ in range(args.steps):
        L, gk, gf, u2, lam = P.value_and_grad(kappa, 1.0, u_obs)
    e1.record(stream)
    e1.synchronize()
    barrier()
    clk = clocks.stop()
    launches = ffgpu.kernel_launches(di) - l0
    it_adj = P.A.stats.iterations
    t_grad = e0.elapsed_time(e1) / args.steps
    # the forward solve alone, for the gradient / forward cost ratio
    fwd_ms = []
    for _ in range(args.steps):
        f0, f1 = ev(), ev()
        torch.cuda.synchronize(dev)
        f0.record(stream)
        P.solve(kappa, 1.0)
        f1.record(stream)
        f1.synchronize()
        fwd_ms.append(f0.elapsed_time(f1))
    it_fwd = P.A.stats.iterations
    t_fwd = statistics.median(fwd_ms)
    # central FD on seeded elements (host path of the same library), outside the timed region
    ek = rng.choice(Th.nt, size=cfg["nfd"], replace=False)
    gk_h = gk.cpu().numpy()
    fd = P.fd_gradient(np.ones(Th.nt), np.ones(Th.nt), u_obs.cpu().numpy(), ek, step=1e-6)
    floor = 1e-3 * np.abs(gk_h).max()
    fd_err = float((np.abs(fd - gk_h[ek]) / np.maximum(np.abs(gk_h[ek]), floor)).max())
    # heat variant: forward alone, then forward + checkpointed backward
    H = adjoint.HeatProblem(Vh, dt=cfg["heat_dt"], nsteps=cfg["heat_steps"], on=cfg["on"],
                            checkpoint=cfg["heat_checkpoint"], eps=cfg["eps"], device=di)
    uN, _ = H.forward(k_true, 1.0, keep_checkpoints=False)
    h_obs = uN + cfg["noise"] * float(torch.sqrt(torch.mean(uN * uN))) * torch.from_numpy(
        rng.standard_normal(Vh.ndof)).to(dev)
    hf, hg = [], []
    for k in range(1 + args.steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        H.forward(kappa, 1.0, keep_checkpoints=False)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        H.value_and_grad(kappa, 1.0, h_obs)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if k >= 1:
            hf.append((t1 - t0) * 1e3)
            hg.append((t2 - t1) * 1e3)
    # e2e: the same gradient from host arrays through the public API
    P2 = adjoint.DiffusionProblem(Vh, on=cfg["on"], eps=cfg["eps"], device=di)
    uo_h = u_obs.cpu().numpy()
    e2e = []
    for k in range(1 + args.steps):
        t0 = time.perf_counter()
        P2.value_and_grad(np.ones(Th.nt), np.ones(Th.nt), uo_h)
        if k >= 1:
            e2e.append((time.perf_counter() - t0) * 1e3)
    t_e2e = statistics.median(e2e)
    t_grad, t_e2e = dist_max([t_grad, t_e2e], world, dev)
    if rank != 0:
        return None
    value = world * Vh.ndof / (t_grad * 1e-3)
    cb, _ = (None, None) if args.no_cpu_baseline else cpu_baseline(args.config, procs=1)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t_grad, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": args.config, "mesh": f"square({n})", "fe": "P1", "ndof": Vh.ndof,
                      "params": Th.nt, "eps": cfg["eps"], "step": "L and dL/dkappa, dL/df at kappa=1",
                      "forward_ms": t_fwd, "gradient_ms": t_grad,
                      "gradient_over_forward": t_grad / t_fwd, "cg_iterations_forward": it_fwd,
                      "cg_iterations_adjoint": it_adj, "fd_elements": int(cfg["nfd"]),
                      "fd_max_rel_err": fd_err,
                      "heat": {"steps": cfg["heat_steps"], "dt": cfg["heat_dt"],
                               "checkpoint": cfg["heat_checkpoint"], "forward_ms": statistics.median(hf),
                               "gradient_ms": statistics.median(hg),
                               "gradient_over_forward": statistics.median(hg) / statistics.median(hf),
                               "solves_gradient": H.solves},
                      "l2": "working set below L2 (square(512)); timing is of repeated gradients"},
           "e2e": {"value": world * Vh.ndof / (t_e2e * 1e-3), "unit": UNIT,
                   "h2d_bytes_per_step": int(2 * Th.nt * 8 + Vh.ndof * 8),
                   "d2h_bytes_per_step": int(2 * Th.nt * 8 + 2 * Vh.ndof * 8), "ms_per_step": t_e2e},
           "gpu_launches": int(launches), "clocks": clk, "roofline": None,
           "roofline_note": "square(512): matrix and vectors stay in L2 between kernels; no HBM roofline"}
    if cb:
        out["cpu_baseline"] = cb
    print(json.dumps(out))


def run_batch(args, rank=0, world=1):
    """Batched independent problems: one assembly pass and one persistent solve per step.  On
    N ranks every rank solves its own batch of the same size (seed + rank): weak scaling, no
    collective on the data path; value = the DOFs of all ranks / the slowest rank's time."""
    import numpy as np
    import torch
    import ffgpu
    from ffgpu import batch
    from ffgpu.build import build
    build()
    cfg = CONFIGS[args.config]
    di = rank_device(rank, world)
    dev = torch.device("cuda", di)
    torch.cuda.set_device(dev)
    meshes, kappas, Ns = batch.c5_meshes(cfg["nprob"], cfg["nmin"], cfg["nmax"], seed=cfg["seed"] + rank)
    ndof = int(sum(m.nv for m in meshes))
    ffgpu.context(di)
    stream = torch.cuda.ExternalStream(ffgpu.stream_handle(di), device=dev)
    B = batch.Batch(meshes, device=di)
    kap = torch.from_numpy(np.concatenate(kappas)).to(dev)
    x = torch.zeros(ndof, dtype=torch.float64, device=dev)

    def step():
        B.assemble(kap, f=1.0)
        return B.solve(eps=cfg["eps"], out=x)

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    l0 = ffgpu.kernel_launches(di)
    clocks = ClockSampler()
    clocks.start()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    e1.synchronize()
    barrier()
    clk = clocks.stop()
    launches = ffgpu.kernel_launches(di) - l0
    ms = e0.elapsed_time(e1) / args.steps
    ms, = dist_max([ms], world, dev)
    ndof_all, = dist_sum([ndof], world, dev)
    solve_ms = B.stats.elapsed_ms
    nt_, lanes, tms = B.tuned()
    # accuracy against the FP64 oracle on a sample of problems
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ffo
    from ffgpu.fespace import FESpace
    xs = B.split(x.cpu().numpy())
    errs = []
    rng = np.random.Generator(np.random.PCG64(1))
    for p in rng.choice(len(meshes), size=8, replace=False):
        Th = meshes[p]
        Vh = FESpace(Th, "P1")
        A = ffo.assemble(Th, Vh, kappa=kappas[p])
        bo = ffo.rhs(Th, Vh, f=1.0)
        ffo.setbc(A, bo, Vh.on((1, 2, 3, 4)))
        uo, it, r, _ = ffo.cg(A, bo, eps=1e-10)
        errs.append(float(np.linalg.norm(xs[p] - uo) / np.linalg.norm(uo)))
    # e2e from host arrays: the batch as the C ABI takes it (counts, coordinates, elements,
    # on() mask, coefficients back to back), copied in and solved every step
    arrays = batch.batch_arrays(meshes)
    kap_h = np.concatenate(kappas)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        B2 = batch.Batch(arrays=arrays, device=di)
        B2.assemble(kap_h, f=1.0)
        xh = B2.solve(eps=cfg["eps"])
        B2.close()
    t_e2e = (time.perf_counter() - t0) * 1e3 / args.steps
    t_e2e, = dist_max([t_e2e], world, dev)
    if rank != 0:
        return None
    h2d = sum(m.coords.nbytes + m.elems.nbytes for m in meshes) + sum(k.nbytes for k in kappas) + ndof
    # CPU: the oracle (single core) on 16 sampled problems, FP64 CG to the same eps
    t0 = time.perf_counter()
    nd = 0
    for p in rng.choice(len(meshes), size=16, replace=False):
        Th = meshes[p]
        Vh = FESpace(Th, "P1")
        A = ffo.assemble(Th, Vh, kappa=kappas[p])
        bo = ffo.rhs(Th, Vh, f=1.0)
        ffo.setbc(A, bo, Vh.on((1, 2, 3, 4)))
        ffo.cg(A, bo, eps=cfg["eps"])
        nd += Vh.ndof
    cpu_v = nd / (time.perf_counter() - t0)
    peaks = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(REPO, "MEASURED_PEAKS.json")) else {}
    out = {"metric": METRIC, "value": ndof_all / (ms * 1e-3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 inner / f64 refinement", "data": "synthetic",
           "config": {"workload": args.config, "nprob": len(meshes), "ndof": ndof,
                      "parallelism": f"{world} ranks, one batch each" if world > 1 else "single GPU",
                      "N_range": [int(Ns.min()), int(Ns.max())], "eps": cfg["eps"],
                      "solve_ms": solve_ms, "inner_iterations_total": int(B.stats.iterations),
                      "max_outer": int(B.stats.outer_iterations), "tuned_cta_threads": nt_,
                      "tuned_lanes_per_row": lanes, "rel_err_vs_fp64_oracle_max": max(errs),
                      "l2": "working set %.0f MB" % ((ndof * 7 * 12) / 1e6)},
           "e2e": {"value": ndof_all / (t_e2e * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                   "d2h_bytes_per_step": int(ndof * 8), "ms_per_step": t_e2e},
           "gpu_launches": int(launches), "clocks": clk,
           "cpu_baseline": {"value": cpu_v, "unit": UNIT, "cores": 1, "kind": "port",
                            "sample": "16 of the batch's problems, oracle FP64 CG, single core"},
           "roofline": None, "peak_hbm_gbs": peaks.get("hbm_gbs"),
           "roofline_note": "one persistent launch over 1024 small problems (each CTA's problem in L1/L2)"}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="elasticity_p2_cube64", choices=sorted(CONFIGS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--profile-case", choices=["elasticity", "diffusion3d", "poisson2d"], default=None,
                    help="run a small case for ncu instead of the benchmark")
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--iters", type=int, default=40)
    ap.add_argument("--spmv-mode", type=int, default=0,
                    help="profile case: 0 FP64 CG, 1 double-float SpMV CG, 2 FP32-inner refinement")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case, args.n, args.iters, args.spmv_mode)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    special = CONFIGS[args.config].get("batch") or CONFIGS[args.config].get("adjoint")
    if special and args.impl != "reference":
        if world > 1:
            import torch
            torch.distributed.init_process_group("nccl")
        if CONFIGS[args.config].get("batch"):
            run_batch(args, rank, world)
        else:
            run_adjoint(args, rank, world)
        if world > 1:
            import torch
            torch.distributed.destroy_process_group()
        return
    if args.impl == "reference":
        if rank != 0:
            return
        procs = os.cpu_count() or 1
        vals = []
        for _ in range(args.warmup + args.steps):
            cb, wall = cpu_baseline(args.config, procs=procs)
            vals.append((cb, wall))
        timed = vals[args.warmup:]
        value = statistics.median(v[0]["value"] for v in timed)
        cb = timed[-1][0]
        cb["value"] = value
        print(json.dumps({
            "metric": METRIC, "impl": "reference", "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.median(v[1] for v in timed) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.config}, "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    out = run_gpu(args, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            cb, _ = cpu_baseline(args.config, procs=1)
            out["cpu_baseline"] = cb
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
