"""Benchmark of the FreeFEM assemble-and-solve path on one GB300.

Headline workload (default): 3D linear elasticity on the unit cube, cube(64,64,64) split into
6 tets per hexahedron (1,572,864 tets), [P2,P2,P2] (6,440,067 DOFs), E=1, nu=0.3, clamped on the
face x=0 (label 4), body force (0,0,-1), FP64, Jacobi-PCG to FreeFEM's eps=1e-10.  A step is one
full pass of the path from the mesh + DOF table to the solution:
    space setup (node->element incidence) + matrix A = a(Vh,Vh) (pattern, values, tgv)
    + b = a(0,Vh) (same pass) + u[] = A^-1*b (CG)
value: inputs (coordinates, elements, DOF table) resident in HBM before the timed region.
e2e:   the same through the public API from host (numpy) arrays, host<->device copies timed.
The matrix (~6 GB) is larger than L2 (129 MB), so no flush is needed between its steps.

The default run also measures the four other workloads of the same family and puts each in
`workloads` of the one JSON line, with its own value, e2e, roofline, CPU baseline and accuracy
against the FP64 oracle: 2D P1 Poisson on square(256); 3D P1 diffusion with a lognormal P0
kappa on cube(160), FP64 CG against FP32-inner / FP64-refinement; the adjoint gradient of a 2D
inverse diffusion problem on square(512) (and its implicit-Euler heat variant); 1024 batched
jittered squares.  Working sets below L2 are timed with an L2 flush between steps.

--impl reference times the oracle port of FreeFEM's CPU path (oracle/ffo.c, pinned bit for bit
to FreeFEM's own HashMatrix + ConjugueGradient) on all host cores, one single-threaded instance
per core (FreeFEM's core is single-threaded).  Workloads small enough for the host run at full
size; cube(64) [P2]^3 and cube(160) P1 (an hour and minutes per instance) are timed at four
smaller sizes of the same varf every step and extrapolated: assembly linear in the elements,
CG iterations linear in n, time per iteration linear in nnz (nnz is an exact cubic in n).
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
DEFAULT = "elasticity_p2_cube64"

CONFIGS = {
    "elasticity_p2_cube64": dict(mesh=("cube", 64), kind="P2vec", form="elasticity", on=(4,),
                                 eps=1e-10),
    "poisson_p1_square256": dict(mesh=("square", 256), kind="P1", form="diffusion",
                                 on=(1, 2, 3, 4), eps=1e-10, small=True),
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
# the workloads measured after the headline, in this order
SUB_ORDER = ["poisson_p1_square256", "diffusion_p1_cube160", "inverse_diffusion_p1_square512",
             "batched_p1_1024"]
# bounded single-core CPU sample of our arm's cpu_baseline (and the size of its oracle check)
SAMPLE = {"elasticity_p2_cube64": ("cube", 12), "poisson_p1_square256": ("square", 256),
          "diffusion_p1_cube160": ("cube", 40), "batched_p1_1024": ("square", 64),
          "inverse_diffusion_p1_square512": ("square", 256)}
# sizes the reference arm times and extrapolates from (workloads too large for the host)
REF_FIT = {"elasticity_p2_cube64": (6, 8, 10, 12), "diffusion_p1_cube160": (16, 24, 32, 40)}


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


def rel_err(u, ref):
    import numpy as np
    u = u.cpu().numpy() if hasattr(u, "cpu") else np.asarray(u)
    return float(np.linalg.norm(u - ref) / np.linalg.norm(ref))


# ------------------------------------------------------------------ CPU: the oracle port
def _oracle_run(args):
    """One single-threaded oracle solve of a workload at `size`: assemble + rhs + on() + CG.
    Returns the sizes, the assembly and CG times, the iterations (and the solution on request)."""
    cfgname, size, want_u = args
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
    t1 = time.perf_counter()
    u, it, r, _ = ffo.cg(A, b, eps=cfg["eps"])
    t2 = time.perf_counter()
    return dict(ndof=Vh.ndof, nt=Th.nt, nnz=A.nnz, t_asm=t1 - t0, t_cg=t2 - t1, t=t2 - t0, its=it,
                size=size, u=u if want_u else None)


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
    return dict(ndof=Vh.ndof, nt=Th.nt, nnz=A.nnz, t=dt, its=it + it2, size=size, u=None)


def _oracle_batch_run(args):
    """Oracle FP64 CG of problems `idx` of the batched workload (regenerated from its seed)."""
    cfgname, idx = args
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ffo
    from ffgpu import batch
    from ffgpu.fespace import FESpace
    cfg = CONFIGS[cfgname]
    meshes, kappas, _ = batch.c5_meshes(cfg["nprob"], cfg["nmin"], cfg["nmax"], seed=cfg["seed"])
    t0 = time.perf_counter()
    nd = its = 0
    for p in idx:
        Th = meshes[p]
        Vh = FESpace(Th, "P1")
        A = ffo.assemble(Th, Vh, kappa=kappas[p])
        bo = ffo.rhs(Th, Vh, f=1.0)
        ffo.setbc(A, bo, Vh.on((1, 2, 3, 4)))
        its += ffo.cg(A, bo, eps=cfg["eps"])[1]
        nd += Vh.ndof
    return dict(ndof=nd, t=time.perf_counter() - t0, its=its)


def cpu_baseline(cfgname, want_u=False):
    """DOFs/s of one single-threaded oracle instance on the bounded sample of the workload;
    with want_u also the oracle's run (its solution) for the accuracy check of the GPU path."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ffo
    ffo.build()
    size = SAMPLE[cfgname]
    r = _oracle_run((cfgname, size, want_u))
    what = ("forward CG + transpose CG + P0 sensitivities" if CONFIGS[cfgname].get("adjoint")
            else "full assemble+rhs+CG")
    cb = dict(value=r["ndof"] / r["t"], unit=UNIT, cores=1, kind="port",
              sample=f"{size[0]}({size[1]}) same varf, {what} (eps={CONFIGS[cfgname]['eps']}), "
                     f"{r['its']} CG iterations, single-threaded oracle (oracle/ffo.c)")
    return cb, r


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


_FLUSH = {}


def flush_l2(dev):
    """Writes 256 MB (twice the 129 MB L2) so that the next step starts from HBM."""
    import torch
    buf = _FLUSH.get(dev)
    if buf is None:
        buf = _FLUSH[dev] = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    buf.fill_(1.0)
    torch.cuda.synchronize(dev)


def pinned(a):
    """A page-locked host copy of a numpy array (the e2e legs copy from pinned memory)."""
    import numpy as np
    import torch
    a = np.ascontiguousarray(a)
    t = torch.empty(a.shape, dtype=torch.from_numpy(a[:0] if a.ndim else a.reshape(1)[:0]).dtype,
                    pin_memory=True)
    out = t.numpy()           # the array keeps the pinned tensor alive
    out[...] = a
    return out


def pinned_problem(Th, Vh, a):
    """The mesh, FE space and varf with every array the e2e leg hands over in pinned memory."""
    import copy
    Th_p = dataclasses.replace(Th, coords=pinned(Th.coords), elems=pinned(Th.elems),
                               belems=pinned(Th.belems), blabel=pinned(Th.blabel))
    Vh_p = copy.copy(Vh)
    Vh_p.Th = Th_p
    Vh_p.dof = Th_p.elems if Vh.kind == "P1" else pinned(Vh.dof)
    import numpy as np
    kap = getattr(a, "kappa", None)
    a_p = dataclasses.replace(a, kappa=pinned(kap)) if isinstance(kap, np.ndarray) else a
    return Th_p, Vh_p, a_p


def peak_hbm():
    try:
        return float(json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))["hbm_gbs"]), \
            "MEASURED_PEAKS.json hbm_gbs (measured)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s (no MEASURED_PEAKS.json)"


# ------------------------------------------------------------------ GPU arm: one problem
def run_gpu(args, cfgname, steps, warmup, rank, world, variants=(), cpu=True):
    """Assemble + solve of one problem per rank (C1, C2, C3); `variants` from "doublefloat"
    (FP64 CG with the double-float SpMV), "mixed" (FP32 inner / FP64 refinement), "gmres",
    "cholesky" (the direct solver)."""
    import numpy as np
    import torch
    import ffgpu
    cfg = CONFIGS[cfgname]
    small = cfg.get("small", False)
    dev = rank_device(rank, world)
    torch.cuda.set_device(dev)
    Th, Vh, a, _ = build_problem(cfg)
    ffgpu.context(dev)
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
        return S, A, u, t[0].elapsed_time(t[3])

    def barrier():
        torch.cuda.synchronize(dev)
        if world > 1:
            torch.distributed.barrier()

    for _ in range(warmup):
        S, A, u, _ = step_device()
        del A, S
    barrier()
    clocks = ClockSampler()
    clocks.start()
    l0 = ffgpu.kernel_launches(dev)
    times, iters = [], []
    for k in range(steps):
        if small:
            flush_l2(dev)
        S, A, u, ms = step_device()
        times.append(ms)
        iters.append(A.stats.iterations)
        keep = (S, A, u)
    barrier()
    launches = ffgpu.kernel_launches(dev) - l0
    clk = clocks.stop()
    S, A, u = keep
    # accuracy: relative residual of the solution on non-tgv rows
    r = A.mult(u)
    rh = (b - r).cpu().numpy()
    mask = onbc.astype(bool)
    rel_res = float(np.linalg.norm(rh[~mask]) / np.linalg.norm(b.cpu().numpy()[~mask]))
    # dominant kernel: the SpMV of the CG (K_a, with its fused dot), in the layout the tuner
    # chose, launched back to back on the library stream and timed there with CUDA events
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
        stored = ent * (8 * bs * bs + col_bytes) + 4 * nb + 8 * n + 8 * n
    else:
        stored = 8 * nnz + 4 * nnzb + 4 * (nb + 1) + 8 * n + 8 * n
    achieved = spmv_bytes / (spmv_avg * 1e-3) / 1e9
    peak, peak_src = peak_hbm()
    traffic = None
    try:
        tr = json.load(open(os.path.join(REPO, "profiles", "traffic.json")))
        traffic = tr.get(cfgname, {}).get("spmv_bytes_per_launch")
    except Exception:
        pass
    cluster = bool(ffgpu.lib().ffgpu_matrix_spmv_layout(A.h, 5))
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": traffic,
            "kernel": f"FP64 SpMV of the CG (K_a), layout {layout}, block size {bs}",
            "bytes_per_launch": spmv_bytes, "ms_per_launch": spmv_avg,
            "stored_bytes_per_launch": stored,
            "frac_of_stored_bytes": stored / (spmv_avg * 1e-3) / 1e9 / peak,
            "peak_source": peak_src}
    if cluster:
        # the whole CG loop is one kernel (one thread-block cluster): its time per iteration
        # against the algorithmic bytes of one fused PCG iteration, B_spmv + 56 n; the matrix
        # (below L2) streams from L2, so HBM is not what bounds it
        its_c = max(1, iters[-1])
        it_ms = statistics.median(phase["solve"][-steps:]) / its_c
        b_it = spmv_bytes + 56 * n
        ach = b_it / (it_ms * 1e-3) / 1e9
        roof = {"bound": "latency / L2 (whole CG loop in one cluster of thread blocks)", "achieved": ach,
                "peak": peak, "unit": "GB/s", "frac": ach / peak, "traffic": None,
                "kernel": "cg_cluster (one launch per solve, %d iterations)" % its_c,
                "bytes_per_iteration": b_it, "ms_per_iteration": it_ms, "peak_source": peak_src,
                "regular_path_spmv": {"kernel": f"K_a, layout {layout}", "ms_per_launch": spmv_avg,
                                      "frac": achieved / peak}}
    u_ref = u.clone()
    var = {}
    elem = None
    if cfg["kind"] in ("P2", "P2vec"):
        # the assembly with the element matrices from the tensor cores (the default) and from
        # the FP64 path inside the row gather, on the same inputs (median of 2 after 1 warm-up)
        def asm_ms(tc):
            os.environ["FFGPU_ELEM_TC"] = "1" if tc else "0"
            try:
                ts = []
                for _ in range(3):
                    S2 = ffgpu.DeviceSpace(Vh, device=dev, coords=X, elems=E, dof=D, belems=BE, blabel=BL)
                    e0 = torch.cuda.Event(enable_timing=True)
                    e1 = torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    A2 = ffgpu.matrix(a, S2, eps=cfg["eps"], itmax=ITMAX, rhs_out=b, device=dev)
                    e1.record(stream)
                    e1.synchronize()
                    ts.append(e0.elapsed_time(e1))
                    del A2, S2
                return statistics.median(ts[1:])
            finally:
                del os.environ["FFGPU_ELEM_TC"]
        elem = {"path": "tensor cores: tcgen05.mma kind::f16, features as five exact 11-bit digits",
                "assemble_ms_tensor_cores": asm_ms(True), "assemble_ms_fp64_elements": asm_ms(False)}

    def timed_variant(fn, reps):
        out, ms = None, []
        for r in range(reps + 1):
            if small:
                flush_l2(dev)
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

    solve_fp64 = statistics.median(phase["solve"][-steps:])
    if "gmres" in variants:
        # solver=GMRES (FreeFEM's fgmres with its default restart, 1000) on the same system: its
        # own step time, iterations and time per iteration, error against the FP64 CG solution
        def run_gm():
            S2 = ffgpu.DeviceSpace(Vh, device=dev, coords=X, elems=E, dof=D, belems=BE, blabel=BL)
            A2 = ffgpu.matrix(a, S2, solver="GMRES", eps=cfg["eps"], itmax=ITMAX, dim_krylov=1000, rhs_out=b,
                              device=dev)
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            ug = A2.solve(b)
            t1.record(stream)
            t1.synchronize()
            return ug, A2.stats.iterations, A2.stats.residual, t0.elapsed_time(t1)
        (ugm, itgm, resgm, solve_gm_ms), msgm = timed_variant(run_gm, 3)
        var["fp64_gmres_restart1000"] = {
            "value": Vh.ndof / (msgm * 1e-3), "ms_per_step": msgm, "iterations": itgm,
            "solve_ms": solve_gm_ms, "ms_per_iteration": solve_gm_ms / max(1, itgm),
            "relative_residual": resgm,
            "rel_err_vs_fp64_cg": float(torch.linalg.norm(ugm - u_ref) / torch.linalg.norm(u_ref))}
    if "cholesky" in variants:
        # the direct solver on the same system: ordering + analysis + factorisation + solve in
        # the first call, then solves alone on the kept factorisation
        def run_ch():
            S2 = ffgpu.DeviceSpace(Vh, device=dev, coords=X, elems=E, dof=D, belems=BE, blabel=BL)
            A2 = ffgpu.matrix(a, S2, solver="CHOLESKY", rhs_out=b, device=dev)
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            t0.record(stream)
            uc = A2.solve(b)
            t1.record(stream)
            t1.synchronize()
            t2 = time.perf_counter()
            A2.solve(b)
            return uc, t0.elapsed_time(t1), (time.perf_counter() - t2) * 1e3
        (uch, first_ms, again_ms), msch = timed_variant(run_ch, 2)
        var["fp64_direct_cholesky"] = {
            "value": Vh.ndof / (msch * 1e-3), "ms_per_step": msch,
            "factor_and_solve_ms": first_ms, "solve_on_kept_factor_ms": again_ms,
            "rel_err_vs_fp64_cg": float(torch.linalg.norm(uch - u_ref) / torch.linalg.norm(u_ref))}
    if "doublefloat" in variants:
        def run_df():
            S2 = ffgpu.DeviceSpace(Vh, device=dev, coords=X, elems=E, dof=D, belems=BE, blabel=BL)
            A2 = ffgpu.matrix(a, S2, eps=cfg["eps"], itmax=ITMAX, rhs_out=b, device=dev)
            return A2.solve(b, spmv_mode=1), A2.stats.iterations, A2.spmv_layout(1), A2
        (udf, itdf, lay, Adf), msdf = timed_variant(run_df, 2)
        var["fp64_values_doublefloat_spmv"] = {
            "value": Vh.ndof / (msdf * 1e-3), "ms_per_step": msdf, "cg_iterations": itdf,
            "spmv_layout": lay, "spmv_ms": Adf.time_spmv(1, 10),
            "rel_err_vs_fp64": float(torch.linalg.norm(udf - u_ref) / torch.linalg.norm(u_ref))}
        del Adf
    if "mixed" in variants:
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
        (uir, itir, outir, lay32, solve_ir_ms, Air), msir = timed_variant(run_ir, 2)
        var["mixed_fp32_inner_fp64_refinement"] = {
            "value": Vh.ndof / (msir * 1e-3), "ms_per_step": msir, "inner_iterations": itir,
            "outer_iterations": outir, "spmv_layout": lay32, "spmv_ms": Air.time_spmv(2, 10),
            "solve_ms": solve_ir_ms,
            "solve_speedup_vs_fp64": solve_fp64 / solve_ir_ms,
            "rel_err_vs_fp64": float(torch.linalg.norm(uir - u_ref) / torch.linalg.norm(u_ref))}
        del Air
    # e2e: public API from pinned host arrays (H2D of mesh/DOF table/P0 coefficient, D2H of b
    # and u; the solve starts from u = 0 as FreeFEM's first solve does)
    e2e_times = []
    Th_p, Vh_p, a_p = pinned_problem(Th, Vh, a_host)
    bh = pinned(np.zeros(Vh.ndof))
    uh = pinned(np.zeros(Vh.ndof))
    w_e2e = max(1, warmup // 3)
    for s in range(w_e2e + steps):
        if small:
            flush_l2(dev)
        barrier()
        t0 = time.perf_counter()
        Ah = ffgpu.matrix(a_p, Vh_p, eps=cfg["eps"], itmax=ITMAX, rhs_out=bh, device=dev)
        uh.fill(0.0)
        Ah.solve(bh, out=uh)
        t1 = time.perf_counter()
        if s >= w_e2e:
            e2e_times.append((t1 - t0) * 1e3)
        del Ah
    # P1 crosses no DOF table (its DOFs are the vertices); the P0 coefficient does cross
    h2d = (Th.coords.nbytes + Th.elems.nbytes + (0 if Vh.kind == "P1" else Vh.dof.nbytes) + Th.belems.nbytes
           + Th.blabel.nbytes + bh.nbytes + (a_host.kappa.nbytes if a_host.kappa is not None else 0))
    d2h = bh.nbytes + uh.nbytes
    t_step = sum(times) / len(times)
    t_e2e = sum(e2e_times) / len(e2e_times)
    t_step, t_e2e = dist_max([t_step, t_e2e], world, torch.device("cuda", dev))
    if rank != 0:
        return None
    value = world * Vh.ndof / (t_step * 1e-3)
    e2e_value = world * Vh.ndof / (t_e2e * 1e-3)
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
        "warmup": warmup, "ms_per_step": t_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": cfgname, "mesh": f"{cfg['mesh'][0]}({cfg['mesh'][1]})",
                   "fe": cfg["kind"], "ndof": Vh.ndof, "nnz": nnz, "nt": Th.nt,
                   "solver": "Jacobi-PCG", "eps": cfg["eps"], "cg_iterations": iters[-1],
                   "l2": ("working set below L2: L2 flushed (256 MB written) before every timed step"
                          if small else "inputs larger than L2 (matrix %.1f GB)" % (nnz * 8 / 1e9)),
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "space_ms": statistics.median(phase["space"][-steps:]),
                   "assemble_ms": statistics.median(phase["assemble"][-steps:]),
                   "solve_ms": solve_fp64,
                   "ms_per_cg_iteration": solve_fp64 / max(1, iters[-1]),
                   "spmv_layout": layout,
                   "cg_path": ("one thread-block cluster (whole iteration loop in one kernel)"
                               if cluster else "CUDA graph of K_a, K_b, K_c per iteration"),
                   "rel_residual": rel_res,
                   "element_matrices": elem},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": t_e2e},
        "gpu_launches": int(launches),
        "roofline": roof,
        "assembly_roofline": assembly_roofline(Th, Vh, cfg, statistics.median(phase["assemble"][-steps:]), peak),
        "clocks": clk,
        "variants": var,
    }
    if cpu:
        cb, orc = cpu_baseline(cfgname, want_u=True)
        out["cpu_baseline"] = cb
        out["oracle_check"] = oracle_check(cfgname, orc, dev, mixed="mixed" in variants)
    return out


def oracle_check(cfgname, orc, dev, mixed):
    """The GPU path (public API, FP64 CG and, with `mixed`, the FP32-inner refinement) on the
    oracle's sample problem, against the oracle's FP64 solution of the same inputs."""
    import ffgpu
    cfg = CONFIGS[cfgname]
    Th, Vh, a, np = build_problem(cfg, orc["size"])
    b = np.empty(Vh.ndof)
    A = ffgpu.matrix(a, Vh, eps=cfg["eps"], itmax=ITMAX, rhs_out=b, device=dev)
    u = A.solve(b)
    out = {"sample": "%s(%d)" % orc["size"], "ndof": Vh.ndof, "nnz": A.nnz, "oracle_nnz": orc["nnz"],
           "cg_iterations": A.stats.iterations, "oracle_cg_iterations": orc["its"],
           "rel_err_fp64_vs_oracle": rel_err(u, orc["u"])}
    if mixed:
        um = A.solve_mixed(b, eps=cfg["eps"])
        out["rel_err_mixed_vs_oracle"] = rel_err(um, orc["u"])
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


def profile_case(kind, n, iters, spmv_mode, solver="CG", dim_krylov=1000):
    """Small case for ncu: space + assembly + a fixed number of CG (or GMRES) iterations, twice."""
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
        A = ffgpu.matrix(a, S, solver=solver, eps=1e-10, itmax=iters, dim_krylov=dim_krylov, rhs_out=b)
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


# ------------------------------------------------------------------ GPU arm: adjoint (C4)
def run_adjoint(args, cfgname, steps, warmup, rank, world, cpu=True):
    """dL/dkappa by the adjoint (forward CG, transpose CG, sensitivity kernel) on the device;
    the heat variant with checkpoint-and-recompute; FD check on seeded elements.  A step is one
    gradient evaluation (L, dL/dkappa, dL/df at kappa = 1, its forward solve included); on N
    ranks every rank evaluates its own replica (weak scaling, no collective on the data path).
    The system (square(512)) fits in L2: L2 is flushed before every timed step."""
    import numpy as np
    import torch
    import ffgpu
    from ffgpu import adjoint
    from ffgpu.fespace import FESpace
    cfg = CONFIGS[cfgname]
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

    for _ in range(warmup):
        P.value_and_grad(kappa, 1.0, u_obs)
    barrier()
    l0 = ffgpu.kernel_launches(di)
    clocks = ClockSampler()
    clocks.start()
    grad_ms = []
    for _ in range(steps):
        flush_l2(di)
        e0, e1 = ev(), ev()
        e0.record(stream)
        L, gk, gf, u2, lam = P.value_and_grad(kappa, 1.0, u_obs)
        e1.record(stream)
        e1.synchronize()
        grad_ms.append(e0.elapsed_time(e1))
    barrier()
    clk = clocks.stop()
    launches = ffgpu.kernel_launches(di) - l0
    it_adj = P.A.stats.iterations
    t_grad = sum(grad_ms) / len(grad_ms)
    # the forward solve alone, for the gradient / forward cost ratio
    fwd_ms = []
    for _ in range(steps):
        flush_l2(di)
        f0, f1 = ev(), ev()
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
    for k in range(1 + max(1, steps // 3)):
        torch.cuda.synchronize()
        H.iterations_state = 0
        t0 = time.perf_counter()
        H.forward(kappa, 1.0, keep_checkpoints=False)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        heat_fwd_its = H.iterations_state
        H.value_and_grad(kappa, 1.0, h_obs)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        if k >= 1:
            hf.append((t1 - t0) * 1e3)
            hg.append((t2 - t1) * 1e3)
    # e2e: the same gradient from host arrays through the public API
    P2 = adjoint.DiffusionProblem(Vh, on=cfg["on"], eps=cfg["eps"], device=di)
    uo_h = pinned(u_obs.cpu().numpy())
    kap_h, f_h = pinned(np.ones(Th.nt)), pinned(np.ones(Th.nt))
    e2e = []
    for k in range(1 + steps):
        flush_l2(di)
        t0 = time.perf_counter()
        P2.value_and_grad(kap_h, f_h, uo_h)
        if k >= 1:
            e2e.append((time.perf_counter() - t0) * 1e3)
    t_e2e = statistics.median(e2e)
    t_grad, t_e2e = dist_max([t_grad, t_e2e], world, dev)
    if rank != 0:
        return None
    value = world * Vh.ndof / (t_grad * 1e-3)
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps,
           "warmup": warmup, "ms_per_step": t_grad, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": cfgname, "mesh": f"square({n})", "fe": "P1", "ndof": Vh.ndof,
                      "params": Th.nt, "eps": cfg["eps"], "step": "L and dL/dkappa, dL/df at kappa=1",
                      "forward_ms": t_fwd, "gradient_ms": t_grad,
                      "gradient_over_forward": t_grad / t_fwd, "cg_iterations_forward": it_fwd,
                      "cg_iterations_adjoint": it_adj, "fd_elements": int(cfg["nfd"]),
                      "fd_max_rel_err": fd_err,
                      "heat": {"steps": cfg["heat_steps"], "dt": cfg["heat_dt"],
                               "checkpoint": cfg["heat_checkpoint"], "forward_ms": statistics.median(hf),
                               "gradient_ms": statistics.median(hg),
                               "gradient_over_forward": statistics.median(hg) / statistics.median(hf),
                               "solves_gradient": H.solves,
                               "cg_iterations_forward": heat_fwd_its,
                               "cg_iterations_gradient_state_solves": H.iterations_state,
                               "cg_iterations_gradient_adjoint_solves": H.iterations_adjoint},
                      "l2": "working set below L2: L2 flushed (256 MB written) before every timed step"},
           "e2e": {"value": world * Vh.ndof / (t_e2e * 1e-3), "unit": UNIT,
                   "h2d_bytes_per_step": int(2 * Th.nt * 8 + Vh.ndof * 8),
                   "d2h_bytes_per_step": int(2 * Th.nt * 8 + 2 * Vh.ndof * 8), "ms_per_step": t_e2e},
           "gpu_launches": int(launches), "clocks": clk, "roofline": None,
           "roofline_note": "square(512): 1.8 M nonzeros, latency-bound chain of small kernels; no HBM roofline"}
    if cpu:
        out["cpu_baseline"], _ = cpu_baseline(cfgname)
    return out


# ------------------------------------------------------------------ GPU arm: batched (C5)
def run_batch(args, cfgname, steps, warmup, rank, world, cpu=True):
    """Batched independent problems: one assembly pass and one persistent solve per step.  On
    N ranks every rank solves its own batch of the same size (seed + rank): weak scaling, no
    collective on the data path; value = the DOFs of all ranks / the slowest rank's time."""
    import numpy as np
    import torch
    import ffgpu
    from ffgpu import batch
    cfg = CONFIGS[cfgname]
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

    for _ in range(warmup):
        step()
    barrier()
    l0 = ffgpu.kernel_launches(di)
    clocks = ClockSampler()
    clocks.start()
    ms_steps = []
    for _ in range(steps):
        flush_l2(di)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        ms_steps.append(e0.elapsed_time(e1))
    barrier()
    clk = clocks.stop()
    launches = ffgpu.kernel_launches(di) - l0
    ms = sum(ms_steps) / len(ms_steps)
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
    arrays = tuple(pinned(x) for x in batch.batch_arrays(meshes))
    kap_h = pinned(np.concatenate(kappas))
    xh = pinned(np.zeros(ndof))
    e2e = []
    for _ in range(steps):
        flush_l2(di)
        barrier()
        t0 = time.perf_counter()
        B2 = batch.Batch(arrays=arrays, device=di)
        B2.assemble(kap_h, f=1.0)
        B2.solve(eps=cfg["eps"], out=xh)   # x is written, not read (each problem starts at 0)
        B2.close()
        e2e.append((time.perf_counter() - t0) * 1e3)
    t_e2e = sum(e2e) / len(e2e)
    t_e2e, = dist_max([t_e2e], world, dev)
    if rank != 0:
        return None
    h2d = sum(m.coords.nbytes + m.elems.nbytes for m in meshes) + sum(k.nbytes for k in kappas) + ndof
    out = {"metric": METRIC, "value": ndof_all / (ms * 1e-3), "unit": UNIT, "n_gpus": world, "steps": steps,
           "warmup": warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 inner / f64 refinement", "data": "synthetic",
           "config": {"workload": cfgname, "nprob": len(meshes), "ndof": ndof,
                      "parallelism": f"{world} ranks, one batch each" if world > 1 else "single GPU",
                      "N_range": [int(Ns.min()), int(Ns.max())], "eps": cfg["eps"],
                      "solve_ms": solve_ms, "inner_iterations_total": int(B.stats.iterations),
                      "max_outer": int(B.stats.outer_iterations), "tuned_cta_threads": nt_,
                      "tuned_lanes_per_row": lanes, "rel_err_vs_fp64_oracle_max": max(errs),
                      "oracle_sample": "8 problems, oracle FP64 CG to 1e-10",
                      "l2": "working set %.0f MB: L2 flushed (256 MB written) before every timed step"
                            % ((ndof * 7 * 12) / 1e6)},
           "e2e": {"value": ndof_all / (t_e2e * 1e-3), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                   "d2h_bytes_per_step": int(ndof * 8), "ms_per_step": t_e2e},
           "gpu_launches": int(launches), "clocks": clk,
           "roofline": None, "peak_hbm_gbs": peak_hbm()[0],
           "roofline_note": "one persistent launch over 1024 small problems (each CTA's problem in L1/L2)"}
    if cpu:
        # the oracle (single core) on 16 of the batch's problems, FP64 CG to the same eps
        idx = [int(p) for p in rng.choice(len(meshes), size=16, replace=False)]
        r = _oracle_batch_run((cfgname, idx))
        out["cpu_baseline"] = {"value": r["ndof"] / r["t"], "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": "16 of the batch's problems, oracle FP64 CG, single core"}
    return out


VARIANTS = {"elasticity_p2_cube64": ("doublefloat", "mixed"), "poisson_p1_square256": ("gmres", "cholesky"),
            "diffusion_p1_cube160": ("doublefloat", "mixed")}


def run_config(args, cfgname, steps, warmup, rank, world, variants=True, cpu=True):
    cfg = CONFIGS[cfgname]
    if cfg.get("batch"):
        return run_batch(args, cfgname, steps, warmup, rank, world, cpu)
    if cfg.get("adjoint"):
        return run_adjoint(args, cfgname, steps, warmup, rank, world, cpu)
    return run_gpu(args, cfgname, steps, warmup, rank, world,
                   variants=VARIANTS.get(cfgname, ()) if variants else (), cpu=cpu)


# ------------------------------------------------------------------ reference arm (host cores)
def _fit(xs, ys, deg):
    import numpy as np
    return np.polyfit(np.asarray(xs, float), np.asarray(ys, float), deg)


def ref_extrapolated(cfgname, runs):
    """Single-instance time of the full workload from the oracle runs at the fit sizes:
    t_asm = a nt + b, CG iterations = c n + d, time per iteration = e nnz + f, with nnz(n) the
    exact cubic through the four sizes and nt(n) = 6 n^3."""
    import numpy as np
    cfg = CONFIGS[cfgname]
    N = cfg["mesh"][1]
    sizes = sorted({r["size"][1] for r in runs})
    med = {}
    for n in sizes:
        rs = [r for r in runs if r["size"][1] == n]
        med[n] = dict(nt=rs[0]["nt"], nnz=rs[0]["nnz"], ndof=rs[0]["ndof"],
                      t_asm=statistics.median(r["t_asm"] for r in rs),
                      t_it=statistics.median(r["t_cg"] / max(1, r["its"]) for r in rs),
                      its=statistics.median(r["its"] for r in rs))
    ca = _fit([med[n]["nt"] for n in sizes], [med[n]["t_asm"] for n in sizes], 1)
    ci = _fit(sizes, [med[n]["its"] for n in sizes], 1)
    ct = _fit([med[n]["nnz"] for n in sizes], [med[n]["t_it"] for n in sizes], 1)
    cz = _fit(sizes, [med[n]["nnz"] for n in sizes], 3)
    nt = 6 * N ** 3
    nnz = float(np.polyval(cz, N))
    its = float(np.polyval(ci, N))
    t = float(np.polyval(ca, nt)) + its * float(np.polyval(ct, nnz))
    fit = {"sizes": sizes, "nnz_full": round(nnz), "cg_iterations_full": its,
           "t_assemble_full_s": float(np.polyval(ca, nt)), "t_per_iteration_full_s": float(np.polyval(ct, nnz)),
           "t_instance_full_s": t,
           "per_size": {str(n): {k: v for k, v in med[n].items()} for n in sizes}}
    return t, fit


def ref_step(cfgname, pool, procs):
    """One step of the reference arm: procs concurrent single-threaded oracle instances.
    Returns (DOFs/s for the full workload, wall seconds, description)."""
    import numpy as np
    cfg = CONFIGS[cfgname]
    t0 = time.perf_counter()
    if cfgname in REF_FIT:
        sizes = REF_FIT[cfgname]
        kind = cfg["mesh"][0]
        jobs = [(cfgname, (kind, sizes[k % len(sizes)]), False) for k in range(max(procs, len(sizes)))]
        runs = pool.map(_oracle_run, jobs)
        wall = time.perf_counter() - t0
        t_inst, fit = ref_extrapolated(cfgname, runs)
        ndof = {"elasticity_p2_cube64": 3 * (2 * cfg["mesh"][1] + 1) ** 3,
                "diffusion_p1_cube160": (cfg["mesh"][1] + 1) ** 3}[cfgname]
        value = procs * ndof / t_inst
        desc = (f"extrapolated: {procs} concurrent single-threaded oracle instances at "
                f"{kind}({', '.join(map(str, sizes))}) per step, fitted (assembly linear in elements, "
                f"iterations linear in n, time per iteration linear in nnz, nnz exact cubic) and "
                f"evaluated at {kind}({cfg['mesh'][1]}); value = {procs} instances x {ndof} DOFs / "
                f"{t_inst:.1f} s")
        return value, wall, desc, fit
    if cfg.get("batch"):
        nprob = cfg["nprob"]
        chunks = [list(range(k, nprob, procs)) for k in range(procs)]
        runs = pool.map(_oracle_batch_run, [(cfgname, c) for c in chunks])
        wall = time.perf_counter() - t0
        nd = sum(r["ndof"] for r in runs)
        return nd / wall, wall, f"all {nprob} problems over {procs} concurrent single-threaded oracle instances", None
    runs = pool.map(_oracle_run, [(cfgname, cfg["mesh"], False)] * procs)
    wall = time.perf_counter() - t0
    nd = sum(r["ndof"] for r in runs)
    what = "gradient (forward + transpose CG + sensitivities)" if cfg.get("adjoint") else "assemble+rhs+CG"
    return nd / wall, wall, (f"full size: {procs} concurrent single-threaded oracle instances, "
                             f"{what}, {runs[0]['its']} CG iterations"), None


def run_reference(args):
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import ffo
    ffo.build()
    procs = os.cpu_count() or 1
    with mp.get_context("spawn").Pool(procs) as pool:
        vals = []
        for _ in range(args.warmup + args.steps):
            vals.append(ref_step(args.config, pool, procs))
        timed = vals[args.warmup:]
        value = statistics.median(v[0] for v in timed)
        out = {
            "metric": METRIC, "impl": "reference", "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.median(v[1] for v in timed) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.config, "same_config": True,
                       "extrapolated": args.config in REF_FIT},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": "port",
                             "sample": timed[-1][2]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if timed[-1][3]:
            out["config"]["fit"] = timed[-1][3]
        if args.config == DEFAULT and not args.single:
            wl = {}
            for name in SUB_ORDER:
                v, wall, desc, fit = ref_step(name, pool, procs)
                wl[name] = {"value": v, "unit": UNIT, "wall_s": wall, "cores": procs, "kind": "port",
                            "sample": desc, "extrapolated": name in REF_FIT}
                if fit:
                    wl[name]["fit"] = fit
            out["workloads"] = wl
    print(json.dumps(out))


# ------------------------------------------------------------------ main
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default=DEFAULT, choices=sorted(CONFIGS))
    ap.add_argument("--single", action="store_true",
                    help="measure only --config (no other workloads in the line)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--profile-case", choices=["elasticity", "diffusion3d", "poisson2d"], default=None,
                    help="run a small case for ncu instead of the benchmark")
    ap.add_argument("--n", type=int, default=32)
    ap.add_argument("--iters", type=int, default=40)
    ap.add_argument("--spmv-mode", type=int, default=0,
                    help="profile case: 0 FP64 CG, 1 double-float SpMV CG, 2 FP32-inner refinement")
    ap.add_argument("--solver", default="CG", choices=["CG", "GMRES"], help="profile case: Krylov solver")
    ap.add_argument("--dim-krylov", type=int, default=1000, help="profile case: GMRES restart length")
    args = ap.parse_args()
    if args.profile_case:
        profile_case(args.profile_case, args.n, args.iters, args.spmv_mode, args.solver, args.dim_krylov)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return
    from ffgpu.build import build
    build()
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    cpu = not args.no_cpu_baseline
    out = run_config(args, args.config, args.steps, args.warmup, rank, world,
                     variants=not args.no_variants, cpu=cpu)
    if args.config == DEFAULT and not args.single:
        # the other workloads: fewer timed steps (each well under a minute), W = 3
        sub_steps = {"poisson_p1_square256": 10, "diffusion_p1_cube160": 5,
                     "inverse_diffusion_p1_square512": 3, "batched_p1_1024": 5}
        wl = {}
        for name in SUB_ORDER:
            r = run_config(args, name, min(args.steps, sub_steps[name]) if args.steps >= 3 else args.steps,
                           3, rank, world, variants=not args.no_variants, cpu=cpu)
            if rank == 0:
                for k in ("metric", "higher_is_better", "scaling", "vs_baseline", "data", "n_gpus"):
                    r.pop(k, None)
                wl[name] = r
        if rank == 0:
            out["workloads"] = wl
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
