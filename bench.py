"""Benchmark of the explicit DG residual-and-update path on GB300.

Workload (one "step" = one SSP-RK3 step = 3 RHS stages over the whole mesh):
  Euler isentropic vortex, periodic [-5,5]^2, 512x512 quads split into 524,288 triangles,
  Dubiner basis p=3 (10 modes x 4 variables = 20,971,520 DOF), gamma=1.4, free stream
  rho=1 u=0.5 v=0 p=1, vortex strength 5 centred at a seeded point of [-2,2]^2,
  CFL 0.05 under dgfem's convective CFL definition (0.1, the figure the workload is named
  with, is unstable for p=3 under that definition; see CFL below).

metric: DOF * RK-stages / s.  `value` is the mixed-precision path with the state resident
in HBM; the FP64 path, the mixed-vs-FP64 speed-up and the L2/Linf error of the mixed
path against the FP64 path after 500 steps are reported beside it.  `e2e` times the
host-pointer C-ABI call (dgx_rk3_step_host) with the state copied in and out each step.
stdout carries one compact JSON line; the other workloads (Navier-Stokes, batched
ensemble, adjoint, quadrilaterals, plain-form 16x16x2, set-up times, forms) go to the
file named by --details.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

With --impl reference the CPU oracle (FP64 restatement of dgfem's path) is timed on all
host cores on a bounded sample of the same workload.  Under torchrun each rank runs an
independent replica (the path is replicated, not sharded, on one-GPU runs).
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "discontinuous-galerkin-fem_gb300"))

N_CELLS, ORDER, BASIS = 512, 3, "dubiner"
# CFL 0.1 under dgfem's CFL definition (dt * max(|u|+c) / shortest edge,
# compressible_solver_base.cpp:114-170) is unstable for p=3: the oracle restatement of
# dgfem's scheme diverges within 50 steps.  The workload runs at 0.05.
GAMMA, CFL, ACC_STEPS = 1.4, 0.05, 500
REF_BUDGET_S = 90.0  # timed CPU work of the reference arm
# per element per RK stage, p=3, FP64 state: 3*Np*V*8 + 92 bytes of geometry/connectivity
ALGO_BYTES_PER_ELEM_STAGE = 1052
MEASURED_PEAKS = ROOT / "MEASURED_PEAKS.json"
# FMA rates of this machine's GB300, measured by a probe of independent FMA chains (1216 x 256 threads):
# the denominators of the flop rooflines of the FP64 path (FP64 pipe) and of the Navier-Stokes leg
MEASURED_FP64_TFLOPS, MEASURED_FP32_TFLOPS = 1.19, 72.6


def flops_per_element_stage(p, viscous):
    """Algorithmic flops of one element's RK stage (triangles, V = 4):
    Euler: 2 Nq Np V (interpolation) + 30 Nq (flux) + 4 Nq Np V (x and y projection)
           + 1.5 Nfq (8 Np V + 100) (traces, Rusanov and lift on both sides of 1.5 faces)
           + 2 Np^2 V (M^-1) + 3 Np V (RK);
    Navier-Stokes adds 4 Nq Np V (gradient interpolation) + 60 Nq (viscous flux) + 4 Nq Np V (its
           projection) + 1.5 (8 Nfq Np V) (two-sided gradient interpolation at the face points)
           + 1.5 Nfq 20 (penalty).
    p=3 Euler: 6680; p=4 Navier-Stokes: 24960."""
    nq = {1: 3, 2: 6, 3: 12, 4: 16}[p]
    np_, nfq, v = (p + 1) * (p + 2) // 2, p + 1, 4
    f = 2 * nq * np_ * v + 30 * nq + 4 * nq * np_ * v + 1.5 * nfq * (8 * np_ * v + 100) + 2 * np_ * np_ * v + 3 * np_ * v
    if viscous:
        f += 4 * nq * np_ * v + 60 * nq + 4 * nq * np_ * v + 1.5 * 8 * nfq * np_ * v + 1.5 * nfq * 20
    return int(f)


def flop_roofline(p, viscous, elements, ms_per_step, peak_tflops, pipe):
    if not ms_per_step:
        return None
    fl = flops_per_element_stage(p, viscous)
    achieved = fl * elements * 3 / (ms_per_step * 1e-3) / 1e12
    return {"bound": pipe, "flops_per_element_stage": fl, "achieved_tflops": achieved, "peak_tflops": peak_tflops,
            "frac": achieved / peak_tflops, "peak_kind": "measured (FMA-chain probe)"}
FALLBACK_HBM_GBS = 6800.0
# The two CUDA-core forms of the mixed stage (the autotuner picks one), p=3:
#  design: bytes per element the form needs, averaged over the three stages;
#  traffic: dram__bytes_read.sum + dram__bytes_write.sum per element of one stage-2 launch,
#           from an ncu capture of that form on the 512x512x2 p=3 workload.
STAGE_FORMS = {
    # stage 1: 400 B, stage 2: 560 B, stage 3: 880 B (FP32 stage state, the double-float state's
    # low parts read and written in stage 3)
    "rows": {"kernel": "dgx::stage_kernel<3, Euler, no boundary> (mixed SSP-RK3 stage, neighbour rows)",
             "design": 613, "traffic": 518,
             "note": "ncu dram read+write of one stage-2 launch (518 B/element, its design bytes are 560)"},
    # FP32 state rows, increments, the double-float state's low parts (stage 3), geometry and
    # connectivity, and the face traces: 192 B written and 192 B read per element; stages 1/2/3
    # 784/944/1264 B (a middle step of a call)
    "traces": {"kernel": "dgx::stage_trace_kernel<3, no boundary> (mixed SSP-RK3 stage, face traces)",
               "design": 997, "traffic": 927,
               "note": "ncu dram read+write of the three stage launches of a middle step, averaged "
                       "(705, 880, 1196 B/element; design 784, 944, 1264)"},
    # the same bytes at 64- and 32-element tiles, one CTA per tile
    "traces, 64-element tiles": {"kernel": "dgx::stage_trace_kernel<3, no boundary, 64-element tiles>",
                                 "design": 997, "traffic": None, "note": "not captured with DRAM counters"},
    "traces, 32-element tiles": {"kernel": "dgx::stage_trace_kernel<3, no boundary, 32-element tiles>",
                                 "design": 997, "traffic": 928,
                                 "note": "ncu dram read+write of the three stage launches of a middle step, "
                                         "averaged (704, 880, 1200 B/element; design 784, 944, 1264)"},
    # each thread copies its neighbours' trace blocks into shared memory (cp.async) while staging
    "traces, 32-element tiles, neighbour blocks in shared memory": {
        "kernel": "dgx::stage_trace_kernel<3, no boundary, 32-element tiles, neighbour blocks in shared memory>",
        "design": 997, "traffic": 919,
        "note": "ncu dram read+write of the three stage launches of a middle step, averaged "
                "(696, 873, 1189 B/element; design 784, 944, 1264)"},
    # the same bytes; each CTA bulk-copies its next tile's inputs while it computes a tile
    "traces pipelined": {"kernel": "dgx::stage_trace_pipe_kernel<3, no ghost blocks> (mixed SSP-RK3 stage, face "
                                   "traces, next tile copied while a tile is computed)",
                         "design": 997, "traffic": None,
                         "note": "not captured with DRAM counters"},
}


def vortex(xy, t=0.0, beta=5.0, xc=0.0, yc=0.0, uinf=0.5, vinf=0.0, gamma=GAMMA, period=10.0):
    """Shu's isentropic vortex on rho=1, p=1, advected with (uinf, vinf), conserved vars."""
    x = xy[..., 0] - (xc + uinf * t)
    y = xy[..., 1] - (yc + vinf * t)
    x = (x + period / 2) % period - period / 2
    y = (y + period / 2) % period - period / 2
    g = beta / (2.0 * np.pi) * np.exp(0.5 * (1.0 - (x * x + y * y)))
    u, v = uinf - y * g, vinf + x * g
    T = 1.0 - (gamma - 1.0) / (2.0 * gamma) * g * g
    rho = T ** (1.0 / (gamma - 1.0))
    p = rho * T
    return np.stack([rho, rho * u, rho * v, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)], -1)


def vortex_device(xy, t=0.0, beta=5.0, xc=0.0, yc=0.0, uinf=0.5, vinf=0.0, gamma=GAMMA, period=10.0):
    """vortex() on a CUDA tensor of points (the initial condition evaluated on the GPU)."""
    import torch
    x = xy[..., 0] - (xc + uinf * t)
    y = xy[..., 1] - (yc + vinf * t)
    x = torch.remainder(x + period / 2, period) - period / 2
    y = torch.remainder(y + period / 2, period) - period / 2
    g = beta / (2.0 * np.pi) * torch.exp(0.5 * (1.0 - (x * x + y * y)))
    u, v = uinf - y * g, vinf + x * g
    T = 1.0 - (gamma - 1.0) / (2.0 * gamma) * g * g
    rho = T ** (1.0 / (gamma - 1.0))
    p = rho * T
    return torch.stack([rho, rho * u, rho * v, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)], -1)


def taylor_green(xy, seed=0, gamma=GAMMA, mach=0.1, noise=1e-3):
    """Decaying Taylor-Green-type vortex on [0, 2 pi]^2 (conserved variables): rho=1,
    u=sin x cos y, v=-cos x sin y, p = 1/(gamma M^2) + (cos 2x + cos 2y)/4, plus seeded
    Gaussian noise of amplitude `noise` on the velocity."""
    x, y = xy[..., 0], xy[..., 1]
    rng = np.random.default_rng(seed)
    u = np.sin(x) * np.cos(y) + noise * rng.standard_normal(x.shape)
    v = -np.cos(x) * np.sin(y) + noise * rng.standard_normal(x.shape)
    p = 1.0 / (gamma * mach * mach) + 0.25 * (np.cos(2 * x) + np.cos(2 * y))
    rho = np.ones_like(x)
    return np.stack([rho, rho * u, rho * v, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)], -1)


def shear_layer(xy, seed=0, gamma=GAMMA, mach=0.3, noise=1e-4):
    """Double shear layer on the periodic unit square (conserved variables): rho=1,
    p = 1/(gamma M^2), u = tanh((|y - 1/2| - 1/4)/0.02), v = 0.05 sin(2 pi x), plus seeded
    Gaussian noise of amplitude `noise` on both velocity components."""
    x, y = xy[..., 0], xy[..., 1]
    rng = np.random.default_rng(seed + 1)
    u = np.tanh((np.abs(y - 0.5) - 0.25) / 0.02) + noise * rng.standard_normal(x.shape)
    v = 0.05 * np.sin(2 * np.pi * x) + noise * rng.standard_normal(x.shape)
    rho = np.ones_like(x)
    p = np.full_like(x, 1.0 / (gamma * mach * mach))
    return np.stack([rho, rho * u, rho * v, p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v)], -1)


def vortex_centre(seed=0):
    return np.random.default_rng(seed).uniform(-2.0, 2.0, size=2)


def dist_init():
    """One process per GPU under torchrun (NCCL); gloo on a host without GPUs (CPU tests).
    Replicas only: the ranks share nothing but the barrier and the max of their times."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
            dist.init_process_group("nccl")
        else:
            dist.init_process_group("gloo")
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, ws):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.dev = device_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, val in zip(names, f[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def hbm_peak():
    try:
        return float(json.loads(MEASURED_PEAKS.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class OracleWorkload:
    """The CPU oracle on the full 512x512x2 p=3 mesh (setup excluded from timing)."""

    def __init__(self, threads, seed):
        sys.path[:0] = [str(ROOT / "oracle"), str(ROOT / "tests")]
        import oracle as O
        from meshes import PERIODIC_PAIRS, periodic_rectangle
        self.O = O
        v, e, b = periodic_rectangle(N_CELLS)
        self.m = O.OracleMesh(v, e, b, order=ORDER, basis=O.DUBINER, periodic=PERIODIC_PAIRS)
        xc, yc = vortex_centre(seed)
        O.set_threads(threads)
        self.threads = threads
        self.u = self.m.project(vortex(self.m.quad_points(), xc=xc, yc=yc))
        self.ph = O.euler(GAMMA)
        self.dof = self.m.ne * self.m.np * 4
        # the GPU arm's step: CFL over dgfem's max CFL number of the initial state
        self.dt = CFL / self.m.max_cfl(GAMMA, self.u, 1.0)

    def run(self, steps):
        """Advance `steps` SSP-RK3 steps of size self.dt; returns (DOF*stages/s, seconds)."""
        t0 = time.perf_counter()
        self.u = self.m.rk3_step(self.ph, self.u, self.dt, steps)
        secs = time.perf_counter() - t0
        return self.dof * 3 * steps / secs, secs


def run_reference(args, rank, ws):
    """Reference arm: dgfem's path restated (oracle) on all host cores; rank 0 only."""
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    w = OracleWorkload(threads, args.seed)
    _, t_warm = w.run(max(1, args.warmup))
    # each timed step is one SSP-RK3 step of the full mesh; at most about REF_BUDGET_S seconds
    # of them are timed, so the arm ends within minutes whatever --steps asks for
    per_step = t_warm / max(1, args.warmup)
    k = max(1, min(args.steps, int(REF_BUDGET_S / max(per_step, 1e-9))))
    rate, secs = w.run(k)
    line = {"metric": "DOF*RK-stages/s", "value": rate, "unit": "DOF*stages/s", "n_gpus": ws,
            "steps": k, "warmup": max(1, args.warmup), "ms_per_step": 1e3 * secs / k, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": workload_config(N_CELLS, w.dof, w.dt, ws),
            "cpu_baseline": {"value": rate, "unit": "DOF*stages/s", "cores": threads, "kind": "port",
                             "sample": f"each step is one SSP-RK3 step of the full 512x512x2 p=3 mesh "
                                       f"({k} of the {args.steps} asked for timed, at most about "
                                       f"{REF_BUDGET_S:.0f} s of work); FP64 oracle restatement of dgfem's path, "
                                       f"OpenMP {threads} threads"},
            "e2e": {"value": rate, "unit": "DOF*stages/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config(cells, dof, dt, ws):
    """The `config` object of both arms' lines (same keys and values for the same workload)."""
    return {"workload": f"euler_vortex_{cells}x{cells}x2_p3_dubiner", "elements": 2 * cells * cells, "order": ORDER,
            "dof": dof, "dt": dt, "cfl": CFL,
            "l2": "inputs larger than L2 (168 MB FP64 state + stage buffers)", "parallelism": f"replicas x{ws}"}


def config1_leg(dg, torch):
    """The plain-form workload: periodic [-5,5]^2, 16x16x2 = 512 triangles, Dubiner p=2,
    beta = 5 vortex at the origin on the free stream (1, 0.5, 0, 1), CFL 0.1 (dgfem's
    definition), 200 FP64 SSP-RK3 steps.  Reports the 512x6x4 state's norm and its relative
    L2 error (coefficients; the Dubiner basis is orthonormal, so this is the L2 norm of the
    field on this uniform mesh) against the exactly advected vortex."""
    mesh = dg.DGMesh.rectangle(16, 16, -5.0, 5.0, -5.0, 5.0, periodic=True)
    ctx = dg.DGContext(mesh, dg.DGSpace("triangle", 2, BASIS), dg.EulerWeakFormulation(GAMMA), "fp64")
    xq = ctx.quad_points()
    u = ctx.project(torch.tensor(vortex(xq), device="cuda"))
    dt = 0.1 / ctx.max_cfl(u, 1.0)
    ctx.rk3_step(u.clone(), dt, 3)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    ctx.rk3_step(u, dt, 200)
    e1.record()
    torch.cuda.synchronize()
    exact = ctx.project(torch.tensor(vortex(xq, t=200 * dt), device="cuda"))
    return {"workload": "euler_vortex_16x16x2_p2_dubiner_fp64_cfl0.1", "elements": ctx.n_elements,
            "state_shape": list(u.shape), "dt": dt, "steps": 200, "ms_per_step": e0.elapsed_time(e1) / 200,
            "state_l2_norm": float(torch.linalg.vector_norm(u)),
            "l2_rel_err_vs_exact": float(torch.linalg.vector_norm(u - exact) / torch.linalg.vector_norm(exact))}


def batch_leg(dg, torch, n_inst, steps, seed):
    """Independent periodic vortex solves on [-5,5]^2: N x N x 2 with N uniform in
    {16, 24, ..., 128}, p uniform in {2, 3}, beta ~ U(1,5), free stream u ~ U(0.2,0.8),
    centre ~ U([-2,2]^2); each instance's dt = CFL / its max CFL number.  Times `steps`
    mixed-precision steps of all instances through one DGBatch (one persistent launch per
    stage) against the same steps through one mixed DGContext per instance in a loop, and
    reports each instance's error against its own FP64 run."""
    rng = np.random.default_rng(seed + 4242)
    Ns = rng.choice(np.arange(16, 129, 8), size=n_inst)
    ps = rng.choice([2, 3], size=n_inst)
    betas = rng.uniform(1.0, 5.0, n_inst)
    uinfs = rng.uniform(0.2, 0.8, n_inst)
    centres = rng.uniform(-2.0, 2.0, (n_inst, 2))
    wf = dg.EulerWeakFormulation(GAMMA)
    meshes = [dg.DGMesh.rectangle(int(N), int(N), -5.0, 5.0, -5.0, 5.0, periodic=True) for N in Ns]
    spaces = [dg.DGSpace("triangle", int(p), BASIS) for p in ps]
    u0s, dts, refs, dofs = [], [], [], []
    t0 = time.perf_counter()
    for i in range(n_inst):  # initial states and each instance's FP64 run
        c = dg.DGContext(meshes[i], spaces[i], wf, "fp64")
        xq = c.quad_points()
        u0 = c.project(torch.tensor(vortex(xq, beta=betas[i], xc=centres[i, 0], yc=centres[i, 1], uinf=uinfs[i]),
                                    device="cuda"))
        dt = CFL / c.max_cfl(u0, 1.0)
        u = u0.clone()
        c.rk3_step(u, dt, steps)
        u0s.append(u0)
        dts.append(dt)
        refs.append(u)
        dofs.append(c.n_elements * c.n_basis * 4)
        del c
    torch.cuda.synchronize()
    t_ref = time.perf_counter() - t0
    total = int(sum(dofs)) * 3 * steps  # DOF * stages of the whole ensemble

    batch = dg.DGBatch(meshes, spaces, wf)
    for i in range(n_inst):
        batch.state(i).copy_(u0s[i])
    batch.rk3_step(dts, 2)  # warm-up: launch-shape tuning and graph capture
    for i in range(n_inst):
        batch.state(i).copy_(u0s[i])
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    batch.rk3_step(dts, steps)
    e1.record()
    torch.cuda.synchronize()
    t_batch = e0.elapsed_time(e1) / 1e3
    outs = [batch.state(i) for i in range(n_inst)]
    l2 = [float(torch.linalg.vector_norm(outs[i] - refs[i]) / torch.linalg.vector_norm(refs[i])) for i in range(n_inst)]
    linf = [float((outs[i] - refs[i]).abs().max() / refs[i].abs().max()) for i in range(n_inst)]
    grid, tiles = batch.launch_shape()
    form = batch.stage_form()
    n_orders = len(set(ps.tolist()))

    ctxs = [dg.DGContext(meshes[i], spaces[i], wf, "mixed") for i in range(n_inst)]
    us = [u0s[i].clone() for i in range(n_inst)]
    for i in range(n_inst):  # warm-up per context, then back to the initial state
        ctxs[i].rk3_step(us[i], dts[i], 2)
        us[i].copy_(u0s[i])
    torch.cuda.synchronize()
    e0.record()
    for i in range(n_inst):
        ctxs[i].rk3_step(us[i], dts[i], steps)
    e1.record()
    torch.cuda.synchronize()
    t_loop = e0.elapsed_time(e1) / 1e3
    same = max(float(torch.linalg.vector_norm(us[i] - outs[i]) / torch.linalg.vector_norm(us[i]))
               for i in range(n_inst))
    del ctxs, us, batch
    torch.cuda.empty_cache()
    return {"workload": f"euler_vortex_ensemble_{n_inst}_instances_N16-128_p2-3_dubiner_mixed",
            "instances": n_inst, "steps": steps, "elements": int(sum(2 * int(N) * int(N) for N in Ns)),
            "orders": {"p2": int((ps == 2).sum()), "p3": int((ps == 3).sum())}, "dof": int(sum(dofs)),
            "value": total / t_batch, "unit": "DOF*stages/s", "s": t_batch,
            "single_solve_loop": {"value": total / t_loop, "s": t_loop},
            "batched_vs_loop": t_loop / t_batch,
            "launch_shape": {"grid": grid, "tiles": tiles}, "stage_form": form,
            # per call: one FP32 conversion per order (and, for the face-trace form, the traces of
            # the start state per order); per stage: one launch, or one per order
            "gpu_launches": (3 * steps * n_orders + 2 * n_orders if form == "traces per order"
                             else 3 * steps + n_orders),
            "batched_vs_loop_max_rel_diff": same,
            "per_instance_vs_fp64": {"l2_rel_max": max(l2), "l2_rel_median": float(np.median(l2)),
                                     "linf_rel_max": max(linf)},
            "fp64_reference_runs_s": t_ref}


def quad_leg(dg, torch, cells, steps, order=3):
    """Bilinear quadrilaterals (DGSpace("quad", order), Legendre basis): the vortex on a periodic
    cells x cells mesh whose interior vertices are moved by up to 20 % of the cell size
    (non-affine elements), FP64, mixed and double-float forms of the quad element kernel,
    each 3 launches per SSP-RK3 step, and their distance from FP64 after `steps` steps."""
    n1 = cells + 1
    xs = np.linspace(-5.0, 5.0, n1)
    X, Y = np.meshgrid(xs, xs)
    V = np.stack([X.ravel(), Y.ravel()], axis=1)
    rng = np.random.default_rng(7)
    inner = (np.abs(np.abs(V[:, 0]) - 5.0) > 1e-12) & (np.abs(np.abs(V[:, 1]) - 5.0) > 1e-12)
    V[inner] += 0.2 * (10.0 / cells) * rng.uniform(-1, 1, (int(inner.sum()), 2))
    vid = lambda i, j: j * n1 + i  # noqa: E731
    E = np.array([(vid(i, j), vid(i + 1, j), vid(i + 1, j + 1), vid(i, j + 1))
                  for j in range(cells) for i in range(cells)], dtype=np.int32)
    edges = {2: [(vid(i, 0), vid(i + 1, 0)) for i in range(cells)],
             3: [(vid(cells, j), vid(cells, j + 1)) for j in range(cells)],
             4: [(vid(i, cells), vid(i + 1, cells)) for i in range(cells)],
             5: [(vid(0, j), vid(0, j + 1)) for j in range(cells)]}
    mesh = dg.DGMesh(V, E, None, {"Bottom": 2, "Right": 3, "Top": 4, "Left": 5}, edges)
    mesh.set_periodic_boundaries("Left", "Right")
    mesh.set_periodic_boundaries("Bottom", "Top")
    space = dg.DGSpace("quad", order)
    wf = dg.EulerWeakFormulation(GAMMA)
    ctxs = {k: dg.DGContext(mesh, space, wf, k) for k in ("fp64", "mixed", "df64")}
    c64 = ctxs["fp64"]
    u0 = c64.project(torch.tensor(vortex(c64.quad_points()), device="cuda"))
    dt = 0.05 / c64.max_cfl(u0, 1.0)
    dof = c64.n_elements * c64.n_basis * 4
    out = {"workload": f"euler_vortex_quads_{cells}x{cells}_distorted_p{order}_legendre",
           "elements": c64.n_elements, "dof": dof, "steps": steps, "dt": dt}
    ref = None
    for name, ctx in ctxs.items():
        u = u0.clone()
        ctx.rk3_step(u, dt, 2)  # warm-up (graph capture)
        u = u0.clone()
        torch.cuda.synchronize()
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        ctx.rk3_step(u, dt, steps)
        e1.record(s)
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / 1e3
        if ref is None:
            ref = u
        out[name] = {"ms_per_step": 1e3 * t / steps, "value": dof * 3 * steps / t,
                     "vs_fp64_l2_rel": float(torch.linalg.vector_norm(u - ref) / torch.linalg.vector_norm(ref))}
    out["mixed_vs_fp64"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    out["df64_vs_fp64"] = out["fp64"]["ms_per_step"] / out["df64"]["ms_per_step"]
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="dgx", choices=["dgx", "reference"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--acc-steps", type=int, default=ACC_STEPS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--cells", type=int, default=N_CELLS, help="quads per side (profiling cases)")
    ap.add_argument("--ns-steps", type=int, default=1000, help="steps of the Navier-Stokes leg (0: skip)")
    ap.add_argument("--adj-steps", type=int, default=1000, help="steps of the adjoint leg (0: skip)")
    ap.add_argument("--adj-dirs", type=int, default=16, help="finite-difference directions of the adjoint check")
    ap.add_argument("--adj-snapshots", type=int, default=20, help="snapshots of the binomial-checkpointing gradient")
    ap.add_argument("--batch-instances", type=int, default=256, help="instances of the batched leg (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=300, help="SSP-RK3 steps of each batched instance")
    ap.add_argument("--quad-cells", type=int, default=256, help="quadrilaterals per side of the quad leg (0: skip)")
    ap.add_argument("--quad-steps", type=int, default=50, help="SSP-RK3 steps of the quad leg")
    ap.add_argument("--details", default="bench_details.json",
                    help="file for the full results of every leg (stdout carries the compact line)")
    args = ap.parse_args()
    rank, ws = dist_init()
    if args.impl == "reference":
        run_reference(args, rank, ws)
        if ws > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
        return

    import torch
    import dgfem_gb300 as dg

    dev = torch.cuda.current_device()
    # set-up cost (host connectivity O(E log E), geometry, device upload, L2 projection on the GPU)
    torch.cuda.synchronize()
    t_setup = time.perf_counter()
    mesh = dg.DGMesh.rectangle(args.cells, args.cells, -5.0, 5.0, -5.0, 5.0, periodic=True)
    t_mesh = time.perf_counter() - t_setup
    space = dg.DGSpace("triangle", ORDER, BASIS)
    wf = dg.EulerWeakFormulation(GAMMA)
    t0 = time.perf_counter()
    c64 = dg.DGContext(mesh, space, wf, "fp64")
    t_ctx = time.perf_counter() - t0
    cmx = dg.DGContext(mesh, space, wf, "mixed")
    ne, nb = c64.n_elements, c64.n_basis
    dof = ne * nb * 4
    xc, yc = vortex_centre(args.seed)
    # torch loads its elementwise kernels on first use (seconds, once per process): load them
    # on a few points first, so that the timing below is the evaluation itself
    vortex_device(torch.zeros((4, 2), dtype=torch.float64, device="cuda"), xc=xc, yc=yc)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    xq_dev = c64.quad_points_device()
    uq = vortex_device(xq_dev, xc=xc, yc=yc)
    torch.cuda.synchronize()
    t_ic = time.perf_counter() - t0
    t0 = time.perf_counter()
    u0 = c64.project(uq)
    torch.cuda.synchronize()
    t_proj = time.perf_counter() - t0
    del uq
    setup = {"elements": ne, "mesh_and_periodic_pairing_s": t_mesh, "context_fp64_s": t_ctx,
             "initial_condition_on_gpu_s": t_ic, "l2_projection_gpu_s": t_proj}
    dt = CFL / c64.max_cfl(u0, 1.0)

    # ---- accuracy at t_final: mixed vs FP64 (the FP64 path matches the oracle to 1e-12 per RHS)
    acc = {}
    if args.acc_steps > 0:
        u64 = u0.clone()
        umx = u0.clone()
        c64.rk3_step(u64, dt, args.acc_steps)
        cmx.rk3_step(umx, dt, args.acc_steps)
        torch.cuda.synchronize()
        exact = c64.project(vortex_device(xq_dev, t=dt * args.acc_steps, xc=xc, yc=yc))
        d = (umx - u64)
        acc = {"steps": args.acc_steps, "t_final": dt * args.acc_steps,
               "mixed_vs_fp64_l2_rel": float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(u64)),
               "mixed_vs_fp64_linf_rel": float(d.abs().max() / u64.abs().max()),
               "fp64_vs_exact_l2_rel": float(torch.linalg.vector_norm(u64 - exact) / torch.linalg.vector_norm(exact)),
               "mixed_vs_exact_l2_rel": float(torch.linalg.vector_norm(umx - exact) / torch.linalg.vector_norm(exact))}
        del u64, umx, exact

    def timed(ctx, k, warm):
        u = u0.clone()
        ctx.rk3_step(u, dt, warm)
        torch.cuda.synchronize()
        barrier(ws)
        torch.cuda.synchronize()
        s = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        ctx.rk3_step(u, dt, k)
        e1.record(s)
        torch.cuda.synchronize()
        barrier(ws)
        return e0.elapsed_time(e1) / 1e3

    with ClockSampler(dev) as clk:
        t_mx = timed(cmx, args.steps, args.warmup)
    clocks = clk.summary()
    t_mx = allreduce_max(t_mx, ws)
    grid, tiles, on_tc = cmx.launch_shape()
    form = cmx.stage_form()
    tile = cmx.stage_tile()
    if form == "traces" and tile != 128:
        form += f", {tile}-element tiles" + (", neighbour blocks in shared memory" if cmx.stage_nbr_shared() else "")
    # the tensor-core (3xTF32 tcgen05) form of the same stage, forced, timed the same way
    os.environ["DGX_STAGE_KERNEL"] = "tc"
    ctc = dg.DGContext(mesh, space, wf, "mixed")
    t_tc = allreduce_max(timed(ctc, args.steps, args.warmup), ws)
    del os.environ["DGX_STAGE_KERNEL"]
    tc_acc = None
    if args.acc_steps > 0:
        u64 = u0.clone()
        utc = u0.clone()
        c64.rk3_step(u64, dt, args.acc_steps)
        ctc.rk3_step(utc, dt, args.acc_steps)
        torch.cuda.synchronize()
        tc_acc = float(torch.linalg.vector_norm(utc - u64) / torch.linalg.vector_norm(u64))
        del u64, utc
    tensor_core = {"kernel": "dgx::stage_tc_kernel<3, no boundary> (3xTF32 tcgen05, TMEM accumulators)",
                   "ms_per_step": 1e3 * t_tc / args.steps, "value": dof * 3 * args.steps * ws / t_tc,
                   "vs_cuda_core_stage": t_tc / t_mx, "mixed_vs_fp64_l2_rel": tc_acc}
    del ctc
    k64 = max(1, min(args.steps, 50))
    t_64 = allreduce_max(timed(c64, k64, min(args.warmup, 3)), ws)
    # the double-float form of the FP64 path (same algorithm and FP64 state, residual in
    # pairs of FP32 numbers on the FP32 pipe), and its distance from FP64 after acc_steps
    cdf = dg.DGContext(mesh, space, wf, "df64")
    t_df = allreduce_max(timed(cdf, k64, min(args.warmup, 3)), ws)
    df_acc = None
    if args.acc_steps > 0:
        u64 = u0.clone()
        udf = u0.clone()
        c64.rk3_step(u64, dt, args.acc_steps)
        cdf.rk3_step(udf, dt, args.acc_steps)
        torch.cuda.synchronize()
        df_acc = float(torch.linalg.vector_norm(udf - u64) / torch.linalg.vector_norm(u64))
        del u64, udf
    df64 = {"kernel": "dgx::element_kernel<3, f2> (double-float arithmetic, FP64 state)",
            "value": dof * 3 * k64 * ws / t_df, "ms_per_step": 1e3 * t_df / k64, "steps": k64,
            "vs_fp64": t_64 / t_df, "vs_fp64_l2_rel_after_acc_steps": df_acc}
    del cdf
    v_mx = dof * 3 * args.steps * ws / t_mx
    v_64 = dof * 3 * k64 * ws / t_64

    # ---- end to end through the host-pointer C-ABI call, pinned host state
    host = u0.cpu().pin_memory()
    hnp = host.numpy()
    cmx.rk3_step(hnp, dt, 1)  # warm the host path (allocations, graph)
    ke = max(1, min(args.steps, 50))
    torch.cuda.synchronize()
    barrier(ws)
    t0 = time.perf_counter()
    lib = dg.load()
    import ctypes as C
    ptr = hnp.ctypes.data_as(C.POINTER(C.c_double))
    for _ in range(ke):
        dg._lib.check(lib.dgx_rk3_step_host(cmx._h, ptr, float(dt), 1))
    t_e2e = allreduce_max(time.perf_counter() - t0, ws)
    v_e2e = dof * 3 * ke * ws / t_e2e

    peak, peak_kind = hbm_peak()
    t_launch = t_mx / (3 * args.steps)
    achieved = ALGO_BYTES_PER_ELEM_STAGE * ne / t_launch / 1e9
    sf = STAGE_FORMS.get(form, STAGE_FORMS["rows"])
    roof = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": peak_kind,
            "traffic": sf["traffic"] * ne if sf["traffic"] else None,
            "kernel": sf["kernel"],
            "algorithmic_bytes_per_launch": ALGO_BYTES_PER_ELEM_STAGE * ne, "launch_ms": t_launch * 1e3,
            "design_bytes_per_launch": sf["design"] * ne,
            "achieved_design_bytes": sf["design"] * ne / t_launch / 1e9,
            "traffic_note": sf["note"]}

    # ---- Navier-Stokes leg: Taylor-Green-type vortex, [0,2pi]^2, 256x256x2, p=4, Re=1600
    ns = None
    if args.ns_steps > 0:
        import math
        del c64, cmx, u0
        torch.cuda.empty_cache()
        nmesh = dg.DGMesh.rectangle(256, 256, 0.0, 2 * math.pi, 0.0, 2 * math.pi, periodic=True)
        nsp = dg.DGSpace("triangle", 4, "dubiner")
        nwf = dg.NavierStokesWeakFormulation(GAMMA, 1.0 / 1600.0, 0.71, 5.0)
        n64 = dg.DGContext(nmesh, nsp, nwf, "fp64")
        nmx = dg.DGContext(nmesh, nsp, nwf, "mixed")
        nu0 = n64.project(torch.tensor(taylor_green(n64.quad_points(), args.seed), device="cuda"))
        # combined CFL: dgfem defines only the convective one.  The oracle diverges within
        # 22 steps at convective CFL 0.05 and runs at 0.025; the viscous bound 0.05 h^2 rho / mu
        # (h the shortest edge) is far larger here.  Independently of dt, dgfem's half-jump
        # viscous face flux lets this flow grow without bound at fine resolution (see `note`)
        h = 2 * math.pi / 256
        ndt = min(0.025 / n64.max_cfl(nu0, 1.0), 0.05 * h * h * 1600.0)
        ndof = n64.n_elements * n64.n_basis * 4

        def ntimed(ctx, k, chunk=25, keep=100):
            """Up to k steps in chunks, event-timed on the device.  Timing stops at the first
            chunk after which the state is no longer finite (that chunk is not counted), so
            only steps on finite states are timed.  Returns (seconds, steps timed, first step
            count with a non-finite state or None, a copy of the state at step `keep`)."""
            u = nu0.clone()
            ctx.rk3_step(u.clone(), ndt, 2)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            secs, timed_steps, first_bad, kept = 0.0, 0, None, None
            for done in range(0, k, chunk):
                n = min(chunk, k - done)
                e0.record()
                ctx.rk3_step(u, ndt, n)
                e1.record()
                torch.cuda.synchronize()
                if not bool(torch.isfinite(u).all()):
                    first_bad = done + n
                    break
                secs += e0.elapsed_time(e1) / 1e3
                timed_steps += n
                if done + n == keep:
                    kept = u.clone()
            return secs, timed_steps, first_bad, kept

        tn_mx, kn_mx, bad_mx, umx = ntimed(nmx, args.ns_steps)
        tn_64, kn_64, bad_64, u64 = ntimed(n64, args.ns_steps)
        acc100 = None if (umx is None or u64 is None) else \
            float(torch.linalg.vector_norm(umx - u64) / torch.linalg.vector_norm(u64))
        ns = {"workload": "navier_stokes_taylor_green_256x256x2_p4_dubiner_re1600", "elements": n64.n_elements,
              "dof": ndof, "dt": ndt, "steps_asked": args.ns_steps,
              "mixed": {"value": ndof * 3 * kn_mx / tn_mx if kn_mx else None,
                        "ms_per_step": 1e3 * tn_mx / kn_mx if kn_mx else None, "steps_timed": kn_mx},
              "fp64": {"value": ndof * 3 * kn_64 / tn_64 if kn_64 else None,
                       "ms_per_step": 1e3 * tn_64 / kn_64 if kn_64 else None, "steps_timed": kn_64},
              "mixed_vs_fp64": (tn_64 / kn_64) / (tn_mx / kn_mx) if kn_mx and kn_64 else None,
              "mixed_vs_fp64_l2_rel_at_step_100": acc100,
              "flop_roofline": {
                  "mixed": flop_roofline(4, True, n64.n_elements, 1e3 * tn_mx / kn_mx if kn_mx else None,
                                         MEASURED_FP32_TFLOPS, "fp32"),
                  "fp64": flop_roofline(4, True, n64.n_elements, 1e3 * tn_64 / kn_64 if kn_64 else None,
                                        MEASURED_FP64_TFLOPS, "fp64")},
              "first_nonfinite_step": {"fp64": bad_64, "mixed": bad_mx},
              "note": "only steps on finite states are timed (timing stops at the first 25-step chunk after "
                      "which the state is not finite).  dgfem's viscous face flux (half jump) grows without "
                      "bound on this flow at fine resolution; the blow-up time does not depend on dt (oracle, "
                      "64x64x2: NaN at t=0.19 with CFL 0.025 and 0.0125)"}
        del n64, nmx

    # ---- adjoint leg: shear layer 128x128x2, p=3, J = kinetic energy after adj_steps steps,
    #      checkpoints every 50 steps, and again with binomial checkpointing (memory held and
    #      forward steps recomputed by each); adjoint/forward time ratio and FD / tangent-linear checks
    adj = None
    if args.adj_steps > 0:
        amesh = dg.DGMesh.rectangle(128, 128, 0.0, 1.0, 0.0, 1.0, periodic=True)
        actx = dg.DGContext(amesh, dg.DGSpace("triangle", 3, "dubiner"), dg.EulerWeakFormulation(GAMMA), "fp64")
        au0 = actx.project(torch.tensor(shear_layer(actx.quad_points(), args.seed), device="cuda"))
        adt = CFL / actx.max_cfl(au0, 1.0)
        na, ce = args.adj_steps, 50
        w = au0.clone()
        actx.rk3_step(w, adt, 3)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w = au0.clone()
        actx.rk3_step(w, adt, na)
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        actx.kinetic_energy_gradient(au0, adt, 2, 1)  # warm the adjoint kernels
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Jv, grad = actx.kinetic_energy_gradient(au0, adt, na, ce)
        torch.cuda.synchronize()
        t_grad = time.perf_counter() - t0
        # binomial checkpointing: adj_snapshots states instead of the uniform scheme's
        # (na / ce + 1) checkpoints and 3 ce + 1 segment states, at the price of recomputed steps
        nsnap = args.adj_snapshots
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Jb, gradb, bst = actx.kinetic_energy_gradient_binomial(au0, adt, na, nsnap)
        torch.cuda.synchronize()
        t_bin = time.perf_counter() - t0
        binomial = dict(bst, snapshots=nsnap, gradient_s=t_bin, gradient_vs_forward_solve=t_bin / t_fwd,
                        equals_uniform_bitwise=bool(Jb == Jv and torch.equal(gradb, grad)),
                        state_mb=bst["states_held"] * au0.numel() * 8 / 1e6)
        del gradb
        uniform_states = (na + ce - 1) // ce + 1 + 3 * min(ce, na) + 1
        rng = np.random.default_rng(1234)
        h = 1e-6
        fd_err, tlm_err, fd_abs, fd_cs = [], [], [], []
        axq = actx.quad_points()
        for k in range(args.adj_dirs):
            # seeded random smooth direction: a few random Fourier modes per variable,
            # projected into the DG space and scaled to the norm of u0, so that h is a step
            # relative to the state.  Wavenumbers start at 0: the layer varies along y only, so
            # modes with kx >= 1 alone are nearly orthogonal to dJ/du and their derivatives
            # drown in rounding
            field = np.zeros(axq.shape[:-1] + (4,))
            for var in range(4):
                for _ in range(3):
                    kx, ky = rng.integers(0, 4, size=2)
                    ph_x, ph_y = rng.uniform(0, 2 * np.pi, size=2)
                    field[..., var] += rng.standard_normal() * np.sin(2 * np.pi * kx * axq[..., 0] + ph_x) * \
                        np.cos(2 * np.pi * ky * axq[..., 1] + ph_y)
            d = actx.project(torch.tensor(field, device="cuda"))
            d *= torch.linalg.vector_norm(au0) / torch.linalg.vector_norm(d)
            up, um = au0 + h * d, au0 - h * d
            actx.rk3_step(up, adt, na)
            actx.rk3_step(um, adt, na)
            fd = (actx.kinetic_energy(up) - actx.kinetic_energy(um)) / (2 * h)
            ad = float(torch.sum(grad * d))
            fd_err.append(abs(ad - fd) / max(abs(fd), 1e-300))
            fd_abs.append(abs(fd))
            fd_cs.append(abs(ad - fd) / float(torch.linalg.vector_norm(grad) * torch.linalg.vector_norm(d)))
            if k < 2:
                ut, dut = au0.clone(), d.clone()
                actx.rk3_step_tlm(ut, dut, adt, na)
                _, gT = actx.kinetic_energy(ut, grad=True)
                tl = float(torch.sum(gT * dut))
                tlm_err.append(abs(ad - tl) / max(abs(tl), 1e-300))
        adj = {"workload": "euler_shear_layer_128x128x2_p3_dubiner_fp64", "elements": actx.n_elements,
               "steps": na, "checkpoint_every": ce, "dt": adt, "J": Jv,
               "forward_ms_per_step": 1e3 * t_fwd / na, "gradient_s": t_grad,
               "gradient_vs_forward_solve": t_grad / t_fwd,
               "adjoint_step_vs_forward_step": (t_grad - t_fwd) / t_fwd,
               "uniform_states_held": uniform_states, "uniform_recomputed_steps": na,
               "uniform_state_mb": uniform_states * au0.numel() * 8 / 1e6, "binomial": binomial,
               "fd_directions": args.adj_dirs, "fd_h": h, "fd_direction_norm": "||d|| = ||u0|| (h is a relative step)",
               "fd_max_rel_err": max(fd_err) if fd_err else None,
               "fd_median_rel_err": float(np.median(fd_err)) if fd_err else None,
               "fd_min_abs_derivative": min(fd_abs) if fd_abs else None,
               "fd_max_err_vs_grad_norm": max(fd_cs) if fd_cs else None,
               "tlm_directions": len(tlm_err), "tlm_max_rel_err": max(tlm_err) if tlm_err else None}
        del actx

    cfg1 = config1_leg(dg, torch)

    quads = None
    if args.quad_cells > 0:
        quads = {f"p{o}": quad_leg(dg, torch, args.quad_cells, args.quad_steps, o) for o in (3, 4)}

    bat = None
    if args.batch_instances > 0:
        bat = batch_leg(dg, torch, args.batch_instances, args.batch_steps, args.seed)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline and args.cells == N_CELLS:
        w = OracleWorkload(1, args.seed)
        rate, secs = w.run(args.cpu_steps)
        cpu = {"value": rate, "unit": "DOF*stages/s", "cores": 1, "kind": "port",
               "sample": f"{args.cpu_steps} SSP-RK3 steps (same dt) of the full 512x512x2 p=3 mesh "
                         f"({secs:.1f} s), FP64 oracle restatement of dgfem's single-threaded path"}

    if rank == 0:
        # compact line: the contract keys and the headline of the metric (mixed vs FP64 at the
        # stated error, adjoint/forward ratio); every leg in full goes to the details file
        line = {"metric": "DOF*RK-stages/s", "value": v_mx, "unit": "DOF*stages/s", "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_mx / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 flux/contractions + f64 geometry, mass inverse, RK3 state",
                "data": "synthetic", "config": workload_config(args.cells, dof, dt, ws),
                "fp64": {"value": v_64, "ms_per_step": 1e3 * t_64 / k64},
                "mixed_vs_fp64": v_mx / v_64,
                "accuracy": {k: acc[k] for k in ("steps", "mixed_vs_fp64_l2_rel", "mixed_vs_fp64_linf_rel",
                                                 "mixed_vs_exact_l2_rel", "fp64_vs_exact_l2_rel") if k in acc},
                "adjoint_forward_ratio": None if adj is None else adj["adjoint_step_vs_forward_step"],
                "stage_kernel": {"form": form, "grid": grid, "tile": tile},
                "tensor_core_form": {"ms_per_step": tensor_core["ms_per_step"],
                                     "mixed_vs_fp64_l2_rel": tensor_core["mixed_vs_fp64_l2_rel"]},
                "e2e": {"value": v_e2e, "unit": "DOF*stages/s", "h2d_bytes_per_step": dof * 8,
                        "d2h_bytes_per_step": dof * 8},
                # per timed rk3_step call: the FP32 copy of u^n, the face traces of it (trace
                # form), then three stage launches per step
                "gpu_launches": 3 * args.steps + (2 if form.startswith("traces") else 1),
                "roofline": {k: roof[k] for k in ("bound", "achieved", "peak", "unit", "frac", "traffic",
                                                  "launch_ms", "peak_kind")},
                "clocks": clocks,
                "cpu_baseline": cpu,
                "details": args.details}
        details = {"line": line, "roofline": roof,
                   "fp64_flop_roofline": flop_roofline(ORDER, False, ne, 1e3 * t_64 / k64, MEASURED_FP64_TFLOPS, "fp64"),
                   "mixed_flop_roofline": flop_roofline(ORDER, False, ne, 1e3 * t_mx / args.steps, MEASURED_FP32_TFLOPS,
                                                        "fp32"),
                   "stage_kernel": {"form": form, "grid": grid, "tiles": tiles,
                                                                    "elements_per_cta": tile,
                                                                    "picked_by": "autotuner (timed on the first step)"},
                   "tensor_core_form": tensor_core, "df64": df64, "accuracy": acc, "navier_stokes": ns,
                   "adjoint": adj, "batched": bat, "config1": cfg1, "quadrilaterals": quads, "setup": setup,
                   "e2e_steps": ke}
        try:
            Path(args.details).parent.mkdir(parents=True, exist_ok=True)
            Path(args.details).write_text(json.dumps(details, indent=1))
        except OSError as ex:
            print(f"bench: could not write {args.details}: {ex}", file=sys.stderr)
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
