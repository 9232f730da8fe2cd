#!/usr/bin/env python
"""Benchmark of the plain CPFEM method on the 32^3 FCC polycrystal (64 Voronoi grains,
304-steel-like constants, tension in 1e-3 strain steps, roller boundary conditions).

One step = one load step of the reference driver loop (global Newton to convergence with
BiCGSTAB + Jacobi, per-cell stress, committed internal variables), as
``singlecrystal_copper/singlecrystal_copper.py:179-233`` runs it.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line.  ``value`` = committed GP updates per second (Gauss points x timed
load steps / device time), ``e2e`` = the same through the public API with host buffers.
"""
from __future__ import annotations

import argparse
import importlib
import json
import math
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GP updates/s; 32³ RVE s/load-step; grad÷fwd & batched÷serial time at 1e-8 err"
UNIT = "GP updates/s"
N_EDGE, N_GRAINS, SEED = 32, 64, 0
STRAIN_STEP, DT = 1e-3, 0.1


def workload_config(n=N_EDGE, config="c1"):
    name = {"c0": f"fcc-single-crystal-{n}^3-copper-tension",
            "c2": f"bcc24-polycrystal-{n}^3-512grains-tantalum-tension"}.get(
        config, f"fcc-polycrystal-{n}^3-{N_GRAINS}grains-304steel-tension")
    grains = {"c0": 1, "c2": 512}.get(config, N_GRAINS)
    return {"workload": name,
            "cells": n ** 3, "gauss_points": 8 * n ** 3, "dofs": 3 * (n + 1) ** 3, "grains": grains,
            "strain_per_step": STRAIN_STEP, "dt_s": DT, "bcs": "rollers x=0,y=0,z=0; u_z(top)",
            "linear_solver": "BiCGSTAB tol=atol=1e-10", "newton": "tol 1e-6 / rel_tol 1e-8",
            "l2": "working set > L2 (state+tangent+CSR ~0.4 GB per step)"}


def _pkg():
    return importlib.import_module("jax-cpfem_gb300")


def make_case(pkg, n=N_EDGE):
    mesh = pkg.box_mesh(n, n, n)
    ori, rng = pkg.mesh.voronoi_grains(mesh, N_GRAINS, SEED)
    quat = pkg.material.random_quaternions(rng, N_GRAINS)
    return mesh, quat, ori


def roller_lists(pkg, mesh, disp):
    p = mesh.points
    fn = pkg.mesh.face_nodes
    nodes = [fn(p, 0, 0.0), fn(p, 1, 0.0), fn(p, 2, 0.0), fn(p, 2, 1.0)]
    return nodes, [0, 1, 2, 2], [0.0, 0.0, 0.0, disp]


class Stepper:
    """Device-resident load-step loop through the public API."""

    def __init__(self, pkg, prob, solver_mod, mesh):
        self.pkg, self.prob, self.solver, self.mesh = pkg, prob, solver_mod, mesh
        self.i = 0
        self.precond = 1
        self.mg_options = None
        self.grid_blocks = 0
        self.params = prob.internal_vars
        import torch
        self.sol = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64, device="cuda")

    def step(self, host_io=None):
        prob = self.prob
        self.i += 1
        prob.dt = DT
        nodes, comps, vals = roller_lists(self.pkg, self.mesh, STRAIN_STEP * self.i)
        prob.fes[0].set_dirichlet_lists(nodes, comps, vals)
        prob.set_params(self.params)
        if host_io is not None:
            sol_h, sig_h = host_io
            guess = sol_h.to("cuda", non_blocking=True)
        else:
            guess = self.sol
        sol = self.solver.solver(prob, {"jax_solver": {"precond": self.precond, "mg_options": self.mg_options,
                                                       "grid_blocks": self.grid_blocks},
                                        "initial_guess": [guess.reshape(-1, 3)]})[0]
        sig = prob.compute_avg_stress(sol, self.params)
        self.params = prob.update_int_vars_gp(sol, self.params)
        self.sol = sol.reshape(-1)
        if host_io is not None:
            sol_h.copy_(self.sol, non_blocking=True)
            sig_h.copy_(sig.reshape(-1), non_blocking=True)
        return sig


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms.  Started before the
    warm-up (its start-up stalls the GPU driver for a moment), and summarised over the samples
    whose timestamps fall inside the timed region."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.dev = device_index
        self.proc = None
        self.window = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)
            self.proc = None

    def summary(self, t0, t1):
        import datetime
        self.stop()
        self.f.flush()
        self.f.seek(0)
        rows = [[c.strip() for c in r.split(",")] for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sel = []
        for r in rows:
            try:
                ts = datetime.datetime.strptime(r[0], "%Y/%m/%d %H:%M:%S.%f").timestamp()
            except (ValueError, IndexError):
                continue
            if t0 - 0.25 <= ts <= t1 + 0.25:
                sel.append(r)
        if not sel:
            sel = rows[-3:]
        if not sel:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        num = lambda v: float(v) if v.replace(".", "", 1).isdigit() else None
        sm = [num(r[2]) for r in sel if len(r) > 3 and num(r[2]) is not None]
        smax = [num(r[3]) for r in sel if len(r) > 3 and num(r[3]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for r in sel:
            for k, nm in enumerate(names):
                if len(r) > 6 + k and r[6 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sel)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def fp64_peak(lib, torch):
    """Measured FP64 FMA throughput of this GPU (TFLOP/s), from cpfem_probe_dfma."""
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    flops = np.zeros(1)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    best = 0.0
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = lib.cpfem_probe_dfma(1024, 8 * sms, out.data_ptr(), flops.ctypes.data,
                                  torch.cuda.current_stream().cuda_stream)
        e1.record()
        torch.cuda.synchronize()
        assert rc == 0
        best = max(best, flops[0] / (e0.elapsed_time(e1) * 1e-3) / 1e12)
    return best


def spmv_roofline(prob, torch, lib, reps=50):
    """Average device time of one sliced-ELL SpMV on the final matrix (events)."""
    x = torch.randn(prob.num_total_dofs_all_vars, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    args = (prob.sell, prob.A_values.data_ptr(), x.data_ptr(), y.data_ptr(), 0,
            torch.cuda.current_stream().cuda_stream)
    for _ in range(3):
        lib.cpfem_spmv(*args)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        lib.cpfem_spmv(*args)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) * 1e-3 / reps
    nnz, nb, ndof = prob.nnz, prob.num_blocks, prob.num_total_dofs_all_vars
    # values + one column index per 3x3 block + x once + y (algorithmic, no padding)
    alg_bytes = 8 * nnz + 4 * nb + 8 * ndof + 8 * ndof
    return t, alg_bytes, 2.0 * nnz


# DRAM bytes (read + write) per launch from the ncu capture summarised in
# profiles/dram_fcc32_loadstep.md, on the 32^3 benchmark matrix: the standalone SpMV and
# the persistent BiCGSTAB (the matrix is read from HBM once per solve, then from L2).
SPMV_DRAM_BYTES = {"c1": 72.4e6}
# DRAM bytes of one k_bicgstab launch from ncu captures of the 32^3 bench matrix, by
# (config, precond, V-cycle precision): Jacobi ~330 iterations, multigrid ~20-30
KRYLOV_DRAM_BYTES_PER_LAUNCH = {("c1", 1, None): 75.7e6, ("c1", 3, "fp64"): 107.9e6, ("c1", 3, "fp32"): 3.684e9}


def krylov_iteration_cost(prob, precond=1):
    """Algorithmic bytes and FP64 flops of one BiCGSTAB iteration: two SpMVs (values, one
    column index per 3x3 block, x and y once) and the vector phases as written (p/phat 5,
    q 2, s/shat 4, t 2, x/r 8 vector reads+writes of 8*ndof bytes); flops 2 per stored
    value per SpMV plus ~30 per dof (updates, Jacobi, six dot products).  With the
    multigrid preconditioner, two V-cycles: per level (pre_sweeps - 1) + residual +
    post_sweeps (coarsest: coarse_sweeps - 1) SpMVs with block-Jacobi applies (18 flops
    per node each), plus restriction (27 x 3 FMAs per coarse node) and prolongation.
    Returns (bytes, FP64 flops, FP32 flops): an FP32 V-cycle moves 4-byte values and
    vectors and its flops leave the FP64 pipe."""
    nnz, nb, ndof = prob.nnz, prob.num_blocks, prob.num_total_dofs_all_vars
    spmv = 8 * nnz + 4 * nb + 16 * ndof
    bytes_it, flops_it, flops32_it = 2 * spmv + 21 * 8 * ndof, 4.0 * nnz + 30.0 * ndof, 0.0
    if precond == 3 and getattr(prob, "mg_layouts", None):
        mg = prob._mg
        w = 4.0 if mg.precision == 1 else 8.0
        L = len(prob.mg_layouts)
        for l, (rowptr, _, _, _) in enumerate(prob.mg_layouts):
            n = rowptr.size - 1
            blocks = int(rowptr[-1])
            ops = (mg.coarse_sweeps - 1) if l == L - 1 else (mg.pre_sweeps - 1 + 1 + mg.post_sweeps)
            lf = ops * (18.0 * blocks + 18.0 * n) + 18.0 * n
            lb = ops * (9 * w * blocks + 4.0 * blocks + 6 * w * n) + 6 * w * n
            if l + 1 < L:
                nc = prob.mg_layouts[l + 1][0].size - 1
                lf += 2 * 27 * 3 * nc + 2 * 8 * 3 * n
                lb += w * 3 * (n + nc) * 2
            if mg.precision == 1:
                flops32_it += 2 * lf
            else:
                flops_it += 2 * lf
            bytes_it += 2 * lb
    return bytes_it, flops_it, flops32_it


def gp_flops_per_eval(num_slip, iters_mean, tangent=True, fp32_direction=True):
    """Algorithmic flops of one GP update (FMA = 2; pow, div, sqrt = 1 each), returned as
    (FP64, FP32): per local iteration one residual (tau 12N, power/slip 6N, L_p 18N, 3x3
    products and strain 130) in FP64, and one 6x6 Jacobian (per slip M^T d 18,
    sym(. (x) n) 15, kk pv 6, rank-one update 72; the cubic stiffness once on six columns,
    ~100) + LU/solve (~230), in FP32 when the local Newton takes FP32 directions (counted
    so for every iteration: a lower bound of the FP64 work); the tangent (FP64) adds a
    Jacobian + LU, 6 dP/ds directions (20N+220 each) and 9 columns (~220 each)."""
    N = num_slip
    residual = 36 * N + 130
    jac = 111 * N + 100
    lu = 230
    setup = 120 + residual
    tan = (jac + lu + 6 * (20 * N + 220) + 9 * 220) if tangent else 0
    direction = iters_mean * (jac + lu)
    fp64 = setup + iters_mean * residual + tan + 60 + (0 if fp32_direction else direction)
    return fp64, (direction if fp32_direction else 0.0)


def _oracle_pass_worker(job):
    """One host process: the oracle's constitutive + tangent + element pass on a chunk of
    cells, started at a common wall-clock instant; returns (start, end)."""
    points, cells, quat, ori, spec, start_at = job
    from oracle import cpfem_oracle as O
    used, inv = np.unique(cells, return_inverse=True)
    orc = O.OracleProblem(points[used], inv.reshape(cells.shape), O.FCC12, spec["C11"], spec["C12"], spec["C44"],
                          quat, ori, gss_initial=spec["gss_initial"], h=spec["h"], t_sat=spec["t_sat"],
                          gss_a=spec["gss_a"], xm=spec["xm"], r=spec["r"], coplanar=True)
    orc.dt = DT
    u = np.zeros(orc.ndof)
    u[2::3] = STRAIN_STEP * orc.points[:, 2]
    while time.time() < start_at:
        time.sleep(0.001)
    t0 = time.time()
    orc.newton_update(u)
    return t0, time.time()


def _spmv_worker(job):
    """One host process: `reps` products of its row block of the tangent pattern with the
    full vector (plus the iteration's vector updates on its rows), from a common start."""
    blk, ndof, reps, start_at = job
    x = np.ones(ndof)
    y = np.empty(blk.shape[0])
    while time.time() < start_at:
        time.sleep(0.001)
    t0 = time.time()
    for _ in range(reps):
        y = blk @ x
        y = blk @ x
        for _k in range(5):        # p, s, x, r updates and the six dots on the block's rows
            y = y + 0.5 * y
    return t0, time.time()


def cpu_baseline_sample(pkg, mesh, quat, ori, newton_passes, krylov_iters, cores=None, budget_s=20.0):
    """The oracle (numpy/scipy) on the host cores, on a bounded sample of the workload,
    scaled to s per load step.  Constitutive+tangent+assembly: `cores` spawned processes
    each run the oracle pass on 2048 cells at the same time (wall time of the slowest, x the
    passes per step, scaled to all cells).  Krylov: each process multiplies its row block
    of the full 32^3 tangent pattern (two SpMVs + vector updates per iteration); the
    iteration time is the slowest block's (synchronisation between iterations is not
    charged, which favours the CPU)."""
    import multiprocessing as mp
    import scipy.sparse as sp
    cores = cores or os.cpu_count() or 1
    spec = pkg.material.BENCH_STEEL
    sd = {k: getattr(spec, k) for k in ("C11", "C12", "C44", "gss_initial", "h", "t_sat", "gss_a", "xm", "r")}
    E = mesh.cells.shape[0]
    sub = 2048
    nchunk = max(1, min(cores, E // sub))
    ctx = mp.get_context("spawn")
    with ctx.Pool(nchunk) as pool:
        pool.map(abs, range(nchunk))        # start the workers before the common instant
        start = time.time() + 3.0
        jobs = [(mesh.points, mesh.cells[k * sub:(k + 1) * sub], quat, ori[k * sub:(k + 1) * sub], sd, start)
                for k in range(nchunk)]
        spans = pool.map(_oracle_pass_worker, jobs)
        t_pass = max(b for _, b in spans) - min(a for a, _ in spans)
        t_asm = t_pass * E / (sub * nchunk)
        # Krylov on the full pattern, split into row blocks
        dof = (3 * mesh.cells[:, :, None] + np.arange(3)).reshape(E, 24)
        I = np.repeat(dof[:, :, None], 24, axis=2).ravel()
        J = np.repeat(dof[:, None, :], 24, axis=1).ravel()
        ndof = 3 * mesh.points.shape[0]
        A = sp.csr_array((np.random.default_rng(0).random(I.size), (I, J)), shape=(ndof, ndof))
        A.sum_duplicates()
        rows = np.linspace(0, ndof, nchunk + 1).astype(np.int64)
        reps = 40
        start = time.time() + 3.0
        spans = pool.map(_spmv_worker, [(A[rows[k]:rows[k + 1]], ndof, reps, start) for k in range(nchunk)])
        t_it = (max(b for _, b in spans) - min(a for a, _ in spans)) / reps
    t_step = newton_passes * t_asm + krylov_iters * t_it
    return {"value": 8 * E / t_step, "unit": UNIT, "cores": nchunk, "kind": "port",
            "s_per_load_step": t_step,
            "sample": (f"oracle newton_update on {nchunk} processes x {sub} cells at once ({t_pass:.2f} s wall, "
                       f"scaled to {E} cells: {t_asm:.2f} s/pass) x {newton_passes} passes + row-block "
                       f"BiCGSTAB iterations of the full {ndof}-dof pattern on {nchunk} processes "
                       f"({t_it * 1e3:.2f} ms/it, {reps} timed) x {krylov_iters} iterations")}


def run_reference(args):
    """The reference's CPU path is JAX; JAX is not installed, so the reference arm times
    the CPU restatement of the same algorithm (the oracle port) on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    pkg = _pkg()
    mesh, quat, ori = make_case(pkg)
    # counts of this workload's load steps measured on the GPU path (same algorithm)
    newton_passes, krylov_iters = REF_COUNTS["passes_per_step"], REF_COUNTS["krylov_iters_per_step"]
    vals = []
    for k in range(max(1, min(args.steps, 2))):
        vals.append(cpu_baseline_sample(pkg, mesh, quat, ori, newton_passes, krylov_iters))
    v = float(np.median([r["value"] for r in vals]))
    cb = dict(vals[-1])
    cb["value"] = v
    cb["sample"] += "; counts per step from the GPU path on this workload"
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": 8 * N_EDGE ** 3 / v * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload_config(), "impl": "reference",
           "cpu_baseline": cb,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "reference JAX/JAX-FEM path not installable offline; oracle port of the same algorithm"}
    print(json.dumps(out))


# Per-load-step counts of this workload on the GPU path (tension steps 1..20):
# constitutive+tangent passes (Newton iterations + 1) and BiCGSTAB iterations summed over
# the step's linear solves.  Refreshed from the GPU bench run.
REF_COUNTS = {"passes_per_step": 6, "krylov_iters_per_step": 2630}


def run_adjoint_config(args, pkg, problem_mod, torch):
    """configs[3]: gradient of the sigma_zz-curve misfit on the 32^3 / 64-grain RVE with
    respect to (h0, g0, gs, a, m) and the 64x3 Euler angles; backward / forward time."""
    from importlib import import_module
    adjoint = import_module("jax-cpfem_gb300.adjoint")
    n = args.edge
    mesh, quat, ori = make_case(pkg, n)
    spec = pkg.material.BENCH_STEEL
    prob = problem_mod.CrystalPlasticity(mesh, additional_info=(quat, ori), material=spec)
    nsteps = args.load_steps or 20

    def bc_fn(i, d):
        nodes, comps, vals = roller_lists(pkg, mesh, d)
        return nodes, comps, vals

    disps = STRAIN_STEP * np.arange(nsteps + 1)
    ts = DT * np.arange(nsteps + 1)
    # forward and transposed (adjoint) solves with the same preconditioner
    mg = {"precision": args.mg_precision} if args.mg_precision else None
    h = adjoint.LoadHistory(prob, disps, ts, bc_fn, quat,
                            solver_options={"jax_solver": {"precond": args.precond, "mg_options": mg}},
                            adjoint_options={"precond": args.precond, "mg_options": mg})
    theta = np.array([spec.h, spec.gss_initial, spec.t_sat, spec.gss_a, spec.xm])
    euler = np.zeros((N_GRAINS, 3))
    # synthetic target: h0, g0, gs scaled by 1.1 under the same seed
    target = h.forward(theta * np.array([1.1, 1.1, 1.1, 1.0, 1.0]), euler).cpu().numpy()[:, 2, 2]
    # untimed backward of that run: every kernel of the backward path (the library's and
    # torch's) has run once before the clock starts, as the forward's have
    h.backward(np.ones((nsteps, 3, 3)))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s = h.forward(theta, euler).cpu().numpy()[:, 2, 2]
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    sbar = np.zeros((nsteps, 3, 3))
    sbar[:, 2, 2] = 2.0 * (s - target) / nsteps
    t0 = time.perf_counter()
    tb, eb = h.backward(sbar)
    torch.cuda.synchronize()
    t_bwd = time.perf_counter() - t0
    out = {"metric": METRIC, "value": t_bwd / t_fwd, "unit": "backward/forward time", "higher_is_better": False,
           "n_gpus": 1, "steps": nsteps, "warmup": 0, "dtype": "f64", "data": "synthetic",
           "config": dict(workload_config(n), workload=f"adjoint-fcc-polycrystal-{n}^3-{N_GRAINS}grains",
                          load_steps=nsteps, params="h0,g0,gs,a,m + 64x3 Euler angles",
                          precond={1: "jacobi", 2: "block-jacobi-3x3", 3: "multigrid-vcycle"}.get(args.precond),
                          mg_precision=(args.mg_precision or "fp64") if args.precond == 3 else None),
           "forward_s": t_fwd, "backward_s": t_bwd, "gradient_over_forward": (t_fwd + t_bwd) / t_fwd,
           "objective": float(((s - target) ** 2).mean()), "theta_grad": tb.tolist(),
           "euler_grad_norm": float(np.linalg.norm(eb)), "adjoint_krylov_iters": h.krylov_iters}
    if args.fd_check:
        rng = np.random.default_rng(1)
        d_t = rng.normal(size=5) * theta * 1e-6
        d_e = rng.normal(size=euler.shape) * 1e-4
        f = lambda th, eu: float(((h.forward(th, eu, checkpoint=False).cpu().numpy()[:, 2, 2] - target) ** 2).mean())
        # the difference quotient runs the reference's local iterates (S = 0 start, FP64
        # directions): a warm start or an FP32 direction ends the local solve as soon as the
        # residual is below the tolerance, so the map is smooth only to that tolerance (~1e-10
        # relative), which a 1e-6 step amplifies
        prob.warm_start_local = prob.fp32_local_jacobian = False
        fd = (f(theta + d_t, euler + d_e) - f(theta - d_t, euler - d_e)) / 2.0
        prob.warm_start_local = prob.fp32_local_jacobian = True
        ad = float(tb @ d_t + (eb * d_e).sum())
        out["directional_fd_check"] = {"fd": fd, "adjoint": ad, "rel_err": abs(fd - ad) / abs(fd),
                                       "fd_local_solve": "S = 0 start, FP64 directions (the reference's iterates)"}
    print(json.dumps(out))


def run_batch_config(args, pkg, torch):
    """configs[4]: 256 RVEs (edges 8..24, 8-64 grains, parameters +-20 %) batched in one
    ragged launch per Newton stage vs the same solves one at a time."""
    from importlib import import_module
    batch = import_module("jax-cpfem_gb300.batch")
    inst = batch.sample_instances(args.instances, pkg.material.BENCH_STEEL, seed=SEED)
    nsteps = args.load_steps or 2
    disps = STRAIN_STEP * np.arange(1, nsteps + 1)
    # untimed warm-up of every kernel on a tiny batch (module loads, allocator growth)
    w = batch.Batch(batch.sample_instances(2, pkg.material.BENCH_STEEL, seed=SEED + 1, edges=(2,), grains=(2, 2)))
    w.step(STRAIN_STEP, DT)
    batch.run_serial(w.instances, [STRAIN_STEP], DT)
    del w
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = batch.Batch(inst)
    torch.cuda.synchronize()
    t_setup_batch = time.perf_counter() - t0
    b.problem.timing = True
    t0 = time.perf_counter()
    szz = np.stack([b.step(d, DT).cpu().numpy() for d in disps], axis=1)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    regions = b.problem.timer_ms()
    host = dict(b.host_s)
    newton = [int(x.max()) for x in b.stats["newton_iters"]]
    newton_mean = [float(x.mean()) for x in b.stats["newton_iters"]]
    kry = [int(x.max()) for x in b.stats["krylov_iters"]]
    del b
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    prepared = batch.build_serial(inst)
    torch.cuda.synchronize()
    t_setup_serial = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = batch.run_serial(inst, disps, DT, prepared=prepared)
    torch.cuda.synchronize()
    t_serial = time.perf_counter() - t0
    rel = float(np.abs(szz - ref).max() / np.abs(ref).max())
    gps = sum(8 * it.edge ** 3 for it in inst)
    print(json.dumps({"metric": METRIC, "value": t_serial / t_batch, "unit": "serial/batched time",
                      "higher_is_better": True, "n_gpus": 1, "steps": nsteps, "warmup": 1, "dtype": "f64",
                      "data": "synthetic",
                      "config": {"workload": f"batch-{len(inst)}-rves-edges8-24", "instances": len(inst),
                                 "gauss_points": gps, "load_steps": nsteps,
                                 "timed": "load steps only; problem set-up timed separately on both sides"},
                      "batched_s": t_batch, "serial_s": t_serial,
                      "setup_s": {"batched": t_setup_batch, "serial": t_setup_serial},
                      "with_setup_ratio": (t_serial + t_setup_serial) / (t_batch + t_setup_batch),
                      "max_rel_diff_vs_serial": rel,
                      "batched_regions_ms": {k: {"launches": v[0], "ms": v[1]} for k, v in regions.items()},
                      "batched_host_s": host,
                      "batched_newton_iters": newton, "batched_newton_iters_mean": newton_mean,
                      "batched_krylov_iters_max": kry,
                      "batched_gp_updates_per_s": gps * nsteps / t_batch}))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--edge", type=int, default=N_EDGE, help="cube edge in cells (32 = the benchmark)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--mg-refresh", default="newton", choices=["newton", "step"],
                    help="multigrid coarse operators rebuilt per Newton iteration (default) or once per load step")
    ap.add_argument("--no-tune", action="store_true", help="skip the linear-solver autotuning before warm-up ends")
    ap.add_argument("--mg-precision", default=None, choices=["fp64", "fp32"],
                    help="fix the V-cycle precision (default: the autotuner's choice, FP64 untuned)")
    ap.add_argument("--no-jacobi-leg", action="store_true",
                    help="skip the two extra load steps timed with the reference's Jacobi preconditioner")
    ap.add_argument("--config", default="c1", choices=["c0", "c1", "c2", "c3", "c4"],
                    help="c1 (default): 32^3 FCC polycrystal; c0: 10^3 copper single crystal; "
                         "c2: 64^3 BCC24 polycrystal; c3: adjoint on c1; c4: 256-RVE batch")
    ap.add_argument("--load-steps", type=int, default=0)
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--fd-check", action="store_true")
    ap.add_argument("--precond", type=int, default=3, choices=[0, 1, 2, 3],
                    help="BiCGSTAB preconditioner: 3 geometric multigrid V-cycle (default; same stop rule, "
                         "fewer iterations), 1 Jacobi (the reference's), 2 3x3 block-Jacobi")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    pkg = _pkg()
    problem_mod, solver_mod = pkg.load()
    from importlib import import_module
    lib = import_module("jax-cpfem_gb300._capi").load()

    if args.config == "c3":
        run_adjoint_config(args, pkg, problem_mod, torch)
        return
    if args.config == "c4":
        run_batch_config(args, pkg, torch)
        return
    n = args.edge
    spec = pkg.material.BENCH_STEEL
    if args.config == "c0":
        n = 10
        mesh, quat, ori = pkg.box_mesh(n, n, n), np.array([[1.0, 0.0, 0.0, 0.0]]), np.zeros(n ** 3, dtype=np.int64)
        spec = pkg.material.BENCH_COPPER
    elif args.config == "c2":
        n = 64
        mesh = pkg.box_mesh(n, n, n)
        ori, rng = pkg.mesh.voronoi_grains(mesh, 512, SEED)
        quat = pkg.material.random_quaternions(rng, 512)
        spec = pkg.material.BENCH_TANTALUM
    else:
        mesh, quat, ori = make_case(pkg, n)
    prob = problem_mod.CrystalPlasticity(mesh, additional_info=(quat, ori), material=spec)
    counter = CountingLib(prob.lib)
    prob.lib = counter
    st = Stepper(pkg, prob, solver_mod, mesh)
    st.precond = args.precond
    st.mg_options = {"refresh": args.mg_refresh}
    if args.mg_precision:
        st.mg_options["precision"] = args.mg_precision
    clk = ClockSampler(local).start()
    time.sleep(1.0)
    # warm-up with the timers on, so every kernel the timed steps use (including torch's
    # small reductions) has run once before the clock starts
    prob.timing = True
    tuned = None
    for w in range(args.warmup):
        st.step()
        if w == 0 and args.precond == 3 and not args.no_tune:
            # autotune the multigrid / launch settings on the next step's first Newton system
            tuning = import_module("jax-cpfem_gb300.tuning")
            nodes, comps, vals = roller_lists(pkg, mesh, STRAIN_STEP * (st.i + 1))
            prob.fes[0].set_dirichlet_lists(nodes, comps, vals)
            prob.set_params(st.params)
            res, A = solver_mod.newton_update_helper(prob, st.sol)
            x0 = solver_mod.initial_increment(prob, st.sol).clone()
            search = tuning.SEARCH
            start = dict(tuning.DEFAULT)
            if args.mg_precision:   # a fixed precision is not searched
                start["precision"] = args.mg_precision
                search = tuple(kv for kv in search if kv[0] != "precision")
            cfg, table = tuning.tune_linear_solver(prob, A, -res, x0, search=search, start=start)
            st.grid_blocks = cfg["grid_blocks"]
            st.mg_options = dict({k: v for k, v in cfg.items() if k != "grid_blocks"}, refresh=args.mg_refresh)
            tuned = {"chosen": cfg, "candidates": len(table),
                     "default_ms": round(table[0][1], 3), "chosen_ms": round(min(t[1] for t in table
                                                                                   if t[0] == cfg), 3)}
    torch.cuda.synchronize()
    prob.timer_ms()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    prob.timing = True
    prob.stats["krylov_iters"] = []
    passes0 = prob.stats["gp_passes"]
    newton = []
    barrier()
    torch.cuda.synchronize()
    wall0 = time.time()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    counter.counting = True
    e0.record()
    for _ in range(args.steps):
        st.step()
        newton.append(prob.stats["newton_iters"])
    e1.record()
    torch.cuda.synchronize()
    counter.counting = False
    wall1 = time.time()
    barrier()
    t = max_over_ranks(e0.elapsed_time(e1) * 1e-3, world, "cuda")
    regions = prob.timer_ms()
    prob.timing = False
    krylov = list(prob.stats["krylov_iters"])
    passes = prob.stats["gp_passes"] - passes0
    G = prob.num_gp
    value = world * G * args.steps / t
    clocks = clk.summary(wall0, wall1)

    # end-to-end through the public API with pinned host buffers
    e2e = None
    if not args.no_e2e:
        sol_h = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64).pin_memory()
        sol_h.copy_(st.sol.cpu())
        sig_h = torch.zeros(prob.num_cells * 9, dtype=torch.float64).pin_memory()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            st.step(host_io=(sol_h, sig_h))
        torch.cuda.synchronize()
        te = time.perf_counter() - w0
        e2e = {"value": world * G * args.steps / te, "unit": UNIT,
               "h2d_bytes_per_step": int(sol_h.numel() * 8), "d2h_bytes_per_step": int((sol_h.numel() + sig_h.numel()) * 8),
               "s_per_load_step": te / args.steps}

    # the same load steps with the reference's Jacobi-preconditioned BiCGSTAB, for comparison
    jacobi = None
    if args.precond != 1 and not args.no_jacobi_leg:
        st.precond, gb = 1, st.grid_blocks
        st.grid_blocks = 0
        st.step()
        torch.cuda.synchronize()
        k0 = len(prob.stats["krylov_iters"])
        j0, j1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        j0.record()
        for _ in range(2):
            st.step()
        j1.record()
        torch.cuda.synchronize()
        jacobi = {"precond": "jacobi (the reference's)", "steps": 2,
                  "ms_per_step": max_over_ranks(j0.elapsed_time(j1) * 1e-3, world, "cuda") / 2 * 1e3,
                  "krylov_iters": [int(k) for k in prob.stats["krylov_iters"][k0:]]}
        st.precond, st.grid_blocks = args.precond, gb

    # roofline of the dominant kernel (the persistent BiCGSTAB) and of the constitutive pass
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    fp64 = fp64_peak(lib, torch)
    t_spmv, spmv_bytes, spmv_flops = spmv_roofline(prob, torch, lib)
    its_t = prob.stats.get("local_iters_mean", 6.0)
    gp_n, gp_ms = regions.get("gp_eval_tangent", (0, 0.0))
    gp_t = gp_ms * 1e-3 / max(gp_n, 1)
    gp64, gp32 = gp_flops_per_eval(prob.num_slip, its_t, fp32_direction=prob.fp32_local_jacobian)
    gp_flops = G * gp64
    kr_n, kr_ms = regions.get("bicgstab", (0, 0.0))
    kr_its = sum(max(k, 0) for k in krylov)
    kb, kf, kf32 = krylov_iteration_cost(prob, args.precond)
    mg_fp32 = args.precond == 3 and getattr(prob, "_mg", None) is not None and prob._mg.precision == 1
    kr_key = (args.config, args.precond, ("fp32" if mg_fp32 else "fp64") if args.precond == 3 else None)
    kr_roof = None
    if kr_n and kr_ms > 0:
        tflops = kf * kr_its / (kr_ms * 1e-3) / 1e12
        gbs = kb * kr_its / (kr_ms * 1e-3) / 1e9
        kr_roof = {"bound": "fp64", "achieved": tflops, "peak": fp64, "unit": "TFLOP/s", "frac": tflops / fp64,
                   "traffic": KRYLOV_DRAM_BYTES_PER_LAUNCH.get(kr_key) if n == N_EDGE else None,
                   "traffic_note": "DRAM bytes per launch (ncu); algorithmic bytes per launch = "
                                   "algorithmic_bytes_per_iteration x iterations, served from L2",
                   "kernel": ("k_bicgstab<0,%d> (persistent multigrid-preconditioned BiCGSTAB, %s V-cycle, one "
                              "launch per linear solve)" % ((2, "FP32") if mg_fp32 else (1, "FP64"))
                              if args.precond == 3 else
                              "k_bicgstab<0,0> (persistent BiCGSTAB, one launch per linear solve)"),
                   "launches": kr_n, "us_per_iteration": kr_ms * 1e3 / max(kr_its, 1),
                   "algorithmic_bytes_per_iteration": kb, "flops_per_iteration": kf,
                   "fp32_flops_per_iteration": kf32,
                   "limiter": ("grid barriers and load latency (29 grid barriers per iteration; ncu: barrier "
                               "and long-scoreboard stalls dominate, FP64 pipe 14-26 %)" if args.precond == 3
                               else "FP64 pipe (the SpMVs)"),
                   "hbm": {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm if hbm else None},
                   "peak_source": "cpfem_probe_dfma FP64 (of measured); HBM from MEASURED_PEAKS.json (of measured)"}
    spmv_roof = {"bound": "fp64", "achieved": spmv_flops / t_spmv / 1e12, "peak": fp64, "unit": "TFLOP/s",
                 "frac": (spmv_flops / t_spmv / 1e12) / fp64, "traffic": SPMV_DRAM_BYTES.get(args.config) if n == N_EDGE else None,
                 "kernel": "k_spmv (sliced-ELL, standalone)",
                 "hbm": {"achieved": spmv_bytes / t_spmv / 1e9, "peak": hbm, "unit": "GB/s",
                         "frac": (spmv_bytes / t_spmv / 1e9) / hbm if hbm else None},
                 "peak_source": "cpfem_probe_dfma FP64 (of measured); HBM from MEASURED_PEAKS.json (of measured)"}
    gp_roof = {"bound": "fp64", "achieved": gp_flops / gp_t / 1e12 if gp_t else None, "peak": fp64,
               "unit": "TFLOP/s", "frac": (gp_flops / gp_t / 1e12) / fp64 if gp_t else None, "traffic": None,
               "kernel": "k_gp_eval<N,tangent>", "peak_source": "cpfem_probe_dfma (of measured)",
               "local_iters_mean": its_t, "fp64_flops_per_gp": gp64, "fp32_flops_per_gp": gp32,
               "note": "FP64 flops counted with every local Newton direction in FP32 (a lower bound)"}
    shares = {"bicgstab": kr_ms / (t * 1e3), "gp_eval_tangent": gp_ms / (t * 1e3),
              "elem_assemble": regions.get("elem_assemble", (0, 0.0))[1] / (t * 1e3)}
    dominant = kr_roof if (kr_roof is not None and shares["bicgstab"] >= shares["gp_eval_tangent"]) else gp_roof

    cpu = None
    if rank == 0 and not args.no_cpu_baseline and args.config == "c1":
        # the CPU path is the reference's algorithm: Jacobi-preconditioned BiCGSTAB, so its
        # Krylov count per step comes from the Jacobi leg of this run (else the stored one)
        if jacobi is not None:
            kps = sum(max(k, 0) for k in jacobi["krylov_iters"]) / jacobi["steps"]
            src = "Jacobi-leg Krylov counts of this GPU run"
        elif args.precond == 1:
            kps = sum(max(k, 0) for k in krylov) / args.steps
            src = "Krylov counts of this GPU run"
        else:
            kps = REF_COUNTS["krylov_iters_per_step"]
            src = "stored Jacobi Krylov count of this workload"
        cpu = cpu_baseline_sample(pkg, mesh, quat, ori, passes / args.steps, kps)
        cpu["sample"] += f"; constitutive passes per step from this GPU run, {src}"

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": dict(workload_config(n, args.config), parallelism="replicas" if world > 1 else "single-gpu",
                          precond={0: "none", 1: "jacobi", 2: "block-jacobi-3x3", 3: "multigrid-vcycle"}[args.precond],
                          mg_refresh=args.mg_refresh if args.precond == 3 else None),
           "s_per_load_step": t / args.steps, "clocks": clocks, "e2e": e2e,
           "roofline": dominant,
           "roofline_kernels": {"bicgstab": kr_roof, "spmv": spmv_roof, "gp_eval": gp_roof},
           "region_shares": shares, "jacobi_leg": jacobi, "tuned_linear_solver": tuned,
           "cpu_baseline": cpu,
           "regions_ms": {k: {"launches": v[0], "ms": v[1]} for k, v in regions.items()},
           "newton_iters_per_step": newton, "krylov_iters": krylov, "gp_passes": passes,
           "gpu_launches": None}
    out["gpu_launches"] = counter.launches
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def max_over_ranks(t, world, device):
    """The job's time for independent replicas: the slowest rank's (all-reduce MAX)."""
    if world <= 1:
        return t
    import torch
    import torch.distributed as dist
    tt = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


class CountingLib:
    """Forwards to the C ABI and counts the kernels its calls launch (a fixed number per
    entry point, from the sources: the persistent BiCGSTAB is one launch plus the
    preconditioner set-up; every other listed entry point launches one kernel)."""
    LAUNCHES = {"cpfem_gp_eval": 1, "cpfem_elem_assemble": 1, "cpfem_apply_dirichlet": 1, "cpfem_dot": 1,
                "cpfem_bc_initial_guess": 1, "cpfem_axpy": 1, "cpfem_spmv": 1, "cpfem_bicgstab": 2,
                "cpfem_bicgstab_ex": 2, "cpfem_cell_average": 1, "cpfem_segmented_dot": 1,
                "cpfem_bicgstab_batched": 2, "cpfem_gp_vjp": 1}

    def __init__(self, lib):
        self._lib = lib
        self.launches = 0
        self.counting = False

    def __getattr__(self, name):
        f = getattr(self._lib, name)
        k = self.LAUNCHES.get(name)
        if k is None:
            return f

        def call(*a):
            if self.counting:
                self.launches += k
            return f(*a)
        return call


if __name__ == "__main__":
    main()
