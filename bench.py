#!/usr/bin/env python
"""Benchmark of the plain CPFEM method on the 32^3 FCC polycrystal (64 Voronoi grains,
304-steel-like constants, tension in 1e-3 strain steps, roller boundary conditions).

One step = one load step of the reference driver loop (global Newton to convergence,
per-cell stress, committed internal variables), as
``singlecrystal_copper/singlecrystal_copper.py:179-233`` runs it: on the GPU the benchmark
path of ``workloads.BENCH_SETTINGS`` (multigrid BiCGSTAB, extrapolated Newton guess,
inexact Krylov solves, FP32 tangent), on the CPU arm the reference's algorithm (Jacobi
BiCGSTAB to 1e-10) in the compiled oracle.

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
# Newton stop rule.  The CPU arm runs the reference's (tol 1e-6, rel_tol 1e-8,
# crystal_plasticity_OR_design/solver.py:384-385).  The GPU arm stops at an absolute residual
# of 1e-8 instead (same rel_tol): its Newton loop starts from an extrapolated guess and can
# stop after a different iterate than the reference's, and at the tighter limit its solution
# stays within 1e-8 of the discrete solution (the oracle converged to 1e-12), which the
# reference's own limit does not guarantee; in the steady state the last iterate is already
# far below either limit, so this costs no Newton iteration there.
NEWTON_REF = {"tol": 1e-6, "rel_tol": 1e-8}
BENCH = importlib.import_module("jax-cpfem_gb300.workloads").BENCH_SETTINGS
NEWTON = dict(BENCH["newton"])


def workload_config(n=N_EDGE, config="c1"):
    name = {"c0": f"fcc-single-crystal-{n}^3-copper-tension",
            "c2": f"bcc24-polycrystal-{n}^3-512grains-tantalum-tension"}.get(
        config, f"fcc-polycrystal-{n}^3-{N_GRAINS}grains-304steel-tension")
    grains = {"c0": 1, "c2": 512}.get(config, N_GRAINS)
    return {"workload": name,
            "cells": n ** 3, "gauss_points": 8 * n ** 3, "dofs": 3 * (n + 1) ** 3, "grains": grains,
            "strain_per_step": STRAIN_STEP, "dt_s": DT, "bcs": "rollers x=0,y=0,z=0; u_z(top)",
            "linear_solver": "BiCGSTAB, atol 1e-10, relative tol krylov_tol (the reference: 1e-10)",
            "newton": f"tol {NEWTON['tol']:g} / rel_tol {NEWTON['rel_tol']:g}",
            "l2": "working set > L2 (state+tangent+CSR ~0.4 GB per step)"}


def _pkg():
    return importlib.import_module("jax-cpfem_gb300")


def _workloads():
    return importlib.import_module("jax-cpfem_gb300.workloads")


def make_workload(config="c1", n=N_EDGE):
    W = _workloads()
    if config == "c0":
        return W.copper_single_crystal()
    if config == "c2":
        return W.tantalum_polycrystal()
    return W.steel_polycrystal(n, N_GRAINS, SEED)


# ---------------------------------------------------------------------------------------
# CPU path: the compiled oracle (the reference's algorithm, OpenMP on all host cores)
# ---------------------------------------------------------------------------------------
def host_cpu():
    import platform
    model = platform.processor() or platform.machine()
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    return {"cpu_count": os.cpu_count(), "model": model, "machine": platform.machine()}


def oracle_problem(w):
    """The compiled oracle on workload ``w`` with one OpenMP thread per host core."""
    from oracle import coracle
    from oracle import cpfem_oracle as O
    coracle.set_threads(os.cpu_count() or 1)
    s = w.spec
    return coracle.FastOracleProblem(w.mesh.points, w.mesh.cells, O.SLIP_TABLES[s.slip], s.C11, s.C12, s.C44,
                                     w.quat, w.ori, gss_initial=s.gss_initial, h=s.h, t_sat=s.t_sat,
                                     gss_a=s.gss_a, xm=s.xm, r=s.r, ao=s.ao, coplanar=s.coplanar_q,
                                     local_tol=s.local_tol, max_sub_step=s.max_sub_step)


def oracle_load_step(orc, w, i, sol, params):
    """Load step ``i`` (1-based) of the reference driver loop on the oracle
    (``singlecrystal_copper/singlecrystal_copper.py:179-233``): set dt and the top
    displacement, global Newton with Jacobi BiCGSTAB, ``compute_avg_stress``,
    ``update_int_vars_gp``.  Returns (sol, params, cell stresses, solver info)."""
    from oracle import cpfem_oracle as O
    orc.dt = w.dt
    orc.set_bcs(w.bc_triples(w.strain_step * i))
    orc.set_params(params)
    sol, info = O.solver(orc, dict(NEWTON_REF, initial_guess=sol))
    sig = orc.compute_avg_stress(sol, params)
    params = orc.update_int_vars_gp(sol, params)
    return sol, params, sig, info


def cpu_baseline_step(w, i, sol, params4):
    """One full load step (step ``i``) of the oracle on the host cores, started from a
    committed state (``sol``, the four state arrays) of the GPU run: the bounded CPU sample
    of the same workload."""
    from oracle import coracle
    orc = oracle_problem(w)
    params = [np.ascontiguousarray(p) for p in params4] + orc.internal_vars[4:9]
    t0 = time.perf_counter()
    _, _, _, info = oracle_load_step(orc, w, i, np.ascontiguousarray(sol), params)
    t = time.perf_counter() - t0
    kr = [int(k) for k in info["krylov_iters"]]
    threads = coracle.num_threads()
    return {"value": w.num_gp / t, "unit": UNIT, "cores": threads, "kind": "port", "s_per_load_step": t,
            "sample": (f"load step {i} of this workload run end to end by the compiled oracle (the reference's "
                       f"algorithm in C) from the GPU run's committed state at the start of that step: global "
                       f"Newton ({info['newton_iters']} iterations) with Jacobi BiCGSTAB ({sum(kr)} iterations), "
                       f"then compute_avg_stress and update_int_vars_gp, {threads} OpenMP threads"),
            "host": host_cpu(), "newton_iters": info["newton_iters"], "krylov_iters": kr}


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


FP64_PROBE = {"kernel": "k_dfma_probe", "threads": 256, "blocks_per_sm": 16, "chains_per_thread": 16,
              "fma_per_loop_trip": 64, "loop_trips": 512, "repeats": 5}


def fp64_peak(lib, torch):
    """Measured FP64 FMA throughput of this GPU (TFLOP/s), from cpfem_probe_dfma: the best
    of FP64_PROBE["repeats"] timed launches (CUDA events), each ~10-20 ms of DFMAs."""
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    flops = np.zeros(1)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    blocks = FP64_PROBE["blocks_per_sm"] * sms
    best = 0.0
    lib.cpfem_probe_dfma(64, blocks, out.data_ptr(), flops.ctypes.data, torch.cuda.current_stream().cuda_stream)
    for _ in range(FP64_PROBE["repeats"]):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rc = lib.cpfem_probe_dfma(FP64_PROBE["loop_trips"], blocks, out.data_ptr(), flops.ctypes.data,
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


# DRAM bytes (read + write) per launch from ncu captures on the 32^3 benchmark matrix: the
# standalone SpMV (profiles/k_spmv_fcc32.md) and the persistent BiCGSTAB with the FP32
# V-cycle (profiles/k_bicgstab_mg_fcc32.md; one Newton step's solve, ~12 iterations: the
# matrix is read from HBM once per solve, then from L2).
SPMV_DRAM_BYTES = {"c1": 72.4e6}
KRYLOV_DRAM_BYTES_PER_LAUNCH = {("c1", 3, "fp32"): 109.1e6}


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


def gp_flops_per_eval(num_slip, iters_mean, tangent=True, fp32_direction=True, fp32_tangent=False):
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
    fp64 = setup + iters_mean * residual + (0 if fp32_tangent else tan) + 60 + (0 if fp32_direction else direction)
    fp32 = (direction if fp32_direction else 0.0) + (tan if fp32_tangent else 0.0)
    return fp64, fp32


def run_reference(args):
    """The reference's CPU path is JAX, which is not installed; this arm runs the reference's
    algorithm as the compiled oracle, full load steps end to end on all host cores: W
    untimed load steps, then K timed ones (the same load steps the GPU arm times)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import coracle
    w = make_workload("c1", args.edge)
    t_setup = time.perf_counter()
    orc = oracle_problem(w)
    t_setup = time.perf_counter() - t_setup
    sol, params = np.zeros(orc.ndof), orc.internal_vars
    for i in range(1, args.warmup + 1):
        sol, params, _, _ = oracle_load_step(orc, w, i, sol, params)
    per_step, newton, krylov = [], [], []
    t0 = time.perf_counter()
    for i in range(args.warmup + 1, args.warmup + args.steps + 1):
        ts = time.perf_counter()
        sol, params, sig, info = oracle_load_step(orc, w, i, sol, params)
        per_step.append(time.perf_counter() - ts)
        newton.append(info["newton_iters"])
        krylov.append([int(k) for k in info["krylov_iters"]])
    t = time.perf_counter() - t0
    v = w.num_gp * args.steps / t
    threads = coracle.num_threads()
    cb = {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "s_per_load_step": t / args.steps,
          "sample": (f"load steps {args.warmup + 1}-{args.warmup + args.steps} of this workload (after "
                     f"{args.warmup} untimed ones), each run end to end by the compiled oracle: global Newton with "
                     f"Jacobi BiCGSTAB, compute_avg_stress, update_int_vars_gp; {threads} OpenMP threads"),
          "host": host_cpu()}
    out = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": dict(workload_config(args.edge), precond="jacobi", initial_guess="last solution",
                          linear_solver="BiCGSTAB tol=atol=1e-10",
                          newton=f"tol {NEWTON_REF['tol']:g} / rel_tol {NEWTON_REF['rel_tol']:g}"),
           "impl": "reference",
           "cpu_baseline": cb,
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "s_per_load_step": per_step, "newton_iters_per_step": newton, "krylov_iters": krylov,
           "setup_s": t_setup, "mean_sigma_zz_last": float(sig[:, 2, 2].mean()),
           "note": ("the reference's JAX/JAX-FEM path is not installable offline (no jax, jax_fem, meshio); "
                    "this is its algorithm restated in C (oracle/cpfem_oracle_c.c), timed, not modelled")}
    print(json.dumps(out))


def run_adjoint_config(args, pkg, problem_mod, torch):
    """The adjoint workload (gradient on the 32^3 RVE) as its own JSON line."""
    print(json.dumps(adjoint_record(args, pkg, problem_mod, torch)))


def adjoint_record(args, pkg, problem_mod, torch):
    """The adjoint workload: gradient of the sigma_zz-curve misfit on the 32^3 / 64-grain RVE with
    respect to (h0, g0, gs, a, m) and the 64x3 Euler angles; backward / forward time."""
    from importlib import import_module
    adjoint = import_module("jax-cpfem_gb300.adjoint")
    n = args.edge
    w = make_workload("c1", n)
    mesh, quat, ori, spec = w.mesh, w.quat, w.ori, w.spec
    prob = problem_mod.CrystalPlasticity(mesh, additional_info=(quat, ori), material=spec)
    nsteps = args.load_steps or 20

    def bc_fn(i, d):
        return w.bc_lists(d)

    disps = STRAIN_STEP * np.arange(nsteps + 1)
    ts = DT * np.arange(nsteps + 1)
    # forward and transposed (adjoint) solves with the same preconditioner
    mg = dict(_workloads().TUNED_MG)
    if args.mg_precision:
        mg["precision"] = args.mg_precision
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
    return out


def run_batch_config(args, pkg, torch):
    """The RVE batch: 256 RVEs (edges 8..24, 8-64 grains, parameters +-20 %) batched in one
    ragged launch per Newton stage vs the same solves one at a time."""
    from importlib import import_module
    batch = import_module("jax-cpfem_gb300.batch")
    inst = batch.sample_instances(args.instances, pkg.material.BENCH_STEEL, seed=SEED)
    nsteps = args.load_steps or 20
    disps = STRAIN_STEP * np.arange(1, nsteps + 1)
    # both arms run the same per-instance algorithm: Jacobi or 3x3 block-Jacobi BiCGSTAB (the
    # ragged solver's preconditioners), and the benchmark path's predictor, Krylov tolerance,
    # FP32 tangent and Newton limit
    fast = args.predictor == "linear"
    newton = dict(NEWTON) if fast else dict(NEWTON_REF)
    ktol = args.krylov_tol
    pc = args.batch_precond
    serial_opts = dict(newton, jax_solver={"tol": ktol, "precond": {1: True, 2: "block3"}[pc]})
    # untimed warm-up of every kernel on a tiny batch (module loads, allocator growth)
    w = batch.Batch(batch.sample_instances(2, pkg.material.BENCH_STEEL, seed=SEED + 1, edges=(2,), grains=(2, 2)))
    w.step(STRAIN_STEP, DT)
    batch.run_serial(w.instances, [STRAIN_STEP], DT)
    del w
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    b = batch.Batch(inst)
    b.predictor = args.predictor
    b.problem.fp32_tangent = bool(args.fp32_tangent)
    torch.cuda.synchronize()
    t_setup_batch = time.perf_counter() - t0
    b.problem.timing = True
    t0 = time.perf_counter()
    szz = np.stack([b.step(d, DT, ktol=ktol, precond=pc, **newton).cpu().numpy() for d in disps], axis=1)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    regions = b.problem.timer_ms()
    host = dict(b.host_s)
    newton_max = [int(x.max()) for x in b.stats["newton_iters"]]
    newton_mean = [float(x.mean()) for x in b.stats["newton_iters"]]
    fallbacks = int(b.stats.get("predictor_fallbacks", 0))
    kry = [int(x.max()) for x in b.stats["krylov_iters"]]
    del b
    torch.cuda.empty_cache()
    t0 = time.perf_counter()
    prepared = batch.build_serial(inst)
    for p_, _ in prepared:
        p_.fp32_tangent = bool(args.fp32_tangent)
    torch.cuda.synchronize()
    t_setup_serial = time.perf_counter() - t0
    t0 = time.perf_counter()
    ref = batch.run_serial(inst, disps, DT, prepared=prepared, solver_options=serial_opts, predictor=args.predictor)
    torch.cuda.synchronize()
    t_serial = time.perf_counter() - t0
    rel = float(np.abs(szz - ref).max() / np.abs(ref).max())
    gps = sum(8 * it.edge ** 3 for it in inst)
    print(json.dumps({"metric": METRIC, "value": t_serial / t_batch, "unit": "serial/batched time",
                      "higher_is_better": True, "n_gpus": 1, "steps": nsteps, "warmup": 1, "dtype": "f64",
                      "data": "synthetic",
                      "config": {"workload": f"batch-{len(inst)}-rves-edges8-24", "instances": len(inst),
                                 "gauss_points": gps, "load_steps": nsteps,
                                 "timed": "load steps only; problem set-up timed separately on both sides",
                                 "both_arms": {"precond": {1: "jacobi", 2: "block-jacobi-3x3"}[pc],
                                               "krylov_tol": ktol, "predictor": args.predictor,
                                               "tangent": "fp32" if args.fp32_tangent else "fp64",
                                               "newton": f"tol {newton['tol']:g} / rel_tol {newton['rel_tol']:g}"}},
                      "batched_s": t_batch, "serial_s": t_serial,
                      "setup_s": {"batched": t_setup_batch, "serial": t_setup_serial},
                      "with_setup_ratio": (t_serial + t_setup_serial) / (t_batch + t_setup_batch),
                      "max_rel_diff_vs_serial": rel,
                      "batched_regions_ms": {k: {"launches": v[0], "ms": v[1]} for k, v in regions.items()},
                      "batched_host_s": host,
                      "batched_newton_iters": newton_max, "batched_newton_iters_mean": newton_mean,
                      "batched_predictor_fallbacks": fallbacks,
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
    ap.add_argument("--no-sub-records", action="store_true",
                    help="skip the records appended to the default line: the adjoint on the same RVE and the "
                         "10^3 copper and 64^3 BCC24 load histories")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--mg-refresh", default=BENCH["mg_refresh"], choices=["newton", "step"],
                    help="multigrid coarse operators rebuilt once per load step (default: the preconditioner of a "
                         "step's later Newton systems is the first one's) or per Newton iteration")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the linear-solver autotuning during warm-up and use its stored choice for this "
                         "workload (workloads.TUNED_MG)")
    ap.add_argument("--mg-precision", default=None, choices=["fp64", "fp32"],
                    help="fix the V-cycle precision (default: the autotuner's choice, FP64 untuned)")
    ap.add_argument("--no-jacobi-leg", action="store_true",
                    help="skip the two extra load steps timed with the reference's Jacobi preconditioner")
    ap.add_argument("--config", default="c1", choices=["c0", "c1", "c2", "c3", "c4"],
                    help="c1 (default): 32^3 FCC polycrystal; c0: 10^3 copper single crystal; "
                         "c2: 64^3 BCC24 polycrystal; c3: adjoint on c1; c4: 256-RVE batch")
    ap.add_argument("--fp32-tangent", default=int(BENCH["fp32_tangent"]), type=int, choices=[0, 1],
                    help="consistent tangent (the global Newton's Jacobian) in FP32 where the local Jacobian's scale "
                         "allows (1, default) or FP64 (0); the residual and the converged state are FP64 either way")
    ap.add_argument("--predictor", default=BENCH["predictor"], choices=["linear", "previous"],
                    help="initial guess of each load step's Newton solve: linear extrapolation of the last two "
                         "solutions (default) or the last solution (the reference driver's)")
    ap.add_argument("--krylov-tol", type=float, default=BENCH["krylov_tol"],
                    help="relative tolerance of each Newton step's BiCGSTAB (the reference's: 1e-10; atol stays "
                         "1e-10): an inexact Newton step with the same Newton stop rule")
    ap.add_argument("--batch-precond", type=int, default=1, choices=[1, 2],
                    help="RVE batch: the preconditioner of both arms' BiCGSTAB, 1 Jacobi (the reference's) or "
                         "2 3x3 block-Jacobi")
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
    w = make_workload(args.config, args.edge)
    n = round(w.mesh.cells.shape[0] ** (1.0 / 3.0))
    mesh = w.mesh
    prob = problem_mod.CrystalPlasticity(mesh, additional_info=(w.quat, w.ori), material=w.spec)
    counter = CountingLib(prob.lib)
    prob.lib = counter
    W = _workloads()
    st = W.LoadStepper(prob, solver_mod, w, predictor=args.predictor)
    prob.fp32_tangent = bool(args.fp32_tangent)
    mg_options = {"refresh": args.mg_refresh}
    if args.mg_precision:
        mg_options["precision"] = args.mg_precision

    def set_solver(precond, mg, grid_blocks, krylov_tol=args.krylov_tol, newton=NEWTON):
        st.options = dict(newton, jax_solver={"precond": precond, "mg_options": mg, "grid_blocks": grid_blocks,
                                              "tol": krylov_tol})

    if args.no_tune and args.precond == 3:
        mg_options = dict(W.TUNED_MG, refresh=args.mg_refresh, **({"precision": args.mg_precision}
                                                                  if args.mg_precision else {}))
        set_solver(args.precond, mg_options, W.TUNED_GRID_BLOCKS)
    else:
        set_solver(args.precond, mg_options, 0)
    clk = ClockSampler(local).start()
    time.sleep(1.0)
    # warm-up with the timers on, so every kernel the timed steps use (including torch's
    # small reductions) has run once before the clock starts
    prob.timing = True
    tuned = None
    for wi in range(args.warmup):
        st.step()
        if wi == 0 and args.precond == 3 and not args.no_tune:
            # autotune the multigrid / launch settings on the next step's first Newton system
            tuning = import_module("jax-cpfem_gb300.tuning")
            prob.fes[0].set_dirichlet_lists(*w.bc_lists(w.strain_step * (st.i + 1)))
            prob.set_params(st.params)
            res, A = solver_mod.newton_update_helper(prob, st.sol)
            x0 = solver_mod.initial_increment(prob, st.sol).clone()
            search = tuning.SEARCH
            start = dict(tuning.DEFAULT)
            if args.mg_precision:   # a fixed precision is not searched
                start["precision"] = args.mg_precision
                search = tuple(kv for kv in search if kv[0] != "precision")
            # timed at the benchmark's Krylov tolerance; no candidate without post-smoothing:
            # a short solve can rank it first, and the later, harder Newton systems then
            # need twice the iterations
            search = tuple((k, tuple(v for v in vals if not (k == "post_sweeps" and v == 0)))
                           for k, vals in search)
            cfg, table = tuning.tune_linear_solver(prob, A, -res, x0, search=search, start=start,
                                                   tol=args.krylov_tol)
            mg_options = dict({k: v for k, v in cfg.items() if k != "grid_blocks"}, refresh=args.mg_refresh)
            set_solver(args.precond, mg_options, cfg["grid_blocks"])
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
    prob.stats["solves_dropped"] = 0
    passes0 = prob.stats["gp_passes"]
    newton = []
    # the state at the start of the timed steps: the end-to-end run repeats the same load
    # steps from it
    start = (st.i, st.sol.clone(), None if st.prev is None else st.prev.clone(), [t.clone() for t in st.params],
             {k: prob._bufs[k].clone() for k in ("s_warm", "s_dsdf", "s_f", "gp_order") if k in prob._bufs})
    # the committed state at the start of the first timed step (copied before the clock
    # starts): the CPU baseline runs that same load step from it
    snap = None
    if rank == 0 and not args.no_cpu_baseline and args.config == "c1":
        snap = (st.i + 1, st.sol.cpu().numpy().copy(), [p.cpu().numpy().copy() for p in st.params[:4]])
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
    dropped = int(prob.stats.get("solves_dropped", 0))
    passes = prob.stats["gp_passes"] - passes0
    G = prob.num_gp
    value = world * G * args.steps / t
    clocks = clk.summary(wall0, wall1)

    # end-to-end through the public API with pinned host buffers
    e2e = None
    if not args.no_e2e:
        # the same load steps from the same state, local-solve starts included; the state is
        # adopted before the clock starts
        st.i, st.sol, st.prev, st.params = start[0], start[1], start[2], list(start[3])
        for k, v in start[4].items():
            prob._bufs[k].copy_(v)
        prob.set_params(st.params)
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

    # the next load steps with the reference driver's own choices, for comparison: its initial
    # guess (the last solution) with this arm's solver, then also its Jacobi-preconditioned
    # BiCGSTAB (the drop-in's default configuration)
    legs = {}
    if not args.no_jacobi_leg:
        saved, pred, f32t = st.options, st.predictor, prob.fp32_tangent
        prob.fp32_tangent = False
        for name, precond in (("previous_guess", args.precond), ("jacobi", 1)):
            if precond == 1:
                set_solver(1, None, 0, 1e-10, NEWTON_REF)
            else:
                set_solver(args.precond, st.options["jax_solver"]["mg_options"], st.options["jax_solver"]["grid_blocks"],
                           1e-10, NEWTON_REF)
            st.predictor = "previous"
            st.step()
            torch.cuda.synchronize()
            k0 = len(prob.stats["krylov_iters"])
            nl = []
            j0, j1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            j0.record()
            for _ in range(2):
                st.step()
                nl.append(prob.stats["newton_iters"])
            j1.record()
            torch.cuda.synchronize()
            legs[name] = {"initial_guess": "last solution (the reference driver's)", "krylov_tol": 1e-10,
                          "newton": "tol 1e-6 / rel_tol 1e-8 (the reference's)",
                          "tangent": "fp64",
                          "precond": {1: "jacobi (the reference's)", 3: "multigrid-vcycle"}.get(precond, precond),
                          "steps": 2, "ms_per_step": max_over_ranks(j0.elapsed_time(j1) * 1e-3, world, "cuda") / 2 * 1e3,
                          "newton_iters_per_step": nl, "krylov_iters": [int(k) for k in prob.stats["krylov_iters"][k0:]]}
        st.options, st.predictor, prob.fp32_tangent = saved, pred, f32t
    jacobi = legs.get("jacobi")

    # roofline of the dominant kernel (the persistent BiCGSTAB) and of the constitutive pass
    peaks = measured_peaks()
    hbm = peaks.get("hbm_gbs")
    fp64 = fp64_peak(lib, torch)
    t_spmv, spmv_bytes, spmv_flops = spmv_roofline(prob, torch, lib)
    its_t = prob.stats.get("local_iters_mean", 6.0)
    gp_n, gp_ms = regions.get("gp_eval_tangent", (0, 0.0))
    gp_t = gp_ms * 1e-3 / max(gp_n, 1)
    gp64, gp32 = gp_flops_per_eval(prob.num_slip, its_t, fp32_direction=prob.fp32_local_jacobian,
                                   fp32_tangent=prob.fp32_tangent)
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
                               "and long-scoreboard stalls dominate, FP64 pipe 15-17 %)" if args.precond == 3
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
               "note": "FP64 flops counted with every local Newton direction (and, with the FP32 tangent, every "
                       "tangent) in FP32: a lower bound of the FP64 work"}
    # the coloured scatter: algorithmic bytes of a tangent scatter (per GP the tangent, the
    # shape gradients and P read once; per cell the read-add-write of its 64 3x3 blocks and
    # 24 residual entries) and of a residual-only one, over the scatter region's time
    asm_n, asm_ms = regions.get("elem_assemble", (0, 0.0))
    n_tan = regions.get("gp_eval_tangent", (0, 0.0))[0]
    n_res = regions.get("gp_eval_residual", (0, 0.0))[0]
    E = prob.num_cells
    tan_b = 4 if prob.fp32_tangent else 8
    bytes_tan = G * (81 * tan_b + 24 * 8 + 9 * 8) + E * (64 * 9 * 8 * 2 + 24 * 8 * 2)
    bytes_res = G * (24 * 8 + 9 * 8) + E * 24 * 8 * 2
    asm_roof = None
    if asm_ms > 0:
        asm_gbs = (n_tan * bytes_tan + n_res * bytes_res) / (asm_ms * 1e-3) / 1e9
        asm_roof = {"bound": "hbm", "achieved": asm_gbs, "peak": hbm, "unit": "GB/s",
                    "frac": asm_gbs / hbm if hbm else None, "traffic": None,
                    "kernel": "k_elem_assemble (coloured scatter, %s tangent)" % ("FP32" if prob.fp32_tangent else
                                                                                "FP64"),
                    "algorithmic_bytes_per_tangent_scatter": bytes_tan,
                    "algorithmic_bytes_per_residual_scatter": bytes_res, "scatters": [n_tan, n_res],
                    "peak_source": "HBM from MEASURED_PEAKS.json (of measured)"}
    shares = {"bicgstab": kr_ms / (t * 1e3), "gp_eval_tangent": gp_ms / (t * 1e3),
              "elem_assemble": regions.get("elem_assemble", (0, 0.0))[1] / (t * 1e3)}
    dominant = kr_roof if (kr_roof is not None and shares["bicgstab"] >= shares["gp_eval_tangent"]) else gp_roof

    cpu = None
    if snap is not None:
        cpu = cpu_baseline_step(w, *snap)

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": dict(workload_config(n, args.config), parallelism="replicas" if world > 1 else "single-gpu",
                          precond={0: "none", 1: "jacobi", 2: "block-jacobi-3x3", 3: "multigrid-vcycle"}[args.precond],
                          krylov_tol=args.krylov_tol, tangent="fp32 (fp64 where the local scale test fails)"
                          if args.fp32_tangent else "fp64",
                          initial_guess={"linear": "linear extrapolation of the last two solutions",
                                         "previous": "last solution"}[args.predictor],
                          mg_refresh=args.mg_refresh if args.precond == 3 else None),
           "s_per_load_step": t / args.steps, "clocks": clocks, "e2e": e2e,
           "roofline": dominant,
           "roofline_kernels": {"bicgstab": kr_roof, "spmv": spmv_roof, "gp_eval": gp_roof,
                                "elem_assemble": asm_roof},
           "region_shares": shares, "reference_choice_legs": legs, "tuned_linear_solver": tuned,
           "fp64_peak": {"value": fp64, "unit": "TFLOP/s", "probe": FP64_PROBE},
           "cpu_baseline": cpu,
           "regions_ms": {k: {"launches": v[0], "ms": v[1]} for k, v in regions.items()},
           "newton_iters_per_step": newton, "krylov_iters": krylov, "gp_passes": passes,
           "solves_dropped": dropped, "gpu_launches": None}
    out["gpu_launches"] = counter.launches
    if rank == 0 and world == 1 and args.config == "c1" and not args.no_sub_records:
        # the differentiation form on the same RVE, after the timed region, and the 10^3
        # copper single crystal and the 64^3 BCC24 polycrystal
        # over their whole load histories (10 and 30 steps: warm-up + timed), each in a
        # process of its own
        out["sub_records"] = {"c3_adjoint": adjoint_record(args, pkg, problem_mod, torch),
                              "c0_copper": sub_bench(["--config", "c0", "--warmup", "3", "--steps", "7"]),
                              "c2_bcc24": sub_bench(["--config", "c2", "--warmup", "3", "--steps", "27"])}
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def sub_bench(flags):
    """The JSON line of ``bench.py`` run with ``flags`` (and no CPU baseline, Jacobi legs or
    sub-records) in a child process."""
    cmd = [sys.executable, os.path.abspath(__file__), *flags, "--no-cpu-baseline", "--no-jacobi-leg",
           "--no-sub-records"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    if r.returncode != 0 or not lines:
        return {"error": f"exit {r.returncode}: {(r.stderr or r.stdout).strip().splitlines()[-1:]}"}
    return json.loads(lines[-1])


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
    """Forwards to the C ABI and counts the kernels its calls launch, from the sources:
    cpfem_bicgstab_ex is the persistent launch, plus the point preconditioner's set-up
    (precond 1, 2) and the two true-residual kernels (flags bit 0); cpfem_mg_setup is the
    level-0 block inverses, three directional Galerkin passes and a block inversion per
    coarse level, and two FP32 copies per level for the FP32 V-cycle; every other listed
    entry point launches one kernel."""
    LAUNCHES = {"cpfem_gp_eval": 1, "cpfem_elem_assemble": 1, "cpfem_elem_assemble_ex": 1, "cpfem_apply_dirichlet": 1, "cpfem_dot": 1,
                "cpfem_bc_initial_guess": 1, "cpfem_axpy": 1, "cpfem_spmv": 1, "cpfem_bicgstab": 2,
                "cpfem_bicgstab_ex": 2, "cpfem_cell_average": 1, "cpfem_segmented_dot": 1,
                "cpfem_bicgstab_batched": 2, "cpfem_gp_vjp": 1}

    def __init__(self, lib):
        self._lib = lib
        self.launches = 0
        self.counting = False

    @staticmethod
    def _count(name, a, k):
        if name == "cpfem_bicgstab_ex":
            o = a[4]._obj
            return 1 + (1 if o.precond in (1, 2) else 0) + (2 if o.flags & 1 else 0)
        if name == "cpfem_mg_setup":
            mg = a[0]._obj
            return 1 + 4 * (mg.num_levels - 1) + (2 * mg.num_levels if mg.precision == 1 else 0)
        return k

    def __getattr__(self, name):
        f = getattr(self._lib, name)
        k = self.LAUNCHES.get(name)
        if k is None and name != "cpfem_mg_setup":
            return f

        def call(*a):
            if self.counting:
                self.launches += self._count(name, a, k)
            return f(*a)
        return call


if __name__ == "__main__":
    main()
