"""Autotuning of the linear-solve configuration on the problem at hand.

The multigrid-preconditioned BiCGSTAB has settings whose best values depend on the mesh
size, the material state and the GPU: the number of levels, the smoothing sweeps and
damping, and the grid size of the persistent launch (more blocks hide latency in the
SpMVs, fewer make each grid barrier cheaper).  ``tune_linear_solver`` times complete
solves of a real Newton system (CUDA events on the solve's stream, after one untimed
solve per configuration) with a coordinate search over those settings, and returns the
fastest configuration that converged.  Every candidate solves the same system to the
same stop rule, so the choice changes only the time, not the accuracy contract.  The V-cycle
may run in FP32 (the Krylov iteration stays FP64, so the stop rule is the same).  The
damping stays at or below 0.45: block-Jacobi smoothing of these tangents diverges near
0.7, and a tuned value must stay safe for the later, more plastic, Newton systems.
"""
from __future__ import annotations

import torch

from . import solver as _solver

DEFAULT = {"max_levels": 4, "pre_sweeps": 1, "post_sweeps": 1, "coarse_sweeps": 4, "omega": 0.45,
           "precision": "fp64", "local_nodes": 256, "grid_blocks": 0}
# the keys that go to CrystalPlasticity.multigrid (grid_blocks goes to the launch)
MG_KEYS = ("max_levels", "pre_sweeps", "post_sweeps", "coarse_sweeps", "omega", "precision", "local_nodes")
SEARCH = (("precision", ("fp64", "fp32")),
          ("omega", (0.35, 0.4, 0.45)),
          ("pre_sweeps", (1, 2)),
          ("post_sweeps", (0, 1, 2)),
          ("coarse_sweeps", (4, 8, 12)),
          ("max_levels", (3, 4, 5)),
          ("local_nodes", (256, 1024)),
          ("grid_blocks", (0, 76, 104, 152, 304)))


def _time_solve(problem, A, b, x0, cfg, reps, tol=1e-10):
    mg = {k: cfg[k] for k in MG_KEYS}
    _solver.bicgstab(problem, A, b, x0, precond=3, tol=tol, mg_options=mg, grid_blocks=cfg["grid_blocks"])
    best, its, ok = float("inf"), None, True
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        _, k, conv = _solver.bicgstab(problem, A, b, x0, precond=3, tol=tol, mg_options=mg,
                                      grid_blocks=cfg["grid_blocks"])
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
        its, ok = k, ok and conv
    return best, its, ok


def tune_linear_solver(problem, A, b, x0, reps=2, search=SEARCH, start=None, tol=1e-10):
    """Coordinate search over the multigrid / launch settings on the system A x = b, solved
    to the relative tolerance the caller will use (``tol``).
    Returns (best configuration dict, list of (configuration, ms, iterations))."""
    cfg = dict(DEFAULT if start is None else start)
    table = []
    ms, its, ok = _time_solve(problem, A, b, x0, cfg, reps, tol)
    table.append((dict(cfg), ms, its))
    best_ms = ms if ok else float("inf")
    for key, values in search:
        for v in values:
            if v == cfg[key]:
                continue
            trial = dict(cfg)
            trial[key] = v
            try:
                t_ms, t_its, t_ok = _time_solve(problem, A, b, x0, trial, reps, tol)
            except (ValueError, RuntimeError):
                continue
            table.append((dict(trial), t_ms, t_its))
            if t_ok and t_ms < best_ms:
                best_ms, cfg = t_ms, trial
    # leave the problem's hierarchy in the chosen configuration
    problem.multigrid(**{k: cfg[k] for k in MG_KEYS})
    return cfg, table
