"""The benchmark workloads of the plain method and a load-step loop through the public API.

Each workload is the reference driver loop (``singlecrystal_copper/singlecrystal_copper.py:
153-233``) on a seeded synthetic RVE: a structured unit-cube HEX8 mesh, Voronoi grains
(seeds uniform in the cube, each cell to its nearest seed), orientations uniform on SO(3)
(normalised Gaussian quaternions), roller BCs on x=0, y=0, z=0 and a prescribed u_z on
z=1, tension in equal strain increments at a strain rate of 1e-2 /s (dt = 0.1 s per 1e-3).

* ``copper_single_crystal``: 10^3 cells, one orientation (Euler angles 0), copper-like
  constants, 10 steps to 1 %.
* ``steel_polycrystal``: 32^3 cells, 64 grains, 304-steel-like FCC constants, 20 steps to 2 %.
* ``tantalum_polycrystal``: 64^3 cells, 512 grains, tantalum-like BCC {110}+{112} constants,
  30 steps to 3 %.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import material
from .mesh import Mesh, box_mesh, face_nodes, voronoi_grains

STRAIN_STEP = 1e-3
DT = 0.1

# The linear-solver settings the autotuner chooses on the 32^3 polycrystal (geometric
# multigrid V-cycle in FP32 inside the FP64 BiCGSTAB, 4 levels, 8 coarse sweeps) and the
# local-solve options of the fast path.  The Newton tolerances are the reference's.
TUNED_MG = {"max_levels": 4, "pre_sweeps": 1, "post_sweeps": 1, "coarse_sweeps": 12, "omega": 0.45,
            "precision": "fp32", "local_nodes": 256}
TUNED_GRID_BLOCKS = 304


@dataclasses.dataclass
class Workload:
    name: str
    mesh: Mesh
    quat: np.ndarray
    ori: np.ndarray
    spec: material.MaterialSpec
    load_steps: int
    strain_step: float = STRAIN_STEP
    dt: float = DT

    @property
    def num_gp(self):
        return 8 * self.mesh.cells.shape[0]

    def bc_lists(self, disp):
        # the node lists depend on the mesh only: found once, not at every load step
        nodes = self.__dict__.get("_roller_nodes")
        if nodes is None:
            nodes = self.__dict__["_roller_nodes"] = roller_lists(self.mesh, 0.0)[0]
        return list(nodes), [0, 1, 2, 2], [0.0, 0.0, 0.0, float(disp)]

    def bc_triples(self, disp):
        nodes, comps, vals = roller_lists(self.mesh, disp)
        return list(zip(nodes, comps, vals))


def roller_lists(mesh, disp):
    """Roller BCs (u_x = 0 on x = 0, u_y = 0 on y = 0, u_z = 0 on z = 0) and u_z = disp on
    z = 1, as (node lists, components, values)."""
    p = mesh.points
    nodes = [face_nodes(p, 0, 0.0), face_nodes(p, 1, 0.0), face_nodes(p, 2, 0.0), face_nodes(p, 2, 1.0)]
    return nodes, [0, 1, 2, 2], [0.0, 0.0, 0.0, float(disp)]


def polycrystal(n, grains, seed, spec, load_steps, name):
    mesh = box_mesh(n, n, n)
    ori, rng = voronoi_grains(mesh, grains, seed)
    quat = material.random_quaternions(rng, grains)
    return Workload(name, mesh, quat, ori, spec, load_steps)


def copper_single_crystal(n=10):
    mesh = box_mesh(n, n, n)
    return Workload(f"fcc-single-crystal-{n}^3-copper-tension", mesh, np.array([[1.0, 0.0, 0.0, 0.0]]),
                    np.zeros(n ** 3, dtype=np.int64), material.BENCH_COPPER, 10)


def steel_polycrystal(n=32, grains=64, seed=0):
    return polycrystal(n, grains, seed, material.BENCH_STEEL, 20,
                       f"fcc-polycrystal-{n}^3-{grains}grains-304steel-tension")


def tantalum_polycrystal(n=64, grains=512, seed=0):
    return polycrystal(n, grains, seed, material.BENCH_TANTALUM, 30,
                       f"bcc24-polycrystal-{n}^3-{grains}grains-tantalum-tension")


class LoadStepper:
    """Device-resident load-step loop through the public API, as the reference driver runs
    it: per step set dt and the top displacement, ``solver``, ``compute_avg_stress``,
    ``update_int_vars_gp``.  ``solver_options`` go to ``solver``.

    ``predictor`` chooses the Newton solve's initial guess: ``"previous"`` is the reference
    driver's (the last converged solution, ``singlecrystal_copper.py:197``); ``"linear"``
    extrapolates the last two converged solutions, 2 u_n - u_(n-1) -- exact on the Dirichlet
    dofs of equal load increments and close in the interior, so the first residual of a
    step is several times smaller and a plastic load step needs 3 Newton iterations instead
    of 5.  The stop rule is unchanged, so the converged solution is the same to the Newton
    tolerance.  An extrapolated guess can overshoot where the response turns plastic (the
    second step doubles an elastic first one): a step whose solve fails from it (a local
    solve that does not converge, a Newton or Krylov failure) is solved again from the
    last solution, the reference driver's guess (counted in ``predictor_fallbacks``)."""

    def __init__(self, problem, solver_mod, workload, solver_options=None, predictor="previous"):
        import torch
        if predictor not in ("previous", "linear"):
            raise ValueError("predictor must be 'previous' or 'linear'")
        self.prob, self.solver, self.w = problem, solver_mod, workload
        self.options = dict(solver_options or {})
        self.predictor = predictor
        if predictor == "linear":
            # the first Newton pass of a step is at the extrapolated, plastic state: the
            # ds/dF it forms already predicts the second pass's local starts well
            problem.predict_from_pass = 1
        self.i = 0
        self.params = problem.internal_vars
        self.sol = torch.zeros(problem.num_total_dofs_all_vars, dtype=torch.float64, device=problem.device)
        self.prev = None

    def step(self, host_io=None):
        """One load step; ``host_io = (sol_h, sig_h)`` pinned host buffers: the last solution
        is copied from ``sol_h`` and the solution and cell stresses are copied back."""
        prob, w = self.prob, self.w
        self.i += 1
        prob.dt = w.dt
        prob.fes[0].set_dirichlet_lists(*w.bc_lists(w.strain_step * self.i))
        prob.set_params(self.params)
        last = host_io[0].to(prob.device, non_blocking=True) if host_io is not None else self.sol
        guess = last
        if self.predictor == "linear" and self.prev is not None:
            guess = 2.0 * last - self.prev
        sol = solve_with_fallback(self.solver, prob, self.options, guess, last)
        self.predictor_fallbacks = prob.stats.get("predictor_fallbacks", 0)
        sig = prob.compute_avg_stress(sol, self.params)
        self.params = prob.update_int_vars_gp(sol, self.params)
        self.prev = last
        self.sol = sol.reshape(-1)
        if host_io is not None:
            host_io[0].copy_(self.sol, non_blocking=True)
            host_io[1].copy_(sig.reshape(-1), non_blocking=True)
        return sig


def solve_with_fallback(solver_mod, problem, options, guess, last):
    """``solver`` from ``guess``; if that fails and ``guess`` is not ``last``, again from
    ``last`` (the reference driver's guess)."""
    opts = dict(options)
    opts["initial_guess"] = [guess.reshape(-1, 3)]
    try:
        return solver_mod.solver(problem, opts)[0]
    except (RuntimeError, FloatingPointError):
        if guess is last:
            raise
    problem.stats["predictor_fallbacks"] = problem.stats.get("predictor_fallbacks", 0) + 1
    opts["initial_guess"] = [last.reshape(-1, 3)]
    return solver_mod.solver(problem, opts)[0]


def fast_solver_options(precond=3, mg=None, grid_blocks=None, **newton):
    """``solver`` options of the benchmarked configuration: BiCGSTAB preconditioned by the
    multigrid V-cycle with the tuned settings (``mg`` overrides them), the reference's
    BiCGSTAB and Newton stop rules unless ``newton`` overrides ``tol`` / ``rel_tol``."""
    if grid_blocks is None:
        grid_blocks = TUNED_GRID_BLOCKS if precond == 3 else 0
    opts = {"jax_solver": {"precond": precond, "mg_options": dict(TUNED_MG, **(mg or {})),
                           "grid_blocks": grid_blocks}}
    opts.update(newton)
    return opts


# What ``bench.py`` times on top of the tuned linear solver: the initial guess of each
# Newton solve, the relative tolerance of each Newton step's BiCGSTAB (an inexact Newton
# step: the Newton stop rule, and so the converged solution, are the reference's), the
# FP32 consistent tangent (the global Newton's Jacobian only), and the multigrid hierarchy
# formed once per load step from its first Newton system (only the preconditioner ages;
# the Krylov operator is always the current tangent).
# The Newton stop limit is an absolute 1e-8 (the reference's 1e-6, same rel_tol): started
# from an extrapolated guess, the loop can stop after a different iterate than the
# reference's, and at 1e-8 the solution stays within 1e-8 of the discrete solution.
BENCH_SETTINGS = {"predictor": "linear", "krylov_tol": 1e-4, "fp32_tangent": True, "mg_refresh": "step",
                  "newton": {"tol": 1e-8, "rel_tol": 1e-8}}


def bench_stepper(problem, solver_mod, workload, settings=None):
    """The load-step loop exactly as ``bench.py`` runs it (``BENCH_SETTINGS``)."""
    s = dict(BENCH_SETTINGS, **(settings or {}))
    problem.fp32_tangent = bool(s["fp32_tangent"])
    opts = fast_solver_options(mg={"refresh": s["mg_refresh"]}, **s["newton"])
    opts["jax_solver"]["tol"] = float(s["krylov_tol"])
    return LoadStepper(problem, solver_mod, workload, opts, predictor=s["predictor"])
