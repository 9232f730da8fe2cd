"""GPU vs oracle at the benchmark configurations, with the benchmark's solver settings.

The GPU side runs what ``bench.py`` times (``workloads.BENCH_SETTINGS``): the multigrid-
preconditioned BiCGSTAB with the FP32 V-cycle and the tuned settings, warm-started local
Newton with FP32 local directions, the FP32 consistent tangent, no tangent on the last
Newton iterate, each step's Newton solve started from the linear extrapolation of the
last two solutions, an inexact Krylov solve per Newton step, and the reference's Newton
stop rule (tol 1e-6, rel_tol 1e-8, ``crystal_plasticity_OR_design/solver.py:384-385``).
The oracle runs the reference's algorithm (Jacobi BiCGSTAB to 1e-10, local Newton from
S = 0, each step started from the last solution) on the same seeded mesh, orientations
and load.  Compared per load step: the volume-averaged Cauchy stress and the nodal
displacements; after the last step: Fp^-1 and g at every GP.

Two comparisons per configuration:

* same path: the GPU started from the last solution like the oracle, both at the
  reference's tolerances -- both Newton loops take the same iterates, so the results
  agree far below 1e-8 and the comparison is sharp;
* benchmark path: the GPU exactly as benchmarked against the oracle converged far below
  the reference's tolerances (tol 1e-9, rel_tol 1e-12), i.e. the discrete solution
  itself.  The benchmark path reaches a different Newton iterate, so it is compared with
  the solution both loops approximate; two loops stopped at the reference's loose
  tolerance after different iterates differ by that tolerance's effect (~1e-8 in u), not
  by anything in the method.

Configurations: copper single crystal 10^3, all 10 load steps; 304-steel-like
polycrystal 32^3 with 64 grains, the first 3 load steps (the compiled oracle on all host
cores); tantalum-like BCC {110}+{112} polycrystal on a reduced 16^3 box with 24 grains (the
64^3 workload is beyond what the oracle finishes in a test), 4 load steps.
"""
import importlib
import os

import numpy as np
import pytest
import torch

from tests.common import fast_oracle_problem, oracle_history

pytestmark = pytest.mark.gpu

# relative to each field's magnitude over the compared steps
TOL = 1e-8
TIGHT = {"tol": 1e-9, "rel_tol": 1e-12}


def _workload(name):
    W = importlib.import_module("jax-cpfem_gb300.workloads")
    return {"copper": (W.copper_single_crystal(), 10), "steel32": (W.steel_polycrystal(), 3),
            "tantalum16": (W.tantalum_polycrystal(n=16, grains=24), 4)}[name]


def _gpu_history(problem_mod, solver_mod, w, steps, bench_path):
    W = importlib.import_module("jax-cpfem_gb300.workloads")
    prob = problem_mod.CrystalPlasticity(w.mesh, additional_info=(w.quat, w.ori), material=w.spec)
    st = W.bench_stepper(prob, solver_mod, w) if bench_path else \
        W.LoadStepper(prob, solver_mod, w, W.fast_solver_options(), predictor="previous")
    vol = prob.fes[0].JxW.sum(1)
    sig, us, newton = [], [], []
    for _ in range(steps):
        s = st.step()
        sig.append((torch.einsum("eij,e->ij", s, vol) / vol.sum()).cpu().numpy())
        us.append(st.sol.cpu().numpy())
        newton.append(prob.stats["newton_iters"])
    return np.array(sig), np.array(us), [p.cpu().numpy() for p in st.params[:3]], newton


def _compare(gpu, name, bench_path):
    problem_mod, solver_mod = gpu
    w, steps = _workload(name)
    sig, us, state, nit = _gpu_history(problem_mod, solver_mod, w, steps, bench_path)
    from oracle import coracle
    coracle.set_threads(os.cpu_count() or 1)
    orc = fast_oracle_problem(w.spec, w.mesh, w.quat, w.ori)
    oracle_opts = TIGHT if bench_path else {}
    sig_o, us_o, params_o, info = oracle_history(orc, w, steps, oracle_opts)
    g0 = w.spec.gss_initial
    err = {
        "sigma": float(np.abs(sig - sig_o).max() / np.abs(sig_o).max()),
        "u": float(np.abs(us - us_o).max() / np.abs(us_o).max()),
        "Fp_inv": float(np.abs(state[0] - params_o[0]).max() / np.abs(params_o[0]).max()),
        "g": float(np.abs(state[1] - params_o[1]).max() / np.abs(params_o[1]).max()),
        # the same differences against the plastic parts alone (stricter)
        "Fp_inv_vs_plastic": float(np.abs(state[0] - params_o[0]).max() /
                                   np.abs(params_o[0] - np.eye(3)).max()),
        "g_vs_hardening": float(np.abs(state[1] - params_o[1]).max() / np.abs(params_o[1] - g0).max()),
    }
    print(f"\n{w.name} steps={steps} {'bench path vs converged oracle' if bench_path else 'same path'}: "
          f"newton gpu {nit} oracle {[i['newton_iters'] for i in info]}: "
          + " ".join(f"{k}={v:.2e}" for k, v in err.items()))
    for k in ("sigma", "u", "Fp_inv", "g"):
        assert err[k] < TOL, (k, err)
    return err


@pytest.mark.parametrize("name", ["copper", "steel32", "tantalum16"])
def test_same_path_at_reference_tolerances(gpu, name):
    _compare(gpu, name, bench_path=False)


@pytest.mark.parametrize("name", ["copper", "steel32", "tantalum16"])
def test_bench_path_against_converged_oracle(gpu, name):
    _compare(gpu, name, bench_path=True)
