"""GPU vs oracle at the benchmark configurations, with the benchmark's solver settings.

The GPU side runs exactly what ``bench.py`` times: the multigrid-preconditioned BiCGSTAB
with the FP32 V-cycle and the tuned settings, warm-started local Newton with FP32 local
directions, no tangent on the last Newton iterate, and the reference's Newton stop rule
(tol 1e-6, rel_tol 1e-8, ``crystal_plasticity_OR_design/solver.py:384-385``).  The oracle
runs the reference's algorithm (Jacobi BiCGSTAB, local Newton from S = 0) on the same
seeded mesh, orientations and load.  Compared per load step: the volume-averaged Cauchy
stress and the nodal displacements; after the last step: Fp^-1 and g at every GP.

* copper single crystal, 10^3 cells, all 10 load steps;
* 304-steel-like polycrystal, 32^3 cells, 64 grains, the first 2 load steps (the compiled
  oracle on all host cores);
* tantalum-like BCC {110}+{112} polycrystal on a reduced 16^3 box with 24 grains (the 64^3
  workload is beyond what the oracle finishes in a test), 4 load steps.
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


def _gpu_history(pkg, problem_mod, solver_mod, w, steps, opts):
    W = importlib.import_module("jax-cpfem_gb300.workloads")
    prob = problem_mod.CrystalPlasticity(w.mesh, additional_info=(w.quat, w.ori), material=w.spec)
    st = W.LoadStepper(prob, solver_mod, w, opts)
    vol = prob.fes[0].JxW.sum(1)
    sig, us, newton = [], [], []
    for _ in range(steps):
        s = st.step()
        sig.append((torch.einsum("eij,e->ij", s, vol) / vol.sum()).cpu().numpy())
        us.append(st.sol.cpu().numpy())
        newton.append(prob.stats["newton_iters"])
    return np.array(sig), np.array(us), [p.cpu().numpy() for p in st.params[:3]], newton, prob


def _compare(pkg, gpu, w, steps, **newton):
    problem_mod, solver_mod = gpu
    W = importlib.import_module("jax-cpfem_gb300.workloads")
    opts = W.fast_solver_options(**newton)
    sig, us, state, nit, prob = _gpu_history(pkg, problem_mod, solver_mod, w, steps, opts)
    from oracle import coracle
    coracle.set_threads(os.cpu_count() or 1)
    orc = fast_oracle_problem(w.spec, w.mesh, w.quat, w.ori)
    oracle_opts = {k: v for k, v in newton.items() if k in ("tol", "rel_tol")}
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
    print(f"\n{w.name} steps={steps} newton gpu {nit} oracle {[i['newton_iters'] for i in info]} "
          f"opts {oracle_opts}: " + " ".join(f"{k}={v:.2e}" for k, v in err.items()))
    return err


def _check(err):
    for k in ("sigma", "u", "Fp_inv", "g"):
        assert err[k] < TOL, (k, err)


def test_copper_single_crystal_all_steps(pkg, gpu):
    W = importlib.import_module("jax-cpfem_gb300.workloads")
    w = W.copper_single_crystal()
    _check(_compare(pkg, gpu, w, w.load_steps))


def test_steel_polycrystal_32_first_steps(pkg, gpu):
    W = importlib.import_module("jax-cpfem_gb300.workloads")
    _check(_compare(pkg, gpu, W.steel_polycrystal(), 2))


def test_tantalum_bcc24_reduced(pkg, gpu):
    W = importlib.import_module("jax-cpfem_gb300.workloads")
    _check(_compare(pkg, gpu, W.tantalum_polycrystal(n=16, grains=24), 4))
