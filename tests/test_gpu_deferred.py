"""The Newton loop's deferred Krylov checks: each iteration's BiCGSTAB report is read with
the next residual norm (and the next solve may be queued before that read), and an
iteration whose solve fails the check is redone with a checked solve.  The deferred loop
must give the checked loop's iterates exactly."""
import importlib
import os

import numpy as np
import pytest
import torch

from tests.common import gpu_problem

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


def _history(stepper, steps):
    sig, sols = [], []
    for _ in range(steps):
        s = stepper.step()
        sig.append(s.cpu().numpy())
        sols.append(stepper.sol.cpu().numpy())
    return np.array(sig), np.array(sols)


def test_deferred_checks_give_the_checked_iterates(pkg, gpu):
    """The benchmark path on the 10^3 copper crystal, 4 load steps: deferred with the next
    solve queued ahead of each norm read, deferred without it, and checked -- bitwise the
    same stresses and solutions, the same Newton and Krylov counts."""
    problem_mod, solver_mod = gpu
    W = importlib.import_module("jax-cpfem_gb300.workloads")
    out = []
    for defer, ahead in ((True, True), (True, False), (False, False)):
        w = W.copper_single_crystal()
        prob = problem_mod.CrystalPlasticity(w.mesh, additional_info=(w.quat, w.ori), material=w.spec)
        prob.defer_krylov_checks = defer
        prob.queue_next_solve = ahead
        st = W.bench_stepper(prob, solver_mod, w)
        sig, sols = _history(st, 4)
        out.append((sig, sols, list(prob.stats["krylov_iters"]), prob.stats.get("deferred_redone", 0)))
    s0, u0, k0, _ = out[0]
    for s, u, k, r in out:
        assert r == 0 and k == k0
        assert np.array_equal(s, s0) and np.array_equal(u, u0)


def test_deferred_fp32_failure_is_redone(pkg, gpu):
    """Calibration case 4 (corner BCs leave the rigid rotation about z free) with the FP32
    V-cycle requested: the FP32 solve fails its check on this near-singular system, which a
    deferred loop only learns at the next synchronisation; the iteration is redone with the
    FP64 V-cycle and the load steps equal the checked loop's."""
    problem_mod, solver_mod = gpu
    L = 0.0295
    out = []
    for defer in (True, False):   # deferred (with the next solve queued ahead) and checked
        mesh = pkg.box_mesh(20, 20, 20, L, L, L)
        prob = gpu_problem(pkg, problem_mod, pkg.material.CALIB_CASE4, mesh, GOLD["case4_quat"],
                           GOLD["case4_grain"].astype(np.int64))
        prob.defer_krylov_checks = defer
        c = pkg.mesh.corner_nodes(mesh.points, (0.0, 0.0, 0.0))
        bot, top = pkg.mesh.face_nodes(mesh.points, 2, 0.0), pkg.mesh.face_nodes(mesh.points, 2, L)
        disps, ts = np.linspace(0, 0.025 * L, 81), np.linspace(0, 2.5, 81)
        sol = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64, device="cuda")
        params = prob.internal_vars
        szz = []
        for i in range(6):
            prob.dt = float(ts[i + 1] - ts[i])
            prob.fes[0].set_dirichlet_lists([c, c, bot, top], [0, 1, 2, 2], [0.0, 0.0, 0.0, float(disps[i + 1])])
            prob.set_params(params)
            sol = solver_mod.solver(prob, {"jax_solver": {"precond": "mg", "restart_on_breakdown": True,
                                                          "mg_options": {"precision": "fp32"}},
                                           "tol": 1e-7, "initial_guess": [sol.reshape(-1, 3)]})[0].reshape(-1)
            szz.append(float(prob.compute_avg_stress(sol.reshape(-1, 3), params)[:, 2, 2].mean()))
            params = prob.update_int_vars_gp(sol.reshape(-1, 3), params)
        out.append((np.array(szz), sol.cpu().numpy(), prob.stats.get("mg_fp64_fallbacks", 0),
                    prob.stats.get("deferred_redone", 0)))
    (s1, u1, f1, r1), (s2, u2, f2, r2) = out
    assert f1 >= 1 and f2 >= 1 and r1 >= 1 and r2 == 0
    assert np.array_equal(s1, s2) and np.array_equal(u1, u2)
