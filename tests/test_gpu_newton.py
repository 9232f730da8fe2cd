"""The global Newton loop's skipped tangent on the last iterate: the residual histories,
iteration counts and solutions equal those of the loop that forms every tangent, also when
every prediction is forced (so each iterate takes the residual-only pass first and the
tangent pass after a misprediction)."""
import importlib

import numpy as np
import pytest
import torch

from tests.common import gpu_problem, roller_bcs

pytestmark = pytest.mark.gpu


def _run(pkg, problem_mod, solver_mod, skip, steps=3):
    spec = pkg.material.BENCH_STEEL
    mesh = pkg.box_mesh(4, 4, 4)
    ori, rng = pkg.mesh.voronoi_grains(mesh, 4, 7)
    quat = pkg.material.random_quaternions(rng, 4)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori)
    prob.skip_final_tangent = skip
    sol = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64, device="cuda")
    params = prob.internal_vars
    hist, sig = [], []
    for i in range(steps):
        prob.dt = 0.1
        bcs = roller_bcs(pkg.mesh, mesh.points, 1e-3 * (i + 1))
        prob.fes[0].set_dirichlet_lists([b[0] for b in bcs], [b[1] for b in bcs], [b[2] for b in bcs])
        prob.set_params(params)
        sol = solver_mod.solver(prob, {"jax_solver": {}, "initial_guess": [sol.reshape(-1, 3)]})[0].reshape(-1)
        hist.append(list(prob.stats["res_history"]))
        sig.append(prob.compute_avg_stress(sol.reshape(-1, 3), params).cpu().numpy())
        params = prob.update_int_vars_gp(sol.reshape(-1, 3), params)
    return prob, hist, np.array(sig), sol.cpu().numpy()


def test_skipped_final_tangent_keeps_the_newton_path(pkg, gpu):
    problem_mod, solver_mod = gpu
    _, h0, s0, u0 = _run(pkg, problem_mod, solver_mod, skip=False)
    prob, h1, s1, u1 = _run(pkg, problem_mod, solver_mod, skip=True)
    assert [len(h) for h in h1] == [len(h) for h in h0]
    for a, b in zip(h0, h1):
        assert np.allclose(a, b, rtol=1e-9, atol=0.0)
    assert np.abs(s1 - s0).max() / np.abs(s0).max() < 1e-12
    assert np.abs(u1 - u0).max() / np.abs(u0).max() < 1e-12
    assert prob.stats.get("final_tangent_skipped", 0) >= 1


def test_mispredicted_final_tangent_recovers(pkg, gpu, monkeypatch):
    problem_mod, solver_mod = gpu
    _, h0, s0, u0 = _run(pkg, problem_mod, solver_mod, skip=False)
    monkeypatch.setattr(solver_mod, "_expect_converged", lambda history, limit: True)
    prob, h1, s1, u1 = _run(pkg, problem_mod, solver_mod, skip=True)
    assert prob.stats.get("final_tangent_mispredicted", 0) >= 1
    assert [len(h) for h in h1] == [len(h) for h in h0]
    for a, b in zip(h0, h1):
        assert np.allclose(a, b, rtol=1e-9, atol=0.0)
    assert np.abs(u1 - u0).max() / np.abs(u0).max() < 1e-12
