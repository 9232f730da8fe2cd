"""Warm-started local Newton (each GP starts from its last converged S, moved to first
order along F, instead of S = 0): the abandoned warm start reproduces the S = 0 solve bit
for bit, warm and predicted starts converge to the same root, and load steps with and
without them agree and match the oracle."""
import numpy as np
import pytest
import torch

from oracle import cpfem_oracle as O
from tests.common import gpu_problem, oracle_problem, roller_bcs

pytestmark = pytest.mark.gpu


def _case(pkg, problem_mod, n=6, grains=4, strain=3e-3):
    spec = pkg.material.BENCH_STEEL
    mesh = pkg.box_mesh(n, n, n)
    ori, rng = pkg.mesh.voronoi_grains(mesh, grains, 5)
    quat = pkg.material.random_quaternions(rng, grains)
    bcs = roller_bcs(pkg.mesh, mesh.points, strain)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori, bcs)
    prob.dt = 0.1
    P = mesh.points
    u = np.zeros_like(P)
    u[:, 2] = strain * P[:, 2]
    u[:, :2] = -0.3 * strain * P[:, :2]
    return spec, mesh, quat, ori, prob, torch.tensor(u.reshape(-1), device="cuda")


def _pass(prob, u):
    prob.timing = True          # the pass then records every GP's local iteration count
    res, values, status = prob.assemble(u)
    assert int(status.item()) == 0
    return res.clone(), values.clone(), prob._bufs["iters"].clone()


def test_abandoned_warm_start_is_the_cold_solve(pkg, gpu):
    """A non-finite warm start is abandoned at once: every output equals the S = 0 solve
    exactly, with one extra step counted."""
    problem_mod, _ = gpu
    _, _, _, _, prob, u = _case(pkg, problem_mod)
    prob.warm_start_local = False
    r0, v0, i0 = _pass(prob, u)
    prob.warm_start_local = True
    prob._warm().fill_(float("nan"))
    r1, v1, i1 = _pass(prob, u)
    assert torch.equal(r1, r0) and torch.equal(v1, v0)
    assert torch.equal(i1, i0 + 1)
    assert bool(torch.isfinite(prob._warm()).all())


def test_warm_start_converges_to_the_same_root(pkg, gpu):
    problem_mod, _ = gpu
    _, _, _, _, prob, u = _case(pkg, problem_mod)
    prob.warm_start_local = True
    prob.reset_local_start()
    _pass(prob, u)                      # seeds the warm start
    u2 = u * (1.0 + 2e-3)
    rw, vw, iw = _pass(prob, u2)
    prob.warm_start_local = False
    rc, vc, ic = _pass(prob, u2)
    assert float((rw - rc).abs().max() / rc.abs().max()) < 1e-10
    assert float((vw - vc).abs().max() / vc.abs().max()) < 1e-9
    assert float(iw.double().mean()) < 0.6 * float(ic.double().mean()), (iw.double().mean(), ic.double().mean())


def test_linear_predictor_cuts_local_iterations(pkg, gpu):
    """Starting at s_warm + ds/dF (F - F_warm) instead of at s_warm: the same root, fewer
    local iterations."""
    problem_mod, _ = gpu
    _, _, _, _, prob, u = _case(pkg, problem_mod)
    prob.reset_local_start()
    _pass(prob, u)                      # s_warm, its F and ds/dF at u
    _pass(prob, u)                      # (the prediction is used from the third tangent pass)
    saved = {k: prob._bufs[k].clone() for k in ("s_warm", "s_dsdf", "s_f")}
    u2 = u * (1.0 + 2e-2)
    rp, vp, ip = _pass(prob, u2)
    for k, v in saved.items():
        prob._bufs[k].copy_(v)
    prob.predict_local = False
    rw, vw, iw = _pass(prob, u2)
    assert float((rp - rw).abs().max() / rw.abs().max()) < 1e-10
    assert float((vp - vw).abs().max() / vw.abs().max()) < 1e-9
    assert float(ip.double().mean()) < float(iw.double().mean()), (ip.double().mean(), iw.double().mean())


def test_load_steps_with_warm_start_match_cold_and_oracle(pkg, gpu):
    problem_mod, solver_mod = gpu
    spec = pkg.material.BENCH_STEEL
    mesh = pkg.box_mesh(4, 4, 4)
    ori, rng = pkg.mesh.voronoi_grains(mesh, 4, 3)
    quat = pkg.material.random_quaternions(rng, 4)
    disps, ts = np.linspace(0, 4e-3, 5), np.linspace(0, 0.4, 5)
    bcf = lambda d: roller_bcs(pkg.mesh, mesh.points, d)
    runs = {}
    for warm in (True, False):
        prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori)
        prob.warm_start_local = warm
        sol = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64, device="cuda")
        params = prob.internal_vars
        out = []
        for i in range(4):
            prob.dt = float(ts[i + 1] - ts[i])
            bcs = bcf(float(disps[i + 1]))
            prob.fes[0].set_dirichlet_lists([b[0] for b in bcs], [b[1] for b in bcs], [b[2] for b in bcs])
            prob.set_params(params)
            sol = solver_mod.solver(prob, {"jax_solver": {}, "tol": 1e-9, "rel_tol": 1e-12,
                                           "initial_guess": [sol.reshape(-1, 3)]})[0].reshape(-1)
            out.append(prob.compute_avg_stress(sol.reshape(-1, 3), params).cpu().numpy())
            params = prob.update_int_vars_gp(sol.reshape(-1, 3), params)
        runs[warm] = (np.array(out), sol.cpu().numpy())
    sw, uw = runs[True]
    sc, uc = runs[False]
    assert np.abs(sw - sc).max() / np.abs(sc).max() < 1e-10
    assert np.abs(uw - uc).max() / np.abs(uc).max() < 1e-10
    orc = oracle_problem(spec, mesh, quat, ori)
    s_o, u_o = O.run_load_steps(orc, disps, ts, bcf, {"tol": 1e-9, "rel_tol": 1e-12})
    assert np.abs(sw - s_o).max() / np.abs(s_o).max() < 1e-8
    assert np.abs(uw - u_o).max() / np.abs(u_o).max() < 1e-8


def test_fp32_local_newton_direction_converges_to_the_same_root(pkg, gpu):
    """Newton directions from the FP32 local Jacobian (the residual, stop test and tangent in
    FP64): the pass agrees with the FP64-direction pass to the local tolerance, at about the
    same iteration counts."""
    problem_mod, _ = gpu
    _, _, _, _, prob, u = _case(pkg, problem_mod)
    prob.warm_start_local = False
    prob.fp32_local_jacobian = False
    r64, v64, i64 = _pass(prob, u)
    prob.fp32_local_jacobian = True
    r32, v32, i32 = _pass(prob, u)
    assert float((r32 - r64).abs().max() / r64.abs().max()) < 1e-10
    assert float((v32 - v64).abs().max() / v64.abs().max()) < 1e-9
    assert float(i32.double().mean()) <= float(i64.double().mean()) + 0.5, (i32.double().mean(), i64.double().mean())


def test_ordered_pass_gives_the_same_outputs(pkg, gpu):
    """The optional evaluation order (GPs heaviest first by their previous local-Newton
    counts) changes which thread evaluates a GP, not its result: bitwise equal outputs."""
    problem_mod, _ = gpu
    _, _, _, _, prob, u = _case(pkg, problem_mod)
    prob.warm_start_local = False
    prob.sort_gps = False
    r0, v0, i0 = _pass(prob, u)
    prob.sort_gps = True
    _pass(prob, u)                      # forms the order from this pass's counts
    assert "gp_order" in prob._bufs
    r1, v1, i1 = _pass(prob, u)         # evaluated in that order
    assert torch.equal(r1, r0) and torch.equal(v1, v0) and torch.equal(i1, i0)
