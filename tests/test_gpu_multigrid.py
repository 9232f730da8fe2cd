"""Geometric-multigrid preconditioner (precond 3): the device Galerkin coarse operator
against P^T A P formed on the host from the assembled tangent, and multigrid-BiCGSTAB
solves and load steps against the Jacobi path and the oracle."""
import importlib

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from oracle import cpfem_oracle as O
from tests.common import gpu_problem, oracle_problem, roller_bcs

pytestmark = pytest.mark.gpu


def _block_matrix(layout, values):
    """Scalar CSR of a sliced-ELL node-block matrix (rows sorted)."""
    rowptr, cols, goff, _ = layout
    v = values.detach().cpu().numpy()
    n = rowptr.size - 1
    I, J, V = [], [], []
    for a in range(n):
        g, lane = a >> 5, a & 31
        for j in range(rowptr[a + 1] - rowptr[a]):
            b = cols[rowptr[a] + j]
            for r in range(3):
                for c in range(3):
                    I.append(3 * a + r)
                    J.append(3 * b + c)
                    V.append(v[9 * goff[g] + lane + 32 * (9 * j + 3 * r + c)])
    return sp.csr_array((V, (I, J)), shape=(3 * n, 3 * n))


def _prolong(dims):
    def p1(nf):
        nc = (nf - 1) // 2 + 1
        rows, cols, vals = [], [], []
        for i in range(nf):
            if i % 2 == 0:
                rows.append(i)
                cols.append(i // 2)
                vals.append(1.0)
            else:
                rows.extend([i, i])
                cols.extend([(i - 1) // 2, (i + 1) // 2])
                vals.extend([0.5, 0.5])
        return sp.csr_array((vals, (rows, cols)), shape=(nf, nc))
    Pn = sp.kron(sp.kron(p1(dims[2]), p1(dims[1])), p1(dims[0]))
    return sp.kron(Pn, sp.eye(3)).tocsr()


def _plastic_case(pkg, problem_mod, n=8, grains=4, strain=3e-3):
    spec = pkg.material.BENCH_STEEL
    mesh = pkg.box_mesh(n, n, n)
    ori, rng = pkg.mesh.voronoi_grains(mesh, grains, 2)
    quat = pkg.material.random_quaternions(rng, grains)
    bcs = roller_bcs(pkg.mesh, mesh.points, strain)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori, bcs)
    prob.dt = 0.1
    P = mesh.points
    u = np.zeros_like(P)
    u[:, 2] = strain * P[:, 2]
    u[:, :2] = -0.3 * strain * P[:, :2]
    return spec, mesh, quat, ori, bcs, prob, torch.tensor(u.reshape(-1), device="cuda")


def test_coarse_operator_is_galerkin_product(pkg, gpu):
    problem_mod, solver_mod = gpu
    _, mesh, _, _, _, prob, u = _plastic_case(pkg, problem_mod)
    res, A = solver_mod.newton_update_helper(prob, u)
    prob.mg_setup(A.values)
    assert [l[0] for l in prob.mg_levels][:3] == [9, 5, 3]
    A0 = A.to_scipy()
    free = np.ones(A0.shape[0])
    free[prob.fes[0].bc_dofs.cpu().numpy()] = 0.0
    P = sp.diags(free) @ _prolong(prob.mg_levels[0])
    A1 = (P.T @ A0 @ P).toarray()
    D1 = _block_matrix(prob.mg_layouts[1], prob.mg_layouts[1][3]).toarray()
    assert np.abs(D1 - A1).max() / np.abs(A1).max() < 1e-13
    P2 = _prolong(prob.mg_levels[1])
    A2 = (P2.T @ sp.csr_array(A1) @ P2).toarray()
    D2 = _block_matrix(prob.mg_layouts[2], prob.mg_layouts[2][3]).toarray()
    assert np.abs(D2 - A2).max() / np.abs(A2).max() < 1e-13


def test_multigrid_bicgstab_solves_the_tangent(pkg, gpu):
    problem_mod, solver_mod = gpu
    _, _, _, _, _, prob, u = _plastic_case(pkg, problem_mod, n=16)
    res, A = solver_mod.newton_update_helper(prob, u)
    x0 = solver_mod.initial_increment(prob, u)
    xj, kj, okj = solver_mod.bicgstab(prob, A, -res, x0, precond=1)
    xm, km, okm = solver_mod.bicgstab(prob, A, -res, x0, precond=3)
    assert okj and okm and 0 < km < kj / 4, (kj, km)
    assert float((xm - xj).abs().max() / xj.abs().max()) < 1e-8
    r = A.matvec(xm) + res
    assert float(r.norm()) <= 1e-10 * max(float(res.norm()), 1.0) * 10


@pytest.mark.parametrize("local_nodes", [256, 1024])
def test_fp32_vcycle_solves_the_tangent(pkg, gpu, local_nodes):
    """The single-precision V-cycle (local_nodes 1024 also smooths the 9^3 level inside one
    block): the FP64 Krylov iteration still meets the FP64 stop rule, and the solution
    agrees with the Jacobi and FP64-multigrid solves."""
    problem_mod, solver_mod = gpu
    _, _, _, _, _, prob, u = _plastic_case(pkg, problem_mod, n=16)
    res, A = solver_mod.newton_update_helper(prob, u)
    x0 = solver_mod.initial_increment(prob, u)
    xj, kj, okj = solver_mod.bicgstab(prob, A, -res, x0, precond=1)
    xd, kd, okd = solver_mod.bicgstab(prob, A, -res, x0, precond=3, mg_options={"precision": "fp64"})
    xs, ks, oks = solver_mod.bicgstab(prob, A, -res, x0, precond=3,
                                      mg_options={"precision": "fp32", "local_nodes": local_nodes})
    assert prob._mg.precision == 1 and prob._mg.local_nodes == local_nodes
    assert okj and okd and oks and 0 < ks <= kd + 3, (kj, kd, ks)
    assert float((xs - xj).abs().max() / xj.abs().max()) < 1e-8
    r = A.matvec(xs) + res
    assert float(r.norm()) <= 1e-10 * max(float(res.norm()), 1.0) * 10
    # back to FP64 on the same hierarchy: the same iterates as the first FP64 solve
    xd2, kd2, _ = solver_mod.bicgstab(prob, A, -res, x0, precond=3,
                                      mg_options={"precision": "fp64", "local_nodes": 256})
    assert kd2 == kd and torch.equal(xd2, xd)


def test_fp32_vcycle_transposed_solve(pkg, gpu):
    problem_mod, solver_mod = gpu
    _, _, _, _, _, prob, u = _plastic_case(pkg, problem_mod, n=16)
    res, A = solver_mod.newton_update_helper(prob, u)
    f = torch.randn_like(res)
    f[prob.fes[0].bc_dofs.long()] = 0.0
    x0 = torch.zeros_like(res)
    xj, kj, okj = solver_mod.bicgstab(prob, A.T, f, x0, precond=1)
    xs, ks, oks = solver_mod.bicgstab(prob, A.T, f, x0, precond=3, mg_options={"precision": "fp32"})
    assert okj and oks and 0 < ks < kj / 4, (kj, ks)
    assert float((xs - xj).abs().max() / xj.abs().max()) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_load_steps_with_multigrid_match_oracle(pkg, gpu, precision):
    """Three tension steps of a 4^3, 4-grain polycrystal with the multigrid-preconditioned
    linear solve (FP64 or FP32 V-cycle): per-cell stress and u against the oracle (Jacobi
    BiCGSTAB)."""
    problem_mod, solver_mod = gpu
    spec = pkg.material.BENCH_STEEL
    mesh = pkg.box_mesh(4, 4, 4)
    ori, rng = pkg.mesh.voronoi_grains(mesh, 4, 0)
    quat = pkg.material.random_quaternions(rng, 4)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori)
    orc = oracle_problem(spec, mesh, quat, ori)
    disps, ts = np.linspace(0, 3e-3, 4), np.linspace(0, 0.3, 4)
    bcf = lambda d: roller_bcs(pkg.mesh, mesh.points, d)
    sol = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64, device="cuda")
    params = prob.internal_vars
    out = []
    for i in range(3):
        prob.dt = float(ts[i + 1] - ts[i])
        bcs = bcf(float(disps[i + 1]))
        prob.fes[0].set_dirichlet_lists([b[0] for b in bcs], [b[1] for b in bcs], [b[2] for b in bcs])
        prob.set_params(params)
        sol = solver_mod.solver(prob, {"jax_solver": {"precond": "mg", "mg_options": {"precision": precision}},
                                       "tol": 1e-9, "rel_tol": 1e-12,
                                       "initial_guess": [sol.reshape(-1, 3)]})[0].reshape(-1)
        out.append(prob.compute_avg_stress(sol.reshape(-1, 3), params).cpu().numpy())
        params = prob.update_int_vars_gp(sol.reshape(-1, 3), params)
    s_o, u_o = O.run_load_steps(orc, disps, ts, bcf, {"tol": 1e-9, "rel_tol": 1e-12})
    s = np.array(out)
    assert np.abs(s - s_o).max() / np.abs(s_o).max() < 1e-8
    assert float(np.abs(sol.cpu().numpy() - u_o).max() / np.abs(u_o).max()) < 1e-8


def test_autotuner_picks_a_converging_configuration(pkg, gpu):
    problem_mod, solver_mod = gpu
    tuning = importlib.import_module("jax-cpfem_gb300.tuning")
    _, _, _, _, _, prob, u = _plastic_case(pkg, problem_mod, n=8)
    res, A = solver_mod.newton_update_helper(prob, u)
    x0 = solver_mod.initial_increment(prob, u).clone()
    cfg, table = tuning.tune_linear_solver(prob, A, -res, x0, reps=1,
                                           search=(("omega", (0.4, 0.5)), ("grid_blocks", (0, 8))))
    assert len(table) >= 3 and set(cfg) == set(tuning.DEFAULT)
    mg = {k: cfg[k] for k in tuning.MG_KEYS}
    x, k, ok = solver_mod.bicgstab(prob, A, -res, x0, precond=3, mg_options=mg, grid_blocks=cfg["grid_blocks"])
    xj, kj, okj = solver_mod.bicgstab(prob, A, -res, x0, precond=1)
    assert ok and okj and float((x - xj).abs().max() / xj.abs().max()) < 1e-8


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_golden_case4_with_multigrid(pkg, gpu, precision):
    """The first 20 steps of calibration_case4 scenario 0 (20^3 Neper voxels, corner BCs with
    a free rigid rotation about z) with the multigrid-preconditioned solve: mean sigma_zz
    against the reference's curve.  The system is near-singular: an FP32 V-cycle fails on
    it, and the solver re-solves with the FP64 one."""
    import os
    problem_mod, solver_mod = gpu
    gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))
    L = 0.0295
    mesh = pkg.box_mesh(20, 20, 20, L, L, L)
    prob = gpu_problem(pkg, problem_mod, pkg.material.CALIB_CASE4, mesh, gold["case4_quat"],
                       gold["case4_grain"].astype(np.int64))
    c = pkg.mesh.corner_nodes(mesh.points, (0.0, 0.0, 0.0))
    bot, top = pkg.mesh.face_nodes(mesh.points, 2, 0.0), pkg.mesh.face_nodes(mesh.points, 2, L)
    disps, ts = np.linspace(0, 0.025 * L, 81), np.linspace(0, 2.5, 81)
    sol = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64, device="cuda")
    params = prob.internal_vars
    out = []
    for i in range(20):
        prob.dt = float(ts[i + 1] - ts[i])
        prob.fes[0].set_dirichlet_lists([c, c, bot, top], [0, 1, 2, 2], [0.0, 0.0, 0.0, float(disps[i + 1])])
        prob.set_params(params)
        sol = solver_mod.solver(prob, {"jax_solver": {"precond": "mg", "restart_on_breakdown": True,
                                                      "mg_options": {"precision": precision}},
                                       "tol": 1e-7, "line_search_flag": True,
                                       "initial_guess": [sol.reshape(-1, 3)]})[0].reshape(-1)
        out.append(float(prob.compute_avg_stress(sol.reshape(-1, 3), params)[:, 2, 2].mean()))
        params = prob.update_int_vars_gp(sol.reshape(-1, 3), params)
    rel = np.abs((np.array(out) - gold["case4_szz"][:20]) / gold["case4_szz"][:20])
    assert rel.max() < 1e-5, rel
    if precision == "fp32":
        assert prob.stats.get("mg_fp64_fallbacks", 0) >= 1 and prob.mg_fp64_only


def test_transposed_multigrid_solve(pkg, gpu):
    """The adjoint's transposed system A^T mu = f with the same hierarchy: against the
    Jacobi-preconditioned transposed solve."""
    problem_mod, solver_mod = gpu
    _, _, _, _, _, prob, u = _plastic_case(pkg, problem_mod, n=16)
    res, A = solver_mod.newton_update_helper(prob, u)
    f = torch.randn_like(res)
    f[prob.fes[0].bc_dofs.long()] = 0.0
    x0 = torch.zeros_like(res)
    xj, kj, okj = solver_mod.bicgstab(prob, A.T, f, x0, precond=1)
    xm, km, okm = solver_mod.bicgstab(prob, A.T, f, x0, precond=3)
    assert okj and okm and 0 < km < kj / 4, (kj, km)
    assert float((xm - xj).abs().max() / xj.abs().max()) < 1e-8
    r = A.T.matvec(xm) - f
    assert float(r.norm()) <= 1e-9 * max(float(f.norm()), 1.0)
