"""GPU parity: the sm_103a kernels (through the C ABI) against the CPU oracle and the
reference's golden curves.  Tolerances are relative to the largest entry compared."""
import os

import numpy as np
import pytest
import torch

from oracle import cpfem_oracle as O
from tests.common import corner_bcs, gpu_problem, oracle_problem, random_gp_inputs, roller_bcs

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


def _rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().numpy() if torch.is_tensor(b) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("spec_name", ["BENCH_COPPER", "BENCH_TANTALUM", "CALIB_CASE4"])
def test_gp_update_matches_oracle(pkg, gpu, spec_name):
    """S -> P, dP/dF and the new state at random Gauss points."""
    problem_mod, _ = gpu
    spec = getattr(pkg.material, spec_name)
    mesh = pkg.box_mesh(1, 1, 1)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, [[1, 0, 0, 0]], [0])
    prob.dt = 0.1
    rng = np.random.default_rng(11)
    n = 257
    ug, fpi, g, slip, R = random_gp_inputs(rng, n, spec.num_slip)
    P, D, state, its = prob.gp_map(ug, fpi, g, slip, R)
    # oracle
    tab = O.SLIP_TABLES[spec.slip]
    Pr = np.einsum("gia,gjb,kab->gkij", R, R, O.schmid_tensors(tab))
    Cr = O.rotate_rank4(R, O.cubic_stiffness(spec.C11, spec.C12, spec.C44))
    b = O.GPBatch(np.eye(3) + ug, fpi, g, Pr, Cr, spec.xm * np.ones(n), spec.ao, 0.1)
    S, its_o, ok = O.local_newton(b, spec.local_tol, spec.max_sub_step)
    assert ok.all()
    P_o = O.first_pk_stress(b, S)
    D_o = O.tangent(b, S)
    Fn, gn, sn = O.hardening_update(S, b, g, slip, spec.h * np.ones(n), spec.t_sat * np.ones(n),
                                    spec.gss_a * np.ones(n), spec.r * np.ones(n), spec.coplanar_q)
    assert its.cpu().numpy().max() > 1, "test points must be plastic"
    assert _rel(P, P_o) < 1e-9
    assert _rel(D, D_o) < 1e-8
    assert _rel(state[0], Fn) < 1e-12
    assert _rel(state[1], gn) < 1e-10
    assert _rel(state[2], sn) < 1e-9


def test_zero_strain_gives_zero_stress(pkg, gpu):
    problem_mod, _ = gpu
    spec = pkg.material.BENCH_STEEL
    prob = gpu_problem(pkg, problem_mod, spec, pkg.box_mesh(1, 1, 1), [[1, 0, 0, 0]], [0])
    n = 5
    ug, fpi, g, slip, R = random_gp_inputs(np.random.default_rng(3), n, 12, plastic=False)
    P, D, state, its = prob.gp_map(np.zeros((n, 3, 3)), fpi, g, slip, R)
    assert float(P.abs().max()) == 0.0 and int(its.max()) == 0
    assert torch.equal(state[1], torch.as_tensor(g, device=P.device))


def _poly_case(pkg, n=3, grains=4, seed=0, spec=None):
    spec = spec or pkg.material.BENCH_STEEL
    mesh = pkg.box_mesh(n, n, n)
    ori, rng = pkg.mesh.voronoi_grains(mesh, grains, seed)
    quat = pkg.material.random_quaternions(rng, grains)
    return spec, mesh, quat, ori


def test_assembly_residual_and_csr_match_oracle(pkg, gpu):
    problem_mod, _ = gpu
    spec, mesh, quat, ori = _poly_case(pkg)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori)
    orc = oracle_problem(spec, mesh, quat, ori)
    prob.dt = orc.dt = 0.1
    rng = np.random.default_rng(5)
    u = 1e-4 * rng.normal(size=(mesh.points.shape[0], 3))
    u[:, 2] += 1e-3 * mesh.points[:, 2]
    u = u.reshape(-1)
    res_o, A_o = orc.newton_update(u)
    res = prob.newton_update([torch.tensor(u, device="cuda").reshape(-1, 3)])[0].reshape(-1)
    A = problem_mod.DeviceCSR(prob, prob.A_values).to_scipy()
    assert np.array_equal(A.indptr, A_o.indptr) and np.array_equal(A.indices, A_o.indices)
    assert _rel(res, res_o) < 1e-10
    assert _rel(A.data, A_o.data) < 1e-9
    # SpMV and transposed SpMV
    x = torch.randn(A.shape[0], dtype=torch.float64, device="cuda")
    Ad = problem_mod.DeviceCSR(prob, prob.A_values)
    assert _rel(Ad.matvec(x), A_o @ x.cpu().numpy()) < 1e-9
    assert _rel(Ad.T.matvec(x), A_o.T @ x.cpu().numpy()) < 1e-9


def test_bicgstab_matches_oracle(pkg, gpu):
    problem_mod, solver_mod = gpu
    spec, mesh, quat, ori = _poly_case(pkg, n=4)
    bcs = roller_bcs(pkg.mesh, mesh.points, 1e-3)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori, bcs)
    orc = oracle_problem(spec, mesh, quat, ori, bcs)
    prob.dt = orc.dt = 0.1
    u = np.zeros(3 * mesh.points.shape[0])
    res, A = solver_mod.newton_update_helper(prob, torch.tensor(u, device="cuda"))
    res_o, A_o = orc.newton_update(u)
    bd, bv = orc.bc_dofs_vals()
    res_o[bd] = u[bd] - bv
    A_o = O.apply_bc_rows(A_o, bd)
    assert _rel(res, res_o) < 1e-10
    assert _rel(A.to_scipy().toarray(), A_o.toarray()) < 1e-9
    x0 = solver_mod.initial_increment(prob, torch.tensor(u, device="cuda"))
    for pc in (1, 2):
        x, k, ok = solver_mod.bicgstab(prob, A, -res, x0, precond=pc)
        assert ok and k > 0
        x_o, k_o = O.bicgstab(A_o, -res_o, x0.cpu().numpy(), lambda v: v / A_o.diagonal())
        assert _rel(x, x_o) < 1e-8, (pc, k, k_o)


def _run_steps(prob, solver_mod, disps, ts, bc_fn, opts, stress_fn):
    sol = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64, device="cuda")
    params = prob.internal_vars
    out = []
    for i in range(len(ts) - 1):
        prob.dt = float(ts[i + 1] - ts[i])
        bcs = bc_fn(float(disps[i + 1]))
        prob.fes[0].set_dirichlet_lists([b[0] for b in bcs], [b[1] for b in bcs], [b[2] for b in bcs])
        prob.set_params(params)
        o = dict(opts)
        o["initial_guess"] = [sol.reshape(-1, 3)]
        sol = solver_mod.solver(prob, o)[0].reshape(-1)
        sig = prob.compute_avg_stress(sol.reshape(-1, 3), params)
        out.append(stress_fn(sig.cpu().numpy()))
        params = prob.update_int_vars_gp(sol.reshape(-1, 3), params)
    prob.set_params(params)
    return np.array(out), sol


def test_load_steps_polycrystal_match_oracle(pkg, gpu):
    """Four tension steps of a 3^3, 4-grain FCC polycrystal: per-cell stress, u, Fp, g."""
    problem_mod, solver_mod = gpu
    spec, mesh, quat, ori = _poly_case(pkg)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori)
    orc = oracle_problem(spec, mesh, quat, ori)
    disps, ts = np.linspace(0, 4e-3, 5), np.linspace(0, 0.4, 5)
    bcf = lambda d: roller_bcs(pkg.mesh, mesh.points, d)
    opts = {"tol": 1e-9, "rel_tol": 1e-12}
    s_gpu, u_gpu = _run_steps(prob, solver_mod, disps, ts, bcf, opts, lambda s: s)
    s_o, u_o = O.run_load_steps(orc, disps, ts, bcf, opts)
    assert _rel(s_gpu, s_o) < 1e-8
    assert _rel(u_gpu, u_o) < 1e-8
    iv, iv_o = prob.internal_vars, orc.internal_vars
    assert _rel(iv[0], iv_o[0]) < 1e-10
    assert _rel(iv[1], iv_o[1]) < 1e-9
    assert _rel(iv[2], iv_o[2]) < 1e-8


def test_bcc24_load_steps_match_oracle(pkg, gpu):
    problem_mod, solver_mod = gpu
    spec, mesh, quat, ori = _poly_case(pkg, n=2, grains=3, seed=7, spec=pkg.material.BENCH_TANTALUM)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori)
    orc = oracle_problem(spec, mesh, quat, ori)
    disps, ts = np.linspace(0, 6e-3, 4), np.linspace(0, 0.6, 4)
    bcf = lambda d: roller_bcs(pkg.mesh, mesh.points, d)
    opts = {"tol": 1e-9, "rel_tol": 1e-12}
    s_gpu, u_gpu = _run_steps(prob, solver_mod, disps, ts, bcf, opts, lambda s: s)
    s_o, u_o = O.run_load_steps(orc, disps, ts, bcf, opts)
    assert _rel(s_gpu, s_o) < 1e-8 and _rel(u_gpu, u_o) < 1e-8


def test_golden_case1_copper_on_gpu(pkg, gpu):
    problem_mod, solver_mod = gpu
    mesh = pkg.box_mesh(1, 1, 1)
    prob = gpu_problem(pkg, problem_mod, pkg.material.CALIB_CASE1, mesh, [[1, 0, 0, 0]], [0])
    bcf = lambda d: corner_bcs(pkg.mesh, mesh.points, d)
    s, _ = _run_steps(prob, solver_mod, np.linspace(0, 0.025, 21), np.linspace(0, 2.5, 21), bcf,
                      {"jax_solver": {}, "tol": 1e-7}, lambda sg: sg[0, 2, 2])
    gold = GOLD["case1_szz"][:20]
    assert np.abs((s - gold) / gold).max() < 1e-8


def test_golden_case2_tantalum_on_gpu(pkg, gpu):
    problem_mod, solver_mod = gpu
    mesh = pkg.box_mesh(1, 1, 1)
    prob = gpu_problem(pkg, problem_mod, pkg.material.CALIB_CASE2, mesh, [[1, 0, 0, 0]], [0])
    bcf = lambda d: corner_bcs(pkg.mesh, mesh.points, d)
    s, _ = _run_steps(prob, solver_mod, np.linspace(0, -0.10, 41), np.linspace(0, 10.0, 41), bcf,
                      {"jax_solver": {}, "tol": 1e-7, "line_search_flag": True}, lambda sg: sg[0, 2, 2])
    gold = GOLD["case2_szz"][:40]
    assert np.abs((s - gold) / gold).max() < 1e-9


def test_golden_case4_polycrystal_on_gpu(pkg, gpu):
    """calibration_case4 scenario 0: 20^3 voxels, 50 grains (Neper n50-id0), 304 steel,
    80 steps to 2.5 %, mean sigma_zz over cells.  The reference solved with UMFPACK: the
    corner BCs leave the rigid rotation about z free, and on that near-singular matrix
    jax's BiCGSTAB stagnates into an exact rho = 0 breakdown in FP64 and hands Newton an
    unconverged increment.  A direct solve has no such failure, so the linear solve here
    restarts at breakdowns and runs to its tolerance; the free rotation does not change
    sigma_zz."""
    problem_mod, solver_mod = gpu
    L = 0.0295
    mesh = pkg.box_mesh(20, 20, 20, L, L, L)
    prob = gpu_problem(pkg, problem_mod, pkg.material.CALIB_CASE4, mesh, GOLD["case4_quat"],
                       GOLD["case4_grain"].astype(np.int64))
    c = pkg.mesh.corner_nodes(mesh.points, (0.0, 0.0, 0.0))
    bcf = lambda d: [(c, 0, 0.0), (c, 1, 0.0), (pkg.mesh.face_nodes(mesh.points, 2, 0.0), 2, 0.0),
                     (pkg.mesh.face_nodes(mesh.points, 2, L), 2, d)]
    nsteps = 80
    s, _ = _run_steps(prob, solver_mod, np.linspace(0, 0.025 * L, 81)[:nsteps + 1],
                      np.linspace(0, 2.5, 81)[:nsteps + 1], bcf,
                      {"jax_solver": {"restart_on_breakdown": True}, "tol": 1e-7, "line_search_flag": True},
                      lambda sg: sg[:, 2, 2].mean())
    gold = GOLD["case4_szz"][:nsteps]
    rel = np.abs((s - gold) / gold)
    assert rel.max() < 1e-5, rel


def test_local_newton_failure_is_reported(pkg, gpu):
    """Fault injected on the host: max_iter = 1 cannot converge a plastic point."""
    problem_mod, _ = gpu
    spec = pkg.material.BENCH_COPPER.replace(max_iter=1)
    prob = gpu_problem(pkg, problem_mod, spec, pkg.box_mesh(1, 1, 1), [[1, 0, 0, 0]], [0])
    ug, fpi, g, slip, R = random_gp_inputs(np.random.default_rng(0), 8, 12, strain=5e-3)
    with pytest.raises(RuntimeError, match="did not converge"):
        prob.gp_map(ug, fpi, g, slip, R)


def test_nonfinite_state_is_reported(pkg, gpu):
    problem_mod, _ = gpu
    prob = gpu_problem(pkg, problem_mod, pkg.material.BENCH_COPPER, pkg.box_mesh(1, 1, 1), [[1, 0, 0, 0]], [0])
    ug, fpi, g, slip, R = random_gp_inputs(np.random.default_rng(0), 4, 12)
    g[1, 3] = np.nan
    with pytest.raises((FloatingPointError, RuntimeError)):
        prob.gp_map(ug, fpi, g, slip, R)


def test_golden_304steel_cell_stresses_on_gpu(pkg, gpu):
    """polycrystal_304steel: 16^3 voxels, 8 grains, the reference's per-cell sigma_xx/yy/zz
    of its first 16 VTU steps (float32 files; Newton tolerance 1e-6 in the reference)."""
    problem_mod, solver_mod = gpu
    L = 0.016
    mesh = pkg.box_mesh(16, 16, 16, L, L, L)
    prob = gpu_problem(pkg, problem_mod, pkg.material.STEEL304, mesh, GOLD["steel_quat"],
                       GOLD["steel_ori"].astype(np.int64))
    c = pkg.mesh.corner_nodes(mesh.points, (0.0, 0.0, L))
    bcf = lambda d: [(c, 0, 0.0), (c, 1, 0.0), (pkg.mesh.face_nodes(mesh.points, 2, 0.0), 2, 0.0),
                     (pkg.mesh.face_nodes(mesh.points, 2, L), 2, d)]
    s, _ = _run_steps(prob, solver_mod, np.linspace(0, 0.01 * L, 51)[:17], np.linspace(0, 0.1, 51)[:17], bcf,
                      {"jax_solver": {}}, lambda sg: np.stack([sg[:, 0, 0], sg[:, 1, 1], sg[:, 2, 2]]))
    # The reference's BiCGSTAB stops at an absolute 1e-10 residual (solver.py:34-40); on this
    # 0.016 mm mesh that is ~2e-6 of the right-hand side, so its per-cell fields carry
    # ~1e-4 solver noise (the CPU oracle differs from the files by the same amount) while
    # the volume averages agree closely.
    gold = GOLD["steel_sig"]
    for i in range(16):
        scale = np.abs(gold[i][2]).max()
        assert np.abs(s[i] - gold[i]).max() / scale < 2e-3, i
        assert abs(s[i][2].mean() - gold[i][2].mean()) / abs(gold[i][2].mean()) < 1e-6, i


def test_golden_tantalum_single_crystal_on_gpu(pkg, gpu):
    """singlecrystal_tantalum: 10^3 cells, BCC12, compression to 1.25 % in 50 steps."""
    problem_mod, solver_mod = gpu
    L = float(GOLD["ta_L"])
    mesh = pkg.box_mesh(10, 10, 10, L, L, L)
    prob = gpu_problem(pkg, problem_mod, pkg.material.TANTALUM, mesh, [[1.0, 0.0, 0.0, 0.0]],
                       np.zeros(1000, dtype=np.int64))
    c = pkg.mesh.corner_nodes(mesh.points, (0.0, 0.0, L))
    bcf = lambda d: [(c, 0, 0.0), (c, 1, 0.0), (pkg.mesh.face_nodes(mesh.points, 2, 0.0), 2, 0.0),
                     (pkg.mesh.face_nodes(mesh.points, 2, L), 2, d)]
    s, _ = _run_steps(prob, solver_mod, np.linspace(0, -0.0125 * L, 51), np.linspace(0, 12.5, 51), bcf,
                      {"jax_solver": {}}, lambda sg: sg[:, 2, 2])
    gold = GOLD["ta_szz"]
    rel = np.abs(s - gold).max(1) / np.abs(gold).max(1)
    assert rel.max() < 2e-6, rel
