"""GPU checks of the hand-written discrete adjoint: against complex-step derivatives of
the oracle's load history (an independent, cancellation-free derivative of the same
discrete model, to 1e-6 relative), against central finite differences of the GPU forward
(step 1e-6 relative for the Kalidindi parameters, 1e-4 degrees for the Euler angles), and
through the reference's own differentiation interface (``ad_wrapper`` with
``compute_avg_stress`` / ``update_int_vars_gp`` under autograd)."""
import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _history(pkg, problem_mod, n=2, grains=3, steps=3, seed=4):
    adjoint = importlib.import_module("jax-cpfem_gb300.adjoint")
    spec = pkg.material.BENCH_STEEL.replace(local_tol=1e-10)
    mesh = pkg.box_mesh(n, n, n)
    ori, rng = pkg.mesh.voronoi_grains(mesh, grains, seed)
    quat = pkg.material.random_quaternions(rng, grains)
    prob = problem_mod.CrystalPlasticity(mesh, additional_info=(quat, ori), material=spec)
    p = mesh.points
    fn = pkg.mesh.face_nodes

    def bc_fn(i, d):
        return [fn(p, 0, 0.0), fn(p, 1, 0.0), fn(p, 2, 0.0), fn(p, 2, 1.0)], [0, 1, 2, 2], [0.0, 0.0, 0.0, d]

    disps = np.linspace(0, 1e-3 * steps, steps + 1)
    ts = np.linspace(0, 0.1 * steps, steps + 1)
    opts = {"jax_solver": {}, "tol": 1e-10, "rel_tol": 1e-14}
    h = adjoint.LoadHistory(prob, disps, ts, bc_fn, quat, solver_options=opts)
    theta = np.array([spec.h, spec.gss_initial, spec.t_sat, spec.gss_a, spec.xm])
    euler = np.random.default_rng(seed).uniform(-20, 20, size=(grains, 3))
    return adjoint, h, theta, euler


def _objective(h, theta, euler, target):
    s = h.forward(theta, euler).cpu().numpy()[:, 2, 2]
    return float(((s - target) ** 2).sum()), s


def test_adjoint_gradient_matches_central_differences(pkg, gpu):
    problem_mod, _ = gpu
    adjoint, h, theta, euler = _history(pkg, problem_mod)
    s0 = h.forward(theta, euler).cpu().numpy()[:, 2, 2]
    target = 0.97 * s0 + 1.0
    # adjoint
    J, s = _objective(h, theta, euler, target)
    sbar = np.zeros((h.n_steps, 3, 3))
    sbar[:, 2, 2] = 2.0 * (s - target)
    tb, eb = h.backward(sbar)
    # finite differences
    fd_t = np.zeros(5)
    for k in range(5):
        d = np.zeros(5)
        d[k] = 1e-6 * abs(theta[k])
        fd_t[k] = (_objective(h, theta + d, euler, target)[0] - _objective(h, theta - d, euler, target)[0]) / (2 * d[k])
    fd_e = np.zeros_like(euler)
    for g in range(euler.shape[0]):
        for k in range(3):
            d = np.zeros_like(euler)
            d[g, k] = 1e-4
            fd_e[g, k] = (_objective(h, theta, euler + d, target)[0] - _objective(h, theta, euler - d, target)[0]) / 2e-4
    rel_t = np.abs(tb - fd_t) / np.maximum(np.abs(fd_t), 1e-12)
    rel_e = np.abs(eb - fd_e).max() / np.abs(fd_e).max()
    assert rel_t.max() < 1e-4, (tb, fd_t, rel_t)
    assert rel_e < 1e-4, (eb, fd_e)


def test_autograd_function_wraps_the_adjoint(pkg, gpu):
    problem_mod, _ = gpu
    adjoint, h, theta, euler = _history(pkg, problem_mod, steps=2)
    th = torch.tensor(theta, dtype=torch.float64, requires_grad=True)
    eu = torch.tensor(euler, dtype=torch.float64, requires_grad=True)
    out = adjoint.simulate(h, th, eu)
    loss = (out[:, 2, 2] ** 2).sum()
    loss.backward()
    sbar = np.zeros((h.n_steps, 3, 3))
    sbar[:, 2, 2] = 2.0 * out[:, 2, 2].detach().cpu().numpy()
    h.forward(theta, euler)
    tb, eb = h.backward(sbar)
    # every reduction of the forward and the backward has a fixed order (coloured scatter,
    # block-ordered dot products): two runs give the same gradient bit for bit
    assert np.array_equal(th.grad.numpy(), tb)
    assert np.array_equal(eu.grad.numpy(), eb)


def test_calibration_recovers_parameters(pkg, gpu):
    """L-BFGS-B with adjoint gradients (the loop of calibration_case1_..._GB.py) recovers
    h0 and g0 from a target curve made with them scaled by 1.15 and 0.9."""
    problem_mod, _ = gpu
    calib = importlib.import_module("jax-cpfem_gb300.calibration")
    adjoint, h, theta, euler = _history(pkg, problem_mod, steps=5)
    truth = theta.copy()
    truth[0] *= 1.15
    truth[1] *= 0.9
    target = h.forward(truth, euler).cpu().numpy()[:, 2, 2]
    res = calib.calibrate(h, target, theta, euler, names=("h0", "g0"), x0=1.0, bounds=(0.4, 3.0), maxiter=40)
    assert res.objective < 1e-12, res
    np.testing.assert_allclose(res.multipliers, [1.15, 0.9], rtol=1e-4)


def _oracle_history_fn(pkg, h, n, grains, steps, seed, spec):
    """The same load history on the oracle: f(theta, euler) -> per-step mean sigma_zz."""
    from oracle import cpfem_oracle as O
    mesh = pkg.box_mesh(n, n, n)
    ori, rng = pkg.mesh.voronoi_grains(mesh, grains, seed)
    quat = pkg.material.random_quaternions(rng, grains)
    pts = mesh.points

    def bcs(d):
        return [(O.face_nodes(pts, 0, 0.0), 0, 0.0), (O.face_nodes(pts, 1, 0.0), 1, 0.0),
                (O.face_nodes(pts, 2, 0.0), 2, 0.0), (O.face_nodes(pts, 2, 1.0), 2, d)]

    def f(theta, euler):
        return O.history_stress(pts, mesh.cells, O.FCC12, (spec.C11, spec.C12, spec.C44), quat, ori, theta, euler,
                                h.disps, h.ts, bcs, r=spec.r, coplanar=spec.coplanar_q, ao=spec.ao,
                                local_tol=spec.local_tol, max_sub_step=spec.max_sub_step,
                                solver_options={"tol": 1e-10, "rel_tol": 1e-13, "max_newton": 40})[:, 2, 2]
    return f


def test_adjoint_matches_oracle_complex_step(pkg, gpu):
    """3^3 cells, 3 grains, 3 load steps: the GPU adjoint gradient of a sigma_zz-curve misfit
    with respect to (h0, g0, gs, a, m) and every grain's Euler angles against complex-step
    derivatives of the oracle (forward-mode, no subtraction), to 1e-6 relative."""
    from oracle import cpfem_oracle as O
    problem_mod, _ = gpu
    n, grains, steps, seed = 3, 3, 3, 4
    adjoint, h, theta, euler = _history(pkg, problem_mod, n=n, grains=grains, steps=steps, seed=seed)
    spec = pkg.material.BENCH_STEEL.replace(local_tol=1e-10)
    s0 = h.forward(theta, euler).cpu().numpy()[:, 2, 2]
    target = 0.97 * s0 + 1.0
    sbar = np.zeros((steps, 3, 3))
    sbar[:, 2, 2] = 2.0 * (s0 - target)
    tb, eb = h.backward(sbar)
    f = _oracle_history_fn(pkg, h, n, grains, steps, seed, spec)
    s_o = f(theta, euler)
    assert np.abs(s_o - s0).max() < 1e-9 * np.abs(s_o).max()
    w = 2.0 * (s_o - target)
    cs_t = np.array([w @ O.complex_step(lambda th: f(th, euler), theta, np.eye(5)[k]) for k in range(5)])
    cs_e = np.zeros_like(euler)
    for g in range(grains):
        for k in range(3):
            d = np.zeros_like(euler)
            d[g, k] = 1.0
            cs_e[g, k] = w @ O.complex_step(lambda eu: f(theta, eu), euler, d)
    rel_t = np.abs(tb - cs_t) / np.abs(cs_t)
    rel_e = np.abs(eb - cs_e).max() / np.abs(cs_e).max()
    print(f"\nadjoint vs oracle complex step: theta rel {rel_t}, euler rel {rel_e:.2e}")
    assert rel_t.max() < 1e-6, (tb, cs_t, rel_t)
    assert rel_e < 1e-6, (eb, cs_e)


def test_ad_wrapper_reference_loop(pkg, gpu):
    """The calibration drivers' loop (``calibration_case1_singleCrystalCopper_GB.py``):
    ``fwd_pred = ad_wrapper(problem)``, per step ``sol_list = fwd_pred(params)``,
    ``compute_avg_stress``, ``update_int_vars_gp``, the misfit of the sigma_zz curve, then
    the gradient with respect to scalings of the per-GP h field and of the initial slip
    resistances -- by torch autograd through the package's nodes; against the LoadHistory
    adjoint of the same objective (h0, g0)."""
    problem_mod, _ = gpu
    adjoint, h, theta, euler = _history(pkg, problem_mod, n=2, grains=3, steps=3)
    s0 = h.forward(theta, euler).cpu().numpy()[:, 2, 2]
    target = 0.97 * s0 + 1.0
    sbar = np.zeros((h.n_steps, 3, 3))
    sbar[:, 2, 2] = 2.0 * (s0 - target)
    tb, _ = h.backward(sbar)
    # the same problem in the reference's 9-entry parameterised layout, with the
    # LoadHistory's rotations (R_euler R_quat per grain)
    spec = pkg.material.BENCH_STEEL.replace(local_tol=1e-10, per_gp_params=True)
    R = pkg.material.euler_zyx_deg(euler) @ pkg.material.rot_mat(h.grain_quat)
    ori = h.rot_idx0.cpu().numpy()[::8].astype(np.int64)
    prob = problem_mod.CrystalPlasticity(h.p.mesh, additional_info=(h.grain_quat, ori), material=spec)
    fwd_pred = adjoint.ad_wrapper(prob, {"jax_solver": {}, "tol": 1e-10, "rel_tol": 1e-14}, {})
    params0 = [t.clone() for t in prob.internal_vars]
    params0[3] = torch.tensor(np.repeat(R[ori][:, None], 8, axis=1), dtype=torch.float64, device="cuda")
    scale = torch.ones(2, dtype=torch.float64, device="cuda", requires_grad=True)
    params = list(params0)
    params[5] = params[5] * scale[0]          # h
    params[1] = params[1] * scale[1]          # g at the start (g0)
    obj = 0.0
    for i in range(h.n_steps):
        prob.dt = float(h.ts[i + 1] - h.ts[i])
        prob.fes[0].set_dirichlet_lists(*h.bc_fn(i, float(h.disps[i + 1])))
        sol_list = fwd_pred(params)
        sigma = prob.compute_avg_stress(sol_list[0], params)
        obj = obj + (sigma[:, 2, 2].mean() - float(target[i])) ** 2
        params = prob.update_int_vars_gp(sol_list[0], params)
    obj.backward()
    g = scale.grad.cpu().numpy()
    ref = np.array([tb[0] * theta[0], tb[1] * theta[1]])
    J = float(((s0 - target) ** 2).sum())
    assert abs(float(obj.detach()) - J) < 1e-9 * J
    assert np.abs(g - ref).max() < 1e-7 * np.abs(ref).max(), (g, ref)
