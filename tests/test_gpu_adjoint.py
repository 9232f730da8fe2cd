"""GPU checks of the hand-written discrete adjoint against central finite differences
of the GPU forward (step 1e-6 relative for the Kalidindi parameters, 1e-4 degrees for
the Euler angles)."""
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
    # element scatter uses FP64 atomics: two backward runs agree to rounding, not bitwise
    assert np.allclose(th.grad.numpy(), tb, rtol=1e-7, atol=0)
    assert np.allclose(eu.grad.numpy(), eb, rtol=1e-7, atol=1e-300)


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
