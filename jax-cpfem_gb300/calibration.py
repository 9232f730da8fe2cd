"""Parameter calibration on top of the hand-written adjoint.

The reference calibrates Kalidindi parameters against measured stress-strain curves with
scipy's L-BFGS-B, value and gradient from ``jax.value_and_grad`` through its load-step
simulation (``calibration/calibration_case1_singleCrystalCopper_GB.py:280-409``): the design
vector is one multiplier per calibrated parameter (start 1.4, bounds [0.4, 3.0]), the
objective the squared mismatch of the mean sigma_zz curve normalised by the target's
squared norm.  ``calibrate`` runs the same loop with the GPU forward (``LoadHistory``) and
its discrete adjoint supplying the gradient.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from .adjoint import THETA_NAMES


@dataclasses.dataclass
class CalibrationResult:
    theta: np.ndarray          # calibrated (h0, g0, gs, a, m)
    multipliers: np.ndarray    # design vector at the optimum
    objective: float
    iterations: int
    evaluations: int
    history: list              # (multipliers, objective) per evaluation
    success: bool
    message: str


def objective_and_gradient(history, theta, euler, target, component=(2, 2)):
    """Normalised squared mismatch of the mean stress curve and its gradient with respect
    to theta (one forward load history and one adjoint sweep)."""
    i, j = component
    target = np.asarray(target, dtype=np.float64)
    s = history.forward(theta, euler).cpu().numpy()[:, i, j]
    norm = float((target ** 2).sum())
    J = float(((s - target) ** 2).sum()) / norm
    sbar = np.zeros((history.n_steps, 3, 3))
    sbar[:, i, j] = 2.0 * (s - target) / norm
    theta_bar, euler_bar = history.backward(sbar)
    return J, np.asarray(theta_bar), np.asarray(euler_bar), s


def calibrate(history, target, theta_ref, euler, names=("h0", "g0", "gs"), x0=1.4, bounds=(0.4, 3.0),
              maxiter=10, gtol=1e-10, ftol=1e-14):
    """L-BFGS-B over multipliers x of the named parameters (theta = theta_ref with
    theta[k] = x_k theta_ref[k]); returns a ``CalibrationResult``."""
    from scipy.optimize import minimize
    theta_ref = np.asarray(theta_ref, dtype=np.float64)
    idx = [THETA_NAMES.index(n) for n in names]
    trace = []

    def fun(x):
        th = theta_ref.copy()
        th[idx] = np.asarray(x) * theta_ref[idx]
        J, tb, _, _ = objective_and_gradient(history, th, euler, target)
        trace.append((np.array(x, dtype=np.float64), J))
        return J, tb[idx] * theta_ref[idx]

    start = np.full(len(idx), float(x0)) if np.isscalar(x0) else np.asarray(x0, dtype=np.float64)
    res = minimize(fun, start, jac=True, method="L-BFGS-B", bounds=[bounds] * len(idx),
                   options={"maxiter": int(maxiter), "gtol": gtol, "ftol": ftol})
    th = theta_ref.copy()
    th[idx] = res.x * theta_ref[idx]
    return CalibrationResult(theta=th, multipliers=np.asarray(res.x), objective=float(res.fun),
                             iterations=int(res.nit), evaluations=len(trace), history=trace,
                             success=bool(res.success), message=str(res.message))
