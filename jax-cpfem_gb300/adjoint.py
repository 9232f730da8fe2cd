"""Hand-written discrete adjoint of the load-step sequence.

Replaces the reference's differentiation path: ``ad_wrapper`` / ``implicit_vjp``
(``crystal_plasticity_OR_design/solver.py:801-874``, driver copies in
``calibration/calibration_case1_singleCrystalCopper_GB.py:73-94`` and
``crystal_plasticity_OR_design/poly_sensitivity_rot_mesh2.py:70-92``) with ``jax.grad``
running through every load step and through the local Newton's ``custom_jvp``.

Forward: the plain load-step loop, checkpointing ``(u_n, Fp^-1_{n-1}, g_{n-1})`` per step.
Backward, for n = N..1, with lambda_n the cotangent of the committed state z_n:
  1. per GP (mode 1): F_bar from the stress cotangent and lambda_n, through the
     implicit-function VJP of the converged local Newton (recomputed from the checkpoint);
  2. f_u = gather of F_bar over the elements (assembly backward);
  3. A_n^T mu = f_u with the step's row-eliminated tangent (transposed BiCGSTAB);
  4. per GP (mode 2): lambda_{n-1} and the parameter / rotation cotangents from the stress
     cotangent, lambda_n and the equilibrium term -mu^T dR/dp.
Parameters: theta = (h0, g0, gs, a, m) and per-grain 'zyx' Euler angles in degrees
composed as R = R_euler R_q (``poly_sensitivity_rot_mesh2.py:41-65,203``).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi
from .material import euler_zyx_deg
from .problem import _dev_ptr, _stream
from . import solver as _solver

THETA_NAMES = ("h0", "g0", "gs", "a", "m")


def _euler_generators(angles_deg):
    """Spatial angular-velocity vectors w_k (per degree) with [w_k]x = dR/dphi_k R^T for
    R = Rx(c) Ry(b) Rz(a): w_a = Rx Ry e_z, w_b = Rx e_y, w_c = e_x."""
    ang = np.deg2rad(np.asarray(angles_deg, dtype=np.float64))
    b, c = ang[..., 1], ang[..., 2]
    cb, sb, cc, sc = np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    out = np.zeros(ang.shape[:-1] + (3, 3))
    # Ry e_z = (sb, 0, cb); Rx (x, y, z) = (x, cc y - sc z, sc y + cc z)
    out[..., 0, 0] = sb
    out[..., 0, 1] = -sc * cb
    out[..., 0, 2] = cc * cb
    out[..., 1, 1] = cc
    out[..., 1, 2] = sc
    out[..., 2, 0] = 1.0
    return out * (np.pi / 180.0)


class LoadHistory:
    """A load-step sequence on a ``CrystalPlasticity`` problem with checkpoints.

    ``bc_fn(i, disp) -> (node_lists, components, values)`` gives the Dirichlet lists of step
    i.  ``grain_quat`` (n_grains, 4) and the problem's per-GP ``rot_idx`` (the cell's grain)
    define the orientations; ``euler`` rotates them.
    """

    def __init__(self, problem, disps, ts, bc_fn, grain_quat, solver_options=None, adjoint_options=None):
        self.p = problem
        self.disps = np.asarray(disps, dtype=np.float64)
        self.ts = np.asarray(ts, dtype=np.float64)
        self.bc_fn = bc_fn
        self.grain_quat = np.asarray(grain_quat, dtype=np.float64)
        self.opts = dict(solver_options or {"jax_solver": {}})
        self.adj_opts = dict(adjoint_options or {})
        self.rot_idx0 = problem.rot_idx.clone()
        self.n_steps = len(self.ts) - 1

    # ------------------------------------------------------------------ set-up
    def _set_theta(self, theta, euler):
        p = self.p
        h0, g0, gs, a, m = (float(v) for v in theta)
        from .material import rot_mat
        R = euler_zyx_deg(np.asarray(euler, dtype=np.float64)) @ rot_mat(self.grain_quat)
        p.rot_table = torch.tensor(R.reshape(-1, 9), dtype=torch.float64, device=p.device)
        p.rot_idx = self.rot_idx0.clone()
        p.param_table = torch.tensor([[a, h0, gs, m, p.material.r]], dtype=torch.float64, device=p.device)
        p.param_idx = None
        G, N = p.num_gp, p.num_slip
        p.fpi = torch.zeros((9, G), dtype=torch.float64, device=p.device)
        p.fpi[0] = p.fpi[4] = p.fpi[8] = 1.0
        p.g = torch.full((N, G), g0, dtype=torch.float64, device=p.device)
        p.slip = torch.zeros((N, G), dtype=torch.float64, device=p.device)
        p._views = None
        p._post_cache = None

    def _set_step(self, i):
        p = self.p
        p.dt = float(self.ts[i + 1] - self.ts[i])
        nodes, comps, vals = self.bc_fn(i, float(self.disps[i + 1]))
        p.fes[0].set_dirichlet_lists(nodes, comps, vals)

    # ------------------------------------------------------------------ forward
    def forward(self, theta, euler, checkpoint=True):
        """Run the load steps; returns the mean cell Cauchy stress per step (n_steps, 3, 3)."""
        p = self.p
        self._set_theta(theta, euler)
        self.theta = np.asarray(theta, dtype=np.float64)
        self.euler = np.asarray(euler, dtype=np.float64)
        sol = torch.zeros(p.num_total_dofs_all_vars, dtype=torch.float64, device=p.device)
        p.reset_local_start()
        self.ckpt = []
        out = []
        params = p.internal_vars
        for i in range(self.n_steps):
            self._set_step(i)
            p.set_params(params)
            if checkpoint:
                self.ckpt.append((p.fpi.clone(), p.g.clone()))
            o = dict(self.opts)
            o["initial_guess"] = [sol.reshape(-1, 3)]
            sol = _solver.solver(p, o)[0].reshape(-1)
            sig = p.compute_avg_stress(sol.reshape(-1, 3), params)
            out.append(sig.mean(0))
            params = p.update_int_vars_gp(sol.reshape(-1, 3), params)
            if checkpoint:
                # the converged S of every GP (the last pass ran at sol) starts the backward's
                # recomputations of this step's local state
                w = p._warm()
                self.ckpt[-1] = self.ckpt[-1] + (sol.clone(), None if w is None else w.clone())
        p.set_params(params)
        return torch.stack(out)

    # ------------------------------------------------------------------ backward
    def _vjp(self, mode, u, fpi, g, cell_sig_bar, lam_fp, lam_g, mu=None, s_start=None):
        p = self.p
        G, N = p.num_gp, p.num_slip
        a = _capi.VjpArgs()
        a.num_gp, a.num_cells, a.mode, a.dt = G, p.num_cells, mode, float(p.dt)
        a.num_nodes, a.num_rot = p.num_nodes, int(p.rot_table.shape[0])
        a.num_param = int(p.param_table.shape[0])
        fe = p.fes[0]
        a.u, a.cells, a.shape_grads, a.jxw = u.data_ptr(), fe.cells.data_ptr(), fe.shape_grads.data_ptr(), \
            fe.JxW.data_ptr()
        a.fpi, a.g = fpi.data_ptr(), g.data_ptr()
        a.rot_table, a.rot_idx = p.rot_table.data_ptr(), p.rot_idx.data_ptr()
        a.param_table = p.param_table.data_ptr()
        a.param_idx = _dev_ptr(p.param_idx)
        a.elastic_table = _dev_ptr(p.elastic_table)
        a.cell_sig_bar = _dev_ptr(cell_sig_bar)
        a.fpi_bar, a.g_bar = _dev_ptr(lam_fp), _dev_ptr(lam_g)
        a.mu = _dev_ptr(mu)
        a.s_start = _dev_ptr(s_start)
        status = torch.zeros(1, dtype=torch.int32, device=p.device)
        a.status = status.data_ptr()
        outs = {}
        if mode == 1:
            outs["f_bar"] = torch.empty((9, G), dtype=torch.float64, device=p.device)
            a.f_bar = outs["f_bar"].data_ptr()
        else:
            outs["fpi_bar_old"] = torch.empty((9, G), dtype=torch.float64, device=p.device)
            outs["g_bar_old"] = torch.empty((N, G), dtype=torch.float64, device=p.device)
            outs["theta_bar"] = torch.empty((5, G), dtype=torch.float64, device=p.device)
            outs["rot_bar"] = torch.empty((3, G), dtype=torch.float64, device=p.device)
            for k, v in outs.items():
                setattr(a, k, v.data_ptr())
        with p.region(f"gp_vjp{mode}"):
            _capi.check(p.lib.cpfem_gp_vjp(p.mat_c, a, _stream()))
        p._check_status(status)
        return outs

    def backward(self, stress_bar):
        """stress_bar: (n_steps, 3, 3) cotangent of the per-step mean cell stress.
        Returns (theta_bar (5,), euler_bar (n_grains, 3))."""
        p = self.p
        G, N, E = p.num_gp, p.num_slip, p.num_cells
        stress_bar = torch.as_tensor(stress_bar, dtype=torch.float64, device=p.device).reshape(self.n_steps, 9)
        lam_fp = torch.zeros((9, G), dtype=torch.float64, device=p.device)
        lam_g = torch.zeros((N, G), dtype=torch.float64, device=p.device)
        theta_acc = torch.zeros(5, dtype=torch.float64, device=p.device)
        # per-GP rotation cotangents summed over the steps on the device; the per-grain sum
        # happens once on the host at the end
        rot_acc = torch.zeros((3, G), dtype=torch.float64, device=p.device)
        ridx = p.rot_idx.cpu().numpy().astype(np.int64)
        pc = self.adj_opts.get("precond", 1)
        self.krylov_iters = []
        predict, p.predict_local = p.predict_local, False   # starts come from the checkpoints
        try:
            return self._backward(stress_bar, lam_fp, lam_g, theta_acc, rot_acc, ridx, pc)
        finally:
            p.predict_local = predict

    def _backward(self, stress_bar, lam_fp, lam_g, theta_acc, rot_acc, ridx, pc):
        p = self.p
        E = p.num_cells
        for i in reversed(range(self.n_steps)):
            fpi, g, u, s_conv = self.ckpt[i]
            self._set_step(i)
            p.fpi, p.g = fpi, g
            p._views = None
            if s_conv is not None and p._warm() is not None:
                # the step's tangent is re-formed at its converged S: no prediction needed
                p._warm().copy_(s_conv)
            cell_bar = (stress_bar[i] / E).expand(E, 9).contiguous()
            # 1. F cotangent and its gather into the right-hand side
            fb = self._vjp(1, u, fpi, g, cell_bar, lam_fp, lam_g, s_start=s_conv)["f_bar"]
            f_u = torch.zeros(p.num_total_dofs_all_vars, dtype=torch.float64, device=p.device)
            fe = p.fes[0]
            p.scatter(fb, None, f_u, None)
            # 2. the step's tangent, row-eliminated, and the transposed solve
            res, A = _solver.newton_update_helper(p, u)
            mu0 = torch.zeros_like(f_u)
            mu, k, ok = _solver.bicgstab(p, A.T, f_u, mu0, precond=pc, tol=self.adj_opts.get("tol", 1e-10),
                                         atol=self.adj_opts.get("atol", 1e-14),
                                         maxiter=self.adj_opts.get("maxiter", 10000),
                                         mg_options=self.adj_opts.get("mg_options"))
            self.krylov_iters.append(k)
            if not ok:
                raise RuntimeError(f"adjoint solve did not converge (iterations {k})")
            mu[fe.bc_dofs.long()] = 0.0
            # 3. cotangents of the step's inputs
            o = self._vjp(2, u, fpi, g, cell_bar, lam_fp, lam_g, mu, s_start=s_conv)
            lam_fp, lam_g = o["fpi_bar_old"], o["g_bar_old"]
            theta_acc += o["theta_bar"].sum(1)
            rot_acc += o["rot_bar"]
        # parameters: (gss_a, h, t_sat, xm) -> (a, h0, gs, m); g0 through the initial state
        th = theta_acc.cpu().numpy()
        theta_bar = np.array([th[1], float(lam_g.sum()), th[2], th[0], th[3]])
        gen = _euler_generators(self.euler)                       # (n_grains, 3 angles, 3)
        per_gp = rot_acc.cpu().numpy()
        n_rot = p.rot_table.shape[0]
        per_grain = np.stack([np.bincount(ridx, weights=per_gp[c], minlength=n_rot) for c in range(3)], axis=1)
        euler_bar = np.einsum("gkj,gj->gk", gen, per_grain)
        return theta_bar, euler_bar


class SimulationFunction(torch.autograd.Function):
    """torch.autograd.Function over a LoadHistory: (theta (5,), euler (G,3)) -> the per-step
    mean cell stress (n_steps, 3, 3); backward runs the hand-written adjoint."""

    @staticmethod
    def forward(ctx, theta, euler, history):
        ctx.history = history
        out = history.forward(theta.detach().cpu().numpy(), euler.detach().cpu().numpy())
        ctx.save_for_backward(theta, euler)
        return out.to(theta.device)

    @staticmethod
    def backward(ctx, grad_out):
        theta, euler = ctx.saved_tensors
        tb, eb = ctx.history.backward(grad_out)
        return (torch.as_tensor(tb, dtype=theta.dtype, device=theta.device),
                torch.as_tensor(eb, dtype=euler.dtype, device=euler.device), None)


def simulate(history, theta, euler):
    """Differentiable forward: ``SimulationFunction.apply``."""
    return SimulationFunction.apply(theta, euler, history)


# --------------------------------------------------------------------------------------
# The reference's differentiation interface: ad_wrapper / implicit_vjp
# (crystal_plasticity_OR_design/solver.py:801-874) as torch autograd nodes.
#
# fwd_pred(params) -> sol_list is one load step's global solve as a function of the
# internal-variable list; its backward is implicit_vjp: A^T lambda = v with the step's
# row-eliminated tangent, then -lambda^T dc/dparams.  compute_avg_stress and
# update_int_vars_gp become differentiable in (sol, params) whenever an input requires
# grad, so a reference driver's load loop under torch autograd gives the gradient jax.grad
# gives the reference.  Cotangents: Fp^-1, g and the five per-GP parameters (gss_a, h,
# t_sat, xm, r) exactly; rotation matrices through their component tangent to SO(3),
# R_bar = 1/2 [w_bar]x R (what any chain through rotation parameters -- Euler angles,
# quaternions -- sees); slip enters no residual, and a nonzero cotangent of the new slip
# (an objective that reads slip) is refused.
# --------------------------------------------------------------------------------------
def _snap(p):
    fe = p.fes[0]
    return float(p.dt), fe.bc_dofs.clone(), fe.bc_vals.clone()


def _restore(p, snap):
    fe = p.fes[0]
    p.dt = snap[0]
    fe.bc_dofs, fe.bc_vals = snap[1], snap[2]
    fe._bc_dofs_np = None      # the next upload of lists compares against nothing
    fe.bc_token += 1


def _adopt_detached(p, params):
    p.set_params([t.detach() if isinstance(t, torch.Tensor) else t for t in params])


def _gp_vjp_state(p, mode, u, cell_bar=None, lam_fp=None, lam_g=None, mu=None):
    """cpfem_gp_vjp at the problem's adopted state (its Fp^-1, g and tables)."""
    G, N = p.num_gp, p.num_slip
    z = lambda rows: torch.zeros((rows, G), dtype=torch.float64, device=p.device)
    a = _capi.VjpArgs()
    a.num_gp, a.num_cells, a.mode, a.dt = G, p.num_cells, mode, float(p.dt)
    a.num_nodes, a.num_rot = p.num_nodes, int(p.rot_table.shape[0])
    a.num_param = int(p.param_table.shape[0])
    fe = p.fes[0]
    u = u.reshape(-1).contiguous()
    cell_bar = torch.zeros((p.num_cells, 9), dtype=torch.float64, device=p.device) if cell_bar is None \
        else cell_bar.reshape(p.num_cells, 9).contiguous()
    lam_fp = z(9) if lam_fp is None else lam_fp
    lam_g = z(N) if lam_g is None else lam_g
    mu = torch.zeros(p.num_total_dofs_all_vars, dtype=torch.float64, device=p.device) if mu is None else mu
    a.u, a.cells, a.shape_grads, a.jxw = u.data_ptr(), fe.cells.data_ptr(), fe.shape_grads.data_ptr(), \
        fe.JxW.data_ptr()
    a.fpi, a.g = p.fpi.data_ptr(), p.g.data_ptr()
    a.rot_table, a.rot_idx = p.rot_table.data_ptr(), p.rot_idx.data_ptr()
    a.param_table, a.param_idx = p.param_table.data_ptr(), _dev_ptr(p.param_idx)
    a.elastic_table = _dev_ptr(p.elastic_table)
    a.cell_sig_bar, a.fpi_bar, a.g_bar, a.mu = cell_bar.data_ptr(), lam_fp.data_ptr(), lam_g.data_ptr(), \
        mu.data_ptr()
    status = torch.zeros(1, dtype=torch.int32, device=p.device)
    a.status = status.data_ptr()
    out = {}
    if mode == 1:
        out["f_bar"] = z(9)
        a.f_bar = out["f_bar"].data_ptr()
    else:
        out.update(fpi_bar_old=z(9), g_bar_old=z(N), theta_bar=z(5), rot_bar=z(3))
        for k in ("fpi_bar_old", "g_bar_old", "theta_bar", "rot_bar"):
            setattr(a, k, out[k].data_ptr())
    with p.region(f"gp_vjp{mode}"):
        _capi.check(p.lib.cpfem_gp_vjp(p.mat_c, a, _stream()))
    p._check_status(status)
    return out


def _sol_cotangent(p, f_bar):
    """The assembly backward: u_bar_a = sum_q F_bar_q grad N_a (the coloured scatter)."""
    ub = torch.zeros(p.num_total_dofs_all_vars, dtype=torch.float64, device=p.device)
    p.scatter(f_bar, None, ub, None)
    return ub.reshape(p.num_nodes, 3)


def _param_cotangents(p, params, o):
    """Mode-2 outputs in the shapes of the reference's internal-variable list (None for an
    entry that does not require grad)."""
    E, N = p.num_cells, p.num_slip
    out = [o["fpi_bar_old"].t().reshape(E, 8, 3, 3), o["g_bar_old"].t().reshape(E, 8, N), None]
    R = torch.as_tensor(params[3], dtype=torch.float64, device=p.device).reshape(-1, 3, 3)
    w = o["rot_bar"].t()
    W = torch.zeros((w.shape[0], 3, 3), dtype=torch.float64, device=p.device)
    W[:, 0, 1], W[:, 0, 2], W[:, 1, 2] = -w[:, 2], w[:, 1], -w[:, 0]
    W[:, 1, 0], W[:, 2, 0], W[:, 2, 1] = w[:, 2], -w[:, 1], w[:, 0]
    out.append((0.5 * W @ R).reshape(E, 8, 3, 3))
    if len(params) >= 9:
        out += [o["theta_bar"][k].reshape(E, 8) for k in range(5)]
    if len(params) >= 10:
        out.append(None)   # the per-GP stiffness of the multi-phase layout is not differentiated
    return [None if (g is None or not (isinstance(t, torch.Tensor) and t.requires_grad)) else g
            for g, t in zip(out, params)]


class _FwdPred(torch.autograd.Function):
    @staticmethod
    def forward(ctx, p, solver_options, adjoint_options, *params):
        _adopt_detached(p, params)
        opts = dict(solver_options)
        if opts.get("initial_guess") is None and getattr(p, "initial_guess", None) is not None:
            opts["initial_guess"] = p.initial_guess
        sol = _solver.solver(p, opts)[0]
        ctx.p, ctx.adj, ctx.snap, ctx.raw = p, dict(adjoint_options), _snap(p), params
        ctx.save_for_backward(sol)
        return sol

    @staticmethod
    def backward(ctx, v):
        p, o, params = ctx.p, ctx.adj, ctx.raw
        sol = ctx.saved_tensors[0]
        _restore(p, ctx.snap)
        _adopt_detached(p, params)
        _, A = _solver.newton_update_helper(p, sol.reshape(-1))
        lam, k, ok = _solver.bicgstab(p, A.T, v.reshape(-1).contiguous(),
                                      torch.zeros(p.num_total_dofs_all_vars, dtype=torch.float64, device=p.device),
                                      precond=o.get("precond", 1), tol=o.get("tol", 1e-10),
                                      atol=o.get("atol", 1e-14), maxiter=o.get("maxiter", 10000),
                                      mg_options=o.get("mg_options"))
        if not ok:
            raise RuntimeError(f"adjoint solve did not converge (iterations {k})")
        lam[p.fes[0].bc_dofs.long()] = 0.0     # the Dirichlet rows of c do not depend on params
        out = _gp_vjp_state(p, 2, sol, mu=lam)
        return (None, None, None, *_param_cotangents(p, params, out))


def ad_wrapper(problem, solver_options=None, adjoint_solver_options=None):
    """``solver.py:856-874``: returns ``fwd_pred(params) -> sol_list`` whose gradient with
    respect to the internal-variable list runs the adjoint (``implicit_vjp``, :801-853).
    ``problem.initial_guess`` (``set_initial_guess``) seeds the solve when the options give
    none, and the solution becomes the next guess, as the calibration drivers' copy does
    (``calibration_case1_singleCrystalCopper_GB.py:73-94``)."""
    so = dict(solver_options or {})
    ao = dict(adjoint_solver_options or {})

    def fwd_pred(params):
        sol = _FwdPred.apply(problem, so, ao, *params)
        problem.set_initial_guess([sol.detach()])
        return [sol]
    return fwd_pred


class _AvgStress(torch.autograd.Function):
    @staticmethod
    def forward(ctx, p, sol, *params):
        _adopt_detached(p, params)
        sig = p._post_pass(sol.detach(), p.internal_vars)[0].clone()
        ctx.p, ctx.snap, ctx.raw = p, _snap(p), params
        ctx.save_for_backward(sol)
        return sig

    @staticmethod
    def backward(ctx, sig_bar):
        p, params = ctx.p, ctx.raw
        sol = ctx.saved_tensors[0]
        _restore(p, ctx.snap)
        _adopt_detached(p, params)
        cb = sig_bar.reshape(p.num_cells, 9).contiguous()
        u_bar = _sol_cotangent(p, _gp_vjp_state(p, 1, sol, cell_bar=cb)["f_bar"])
        out = _gp_vjp_state(p, 2, sol, cell_bar=cb)
        return (None, u_bar.reshape(sol.shape), *_param_cotangents(p, params, out))


class _UpdateIntVars(torch.autograd.Function):
    @staticmethod
    def forward(ctx, p, sol, *params):
        _adopt_detached(p, params)
        new = p._post_pass(sol.detach(), p.internal_vars)[1]
        ctx.p, ctx.snap, ctx.raw = p, _snap(p), params
        ctx.save_for_backward(sol)
        return tuple(t.clone() for t in new[:3]) + tuple(
            t.detach().clone() if isinstance(t, torch.Tensor) else torch.as_tensor(t) for t in params[3:])

    @staticmethod
    def backward(ctx, *bars):
        p, params = ctx.p, ctx.raw
        sol = ctx.saved_tensors[0]
        if bars[2] is not None and bool((bars[2] != 0).any()):
            raise NotImplementedError("the gradient of an objective that reads the slip variables is not "
                                      "implemented (slip enters no residual of the model)")
        _restore(p, ctx.snap)
        _adopt_detached(p, params)
        G, N = p.num_gp, p.num_slip
        lam_fp = None if bars[0] is None else bars[0].reshape(G, 9).t().contiguous()
        lam_g = None if bars[1] is None else bars[1].reshape(G, N).t().contiguous()
        u_bar = _sol_cotangent(p, _gp_vjp_state(p, 1, sol, lam_fp=lam_fp, lam_g=lam_g)["f_bar"])
        out = _param_cotangents(p, params, _gp_vjp_state(p, 2, sol, lam_fp=lam_fp, lam_g=lam_g))
        # the entries from rot on pass through unchanged
        for k in range(3, len(params)):
            if bars[k] is not None and isinstance(params[k], torch.Tensor) and params[k].requires_grad:
                out[k] = bars[k] if out[k] is None else out[k] + bars[k]
        if bars[2] is not None and isinstance(params[2], torch.Tensor) and params[2].requires_grad:
            out[2] = bars[2]
        return (None, u_bar.reshape(sol.shape), *out)


def avg_stress(problem, sol, params):
    """``compute_avg_stress`` as an autograd node in (sol, params)."""
    return _AvgStress.apply(problem, torch.as_tensor(sol, dtype=torch.float64, device=problem.device), *params)


def update_int_vars(problem, sol, params):
    """``update_int_vars_gp`` as an autograd node in (sol, params)."""
    return list(_UpdateIntVars.apply(problem, torch.as_tensor(sol, dtype=torch.float64, device=problem.device),
                                     *params))
