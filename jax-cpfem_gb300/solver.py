"""Global Newton solver with row elimination -- the ``solver(problem, solver_options)``
entry point of ``crystal_plasticity_OR_design/solver.py`` (a vendored copy of JAX-FEM's
solver), running on the GPU through the C ABI.

Same control flow as the reference (``solver.py:310-437``):
    res, A = newton_update_helper(dofs)
    while rel_res > rel_tol and res > tol:
        dofs = linear_incremental_solver(...)      # BiCGSTAB + Jacobi, optional line search
        res, A = newton_update_helper(dofs)
The tangent never leaves the device: assembly scatters into CSR values built on a
pattern fixed at set-up, and the Dirichlet rows are eliminated in place.
"""
from __future__ import annotations

import ctypes
import math
import time

import numpy as np
import torch

from . import _capi
from .problem import DeviceCSR, _dev_ptr, _flat, _stream

_KEYS = ("jax_solver", "umfpack_solver", "petsc_solver", "custom_solver")


def _dot(problem, x, y):
    ws = problem._buf("dot_ws", (int(problem.lib.cpfem_dot_workspace_bytes(x.numel())) // 8 + 64,))
    out = problem._buf("dot_out", (1,))
    _capi.check(problem.lib.cpfem_dot(x.numel(), _dev_ptr(x), _dev_ptr(y), _dev_ptr(out), _dev_ptr(ws), _stream()))
    return float(out.item())


def norm(problem, x):
    return math.sqrt(_dot(problem, x, x))


def bicgstab(problem, A: DeviceCSR, b, x0, precond=1, tol=1e-10, atol=1e-10, maxiter=10000, restarts=0,
             mg_options=None, grid_blocks=0):
    """``jax.scipy.sparse.linalg.bicgstab`` on the device matrix (``solver.py:34-40``), one
    persistent cooperative launch.  precond: 0 none, 1 Jacobi 1/diag(A) (the
    reference), 2 3x3 block-Jacobi, 3 geometric multigrid V-cycle (structured box
    meshes; ``mg_options`` go to ``CrystalPlasticity.multigrid``).  restarts > 0 restarts at
    a breakdown instead of stopping there (jax stops).  Returns (x, iterations or breakdown
    code, converged)."""
    lib = problem.lib
    x = x0.clone()
    nbytes = int(lib.cpfem_bicgstab_workspace_bytes(problem.num_nodes))
    ws = problem._buf("krylov_ws", (nbytes // 8 + 64,))
    info = np.zeros(2, dtype=np.int32)
    # flags 1: the launch also forms ||b - A x|| of its x (read below with the stats)
    opts = _capi.KrylovOpts(int(precond), 1 if A.transposed else 0, int(maxiter), int(restarts),
                            float(tol), float(atol), None, int(grid_blocks), 1)
    mg_options = dict(mg_options or {})
    if int(precond) == 3:
        if getattr(problem, "mg_fp64_only", False):
            mg_options["precision"] = "fp64"
        # the same hierarchy serves A^T (coarse operators (P^T A P)^T, transposed smoother)
        opts.mg = ctypes.pointer(problem.mg_setup(A.values, **mg_options))
    b = b.contiguous()
    with problem.region("bicgstab"):
        _capi.check(lib.cpfem_bicgstab_ex(problem.sell, _dev_ptr(A.values), _dev_ptr(b), _dev_ptr(x),
                                          ctypes.byref(opts), _dev_ptr(ws), info.ctypes.data, _stream()))
    k, ok = int(info[0]), bool(info[1])
    st = np.zeros(9)
    _capi.check(lib.cpfem_bicgstab_last_stats_ex(st.ctypes.data, 9))
    rn = math.sqrt(st[7]) if st[7] >= 0.0 else float("nan")
    problem._true_res = (x, b, rn)   # jax_solve's ||Ax - b|| check reads it
    if int(precond) == 3 and opts.mg.contents.precision == 1 and \
            not _fp32_solve_ok(ok, rn, math.sqrt(st[8]), tol, atol):
        # the FP32 V-cycle failed on this system (near-singular: see cpfem_mg_t.precision);
        # solve again with the FP64 V-cycle, and keep FP64 for this problem from now on
        problem.mg_fp64_only = True
        problem.stats["mg_fp64_fallbacks"] = problem.stats.get("mg_fp64_fallbacks", 0) + 1
        return bicgstab(problem, A, b, x0, precond, tol, atol, maxiter, restarts, mg_options, grid_blocks)
    return x, k, ok


def _fp32_solve_ok(converged, rn, bn, tol, atol):
    """An FP32-preconditioned solve is kept when it converged and its true residual rn =
    ||b - A x|| (formed by the solve's own launch) meets the stop rule, with a factor 10
    for the drift of the recursive residual."""
    return converged and math.isfinite(rn) and rn <= 10.0 * max(tol * bn, atol)


def jax_solve(problem, A, b, x0, precond=True, opts=None):
    """``solver.py:19-48``: BiCGSTAB, tol = atol = 1e-10, maxiter = 10000, then the
    ``||Ax - b|| < 0.1`` check."""
    opts = opts or {}
    pc = opts.get("precond", precond)
    pc = {True: 1, False: 0, "jacobi": 1, "block3": 2, "block_jacobi": 2, "mg": 3, "multigrid": 3}.get(pc, pc)
    rs = opts.get("restart_on_breakdown", 0)
    rs = 20 if rs is True else int(rs or 0)
    x, k, ok = bicgstab(problem, A, b, x0, precond=pc, tol=opts.get("tol", 1e-10),
                        atol=opts.get("atol", 1e-10), maxiter=opts.get("maxiter", 10000), restarts=rs,
                        mg_options=opts.get("mg_options"), grid_blocks=opts.get("grid_blocks", 0))
    problem.stats["krylov_iters"].append(k)
    last = getattr(problem, "_true_res", None)
    if last is not None and last[0] is x and last[1] is b:
        err = last[2]
    else:
        r = A.matvec(x)
        r.sub_(b)
        err = norm(problem, r)
    problem._true_res = None
    if not err < 0.1:
        raise RuntimeError(f"linear solver failed to converge with err = {err} (iterations {k})")
    return x


def linear_solver(problem, A, b, x0, solver_options):
    """``solver.py:91-113``."""
    if len(solver_options.keys() & set(_KEYS)) == 0:
        solver_options["jax_solver"] = {}
    if "jax_solver" in solver_options:
        o = solver_options["jax_solver"] or {}
        return jax_solve(problem, A, b, x0, o.get("precond", True), o)
    if "custom_solver" in solver_options:
        x = solver_options["custom_solver"](A, b, x0, solver_options)
        return torch.as_tensor(x, dtype=torch.float64, device=problem.device).reshape(-1).contiguous()
    raise NotImplementedError("only 'jax_solver' (device BiCGSTAB) and 'custom_solver' run on the GPU; "
                              "UMFPACK/PETSc host solvers are not part of the device path")


def _norm_checked(problem, x, status):
    """||x|| and the status word of the constitutive pass that produced x, read in one
    device-to-host transfer; raises on a failed local solve as the pass's own check would."""
    ws = problem._buf("dot_ws", (int(problem.lib.cpfem_dot_workspace_bytes(x.numel())) // 8 + 64,))
    out = problem._buf("dot_out", (1,))
    _capi.check(problem.lib.cpfem_dot(x.numel(), _dev_ptr(x), _dev_ptr(x), _dev_ptr(out), _dev_ptr(ws), _stream()))
    both = torch.stack([out[0], status[0].to(torch.float64)]).cpu()
    problem._check_status_bits(int(both[1]))
    return math.sqrt(float(both[0]))


def _update_deferred(problem, dofs):
    """newton_update_helper with the status check left to the next norm (one sync)."""
    u = dofs.reshape(-1)
    res, values, status = problem.assemble(u, need_tangent=True)
    problem.A_values = values
    res = res.reshape(-1)
    problem.apply_dirichlet(res, dofs, values)
    return res, DeviceCSR(problem, values), status


def _residual_deferred(problem, dofs):
    """residual_bc(check=True, keep_trial=True) with the status check left to the norm."""
    res, _, status = problem.assemble(dofs.reshape(-1), need_tangent=False, keep_trial=True)
    res = res.reshape(-1)
    problem.apply_dirichlet(res, dofs, None)
    return res, status


def newton_update_helper(problem, dofs):
    """Residual with BCs applied and the BC-eliminated device tangent (``solver.py:387-400``)."""
    res_list = problem.newton_update(problem.unflatten_fn_sol_list(dofs))
    res = res_list[0].reshape(-1)
    problem.apply_dirichlet(res, dofs, problem.A_values)
    return res, DeviceCSR(problem, problem.A_values)


def residual_bc(problem, dofs, check=True, keep_trial=False):
    res = problem.compute_residual(problem.unflatten_fn_sol_list(dofs), check=check,
                                   keep_trial=keep_trial)[0].reshape(-1)
    problem.apply_dirichlet(res, dofs, None)
    return res


def _expect_converged(history, limit):
    """Newton converges quadratically near the root, r_{k+1} ~ r_k^3 / r_{k-1}^2: True when
    that predicts the next residual well (4x) below the stop limit."""
    if len(history) < 2 or not (history[-2] > 0.0 and history[-1] < history[-2]):
        return False
    return history[-1] ** 3 / history[-2] ** 2 < 0.25 * limit


def initial_increment(problem, dofs):
    """x0 = assign_bc(0) - copy_bc(dofs) (``solver.py:221-227``)."""
    fe = problem.fes[0]
    x0 = problem._buf("x0", (problem.num_total_dofs_all_vars,))
    _capi.check(problem.lib.cpfem_bc_initial_guess(x0.numel(), int(fe.bc_dofs.numel()), _dev_ptr(fe.bc_dofs),
                                                   _dev_ptr(fe.bc_vals), _dev_ptr(dofs), _dev_ptr(x0), _stream()))
    return x0


def line_search(problem, dofs, inc):
    """``solver.py:240-276``: halve alpha up to 3 times while the BC residual norm drops."""
    def res_norm(alpha):
        d = dofs.clone()
        _capi.check(problem.lib.cpfem_axpy(d.numel(), float(alpha), _dev_ptr(inc), _dev_ptr(d), _stream()))
        # a trial step may drive local solves non-finite; its norm then compares false,
        # exactly as NaN does in the reference's loop
        return norm(problem, residual_bc(problem, d, check=False))
    alpha = 1.0
    rn = res_norm(alpha)
    for _ in range(3):
        alpha *= 0.5
        rh = res_norm(alpha)
        if rh > rn:
            alpha *= 2.0
            break
        rn = rh
    out = dofs.clone()
    _capi.check(problem.lib.cpfem_axpy(out.numel(), float(alpha), _dev_ptr(inc), _dev_ptr(out), _stream()))
    return out


def linear_incremental_solver(problem, res_vec, A, dofs, solver_options):
    """``solver.py:213-237``."""
    b = torch.neg(res_vec)
    x0 = initial_increment(problem, dofs)
    inc = linear_solver(problem, A, b, x0, solver_options)
    if solver_options.get("line_search_flag", False):
        return line_search(problem, dofs, inc)
    out = dofs.clone()
    _capi.check(problem.lib.cpfem_axpy(out.numel(), 1.0, _dev_ptr(inc), _dev_ptr(out), _stream()))
    return out


def solver(problem, solver_options=None):
    """Row-elimination Newton solve; returns ``[sol (num_nodes, 3)]``."""
    solver_options = {} if solver_options is None else solver_options
    start = time.time()
    if solver_options.get("initial_guess") is not None:
        dofs = _flat(solver_options["initial_guess"], problem.device).clone()
    else:
        dofs = torch.zeros(problem.num_total_dofs_all_vars, dtype=torch.float64, device=problem.device)
    rel_tol = solver_options.get("rel_tol", 1e-8)
    tol = solver_options.get("tol", 1e-6)
    max_newton = solver_options.get("max_newton", 100)

    res_vec, A, status = _update_deferred(problem, dofs)
    res_val = _norm_checked(problem, res_vec, status)
    res_val_initial = res_val
    rel_res_val = res_val / res_val_initial if res_val_initial > 0 else float("nan")
    history = [res_val]
    it = 0
    limit = max(tol, rel_tol * res_val_initial)
    skip = getattr(problem, "skip_final_tangent", True)
    while (rel_res_val > rel_tol) and (res_val > tol):
        if it >= max_newton:
            raise RuntimeError(f"global Newton did not converge in {max_newton} iterations (res = {res_val})")
        dofs = linear_incremental_solver(problem, res_vec, A, dofs, solver_options)
        res_vec = None
        if skip and _expect_converged(history, limit):
            # the last iterate needs no tangent: residual (and trial state) only, and the
            # tangent pass after all if the residual is not below the limit yet (its local
            # solves then start at their roots)
            res_vec, status = _residual_deferred(problem, dofs)
            res_val = _norm_checked(problem, res_vec, status)
            if (res_val / res_val_initial > rel_tol) and (res_val > tol):
                problem.stats["final_tangent_mispredicted"] = problem.stats.get("final_tangent_mispredicted", 0) + 1
                res_vec = None
            else:
                problem.stats["final_tangent_skipped"] = problem.stats.get("final_tangent_skipped", 0) + 1
        if res_vec is None:
            res_vec, A, status = _update_deferred(problem, dofs)
            res_val = _norm_checked(problem, res_vec, status)
        rel_res_val = res_val / res_val_initial
        history.append(res_val)
        it += 1
    if not math.isfinite(res_val):
        raise FloatingPointError("res_val contains NaN, stop the program!")
    problem.stats["newton_iters"] = it
    problem.stats["res_history"] = history
    problem.stats["solve_time"] = time.time() - start
    return problem.unflatten_fn_sol_list(dofs)
