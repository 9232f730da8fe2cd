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


class DeferredSolveFailed(Exception):
    """A deferred BiCGSTAB solve (``bicgstab(..., deferred=True)``) did not pass its checks
    when its report was read; the Newton iteration that used it is redone with a checked
    solve."""


def _report_buffer(problem, slot=0):
    """The problem's pinned host copies of deferred solves' reports: two slots, used in turn,
    so a solve queued behind a residual norm cannot overwrite the report of the solve that
    norm checks before the host has read it."""
    bufs = getattr(problem, "_report_host", None)
    if bufs is None:
        n = ctypes.sizeof(_capi.SolveReport)
        bufs = problem._report_host = [torch.zeros(n, dtype=torch.uint8).pin_memory() for _ in range(2)]
    return bufs[slot]


def bicgstab(problem, A: DeviceCSR, b, x0, precond=1, tol=1e-10, atol=1e-10, maxiter=10000, restarts=0,
             mg_options=None, grid_blocks=0, deferred=False):
    """``jax.scipy.sparse.linalg.bicgstab`` on the device matrix (``solver.py:34-40``), one
    persistent cooperative launch.  precond: 0 none, 1 Jacobi 1/diag(A) (the
    reference), 2 3x3 block-Jacobi, 3 geometric multigrid V-cycle (structured box
    meshes; ``mg_options`` go to ``CrystalPlasticity.multigrid``).  restarts > 0 restarts at
    a breakdown instead of stopping there (jax stops).  Returns (x, iterations or breakdown
    code, converged).  ``deferred``: the call returns as soon as the solve is queued, with
    (x, None, None); its report is copied to pinned memory behind it and checked by
    ``resolve_deferred`` after the caller's next synchronisation (``solver``'s Newton loop:
    the residual norm of the next iterate), so the host prepares the next pass while the
    solve runs."""
    lib = problem.lib
    x = x0.clone()
    nbytes = int(lib.cpfem_bicgstab_workspace_bytes(problem.num_nodes))
    ws = problem._buf("krylov_ws", (nbytes // 8 + 64,))
    info = np.zeros(2, dtype=np.int32)
    # flags 1: the launch also forms ||b - A x|| of its x (read below with the stats);
    # flags 2: the report goes to pinned memory without waiting
    opts = _capi.KrylovOpts(int(precond), 1 if A.transposed else 0, int(maxiter), int(restarts),
                            float(tol), float(atol), None, int(grid_blocks), 1 | (2 if deferred else 0))
    if deferred:
        slot = problem._report_slot = 1 - getattr(problem, "_report_slot", 1)
        opts.report = _report_buffer(problem, slot).data_ptr()
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
    if deferred:
        problem._pending_solve = {"fp32": int(precond) == 3 and opts.mg.contents.precision == 1,
                                  "tol": float(tol), "atol": float(atol), "slot": slot}
        return x, None, None
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


def resolve_deferred(problem):
    """Check the report of the problem's deferred solve, if one is pending (call after a
    synchronisation of the stream): the Krylov count joins ``stats``; a failed grid barrier,
    an FP32 V-cycle solve that misses the stop rule (which switches the problem to the FP64
    V-cycle, as the checked path does) or a true residual that fails ``jax_solve``'s
    ``||Ax - b|| < 0.1`` raise ``DeferredSolveFailed``."""
    p = getattr(problem, "_pending_solve", None)
    if p is None:
        return
    problem._pending_solve = None
    r = _capi.SolveReport.from_address(_report_buffer(problem, p.get("slot", 0)).data_ptr())
    rn = math.sqrt(r.true_rs) if r.true_rs >= 0.0 else float("nan")
    if r.error:
        raise DeferredSolveFailed("a grid barrier of the solve timed out")
    if p["fp32"] and not _fp32_solve_ok(r.rs <= r.atol2, rn, math.sqrt(r.bb), p["tol"], p["atol"]):
        problem.mg_fp64_only = True
        problem.stats["mg_fp64_fallbacks"] = problem.stats.get("mg_fp64_fallbacks", 0) + 1
        raise DeferredSolveFailed("the FP32 V-cycle solve missed the stop rule")
    if not rn < 0.1:
        raise DeferredSolveFailed(f"the solve's true residual is {rn}")
    problem.stats["krylov_iters"].append(int(r.k))


def jax_solve(problem, A, b, x0, precond=True, opts=None, deferred=False):
    """``solver.py:19-48``: BiCGSTAB, tol = atol = 1e-10, maxiter = 10000, then the
    ``||Ax - b|| < 0.1`` check."""
    opts = opts or {}
    pc = opts.get("precond", precond)
    pc = {True: 1, False: 0, "jacobi": 1, "block3": 2, "block_jacobi": 2, "mg": 3, "multigrid": 3}.get(pc, pc)
    rs = opts.get("restart_on_breakdown", 0)
    rs = 20 if rs is True else int(rs or 0)
    x, k, ok = bicgstab(problem, A, b, x0, precond=pc, tol=opts.get("tol", 1e-10),
                        atol=opts.get("atol", 1e-10), maxiter=opts.get("maxiter", 10000), restarts=rs,
                        mg_options=opts.get("mg_options"), grid_blocks=opts.get("grid_blocks", 0),
                        deferred=deferred)
    if deferred:
        return x
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


def linear_solver(problem, A, b, x0, solver_options, deferred=False):
    """``solver.py:91-113``.  ``deferred`` applies to the device BiCGSTAB (``jax_solver``)."""
    if len(solver_options.keys() & set(_KEYS)) == 0:
        solver_options["jax_solver"] = {}
    if "jax_solver" in solver_options:
        o = solver_options["jax_solver"] or {}
        return jax_solve(problem, A, b, x0, o.get("precond", True), o, deferred=deferred)
    if "custom_solver" in solver_options:
        x = solver_options["custom_solver"](A, b, x0, solver_options)
        return torch.as_tensor(x, dtype=torch.float64, device=problem.device).reshape(-1).contiguous()
    raise NotImplementedError("only 'jax_solver' (device BiCGSTAB) and 'custom_solver' run on the GPU; "
                              "UMFPACK/PETSc host solvers are not part of the device path")


class _NormCopy:
    """||x||^2 and the status word of the pass that produced x, on their way to the
    problem's pinned host buffer behind the work queued so far, with an event after the
    copy: the host may queue more work before ``wait`` reads them.  One copy per problem is
    in flight at a time (each is waited for before the next is queued)."""

    def __init__(self, problem, x, status):
        ws = problem._buf("dot_ws", (int(problem.lib.cpfem_dot_workspace_bytes(x.numel())) // 8 + 64,))
        out = problem._buf("dot_out", (1,))
        _capi.check(problem.lib.cpfem_dot(x.numel(), _dev_ptr(x), _dev_ptr(x), _dev_ptr(out), _dev_ptr(ws),
                                          _stream()))
        host = getattr(problem, "_norm_host", None)
        if host is None:
            host = problem._norm_host = torch.zeros(2, dtype=torch.float64).pin_memory()
            problem._norm_event = torch.cuda.Event()
        host.copy_(torch.stack([out[0], status[0].to(torch.float64)]), non_blocking=True)
        problem._norm_event.record()
        self.host, self.event = host, problem._norm_event

    def wait(self):
        self.event.synchronize()
        return float(self.host[0]), int(self.host[1])


def _norm_queue(problem, x, status):
    """The first half of ``_norm_checked``: queue the norm and status copy; the ticket also
    names the deferred solve whose report that copy follows."""
    return problem._pending_solve, _NormCopy(problem, x, status)


def _norm_wait(problem, ticket):
    """The second half: wait for the copy, check the deferred solve it follows (the pass ran
    at the iterate that solve produced), then raise on a failed local solve as the pass's
    own check would.  A solve queued after the copy stays pending."""
    pending, copy = ticket
    sq, status_word = copy.wait()
    later = problem._pending_solve if problem._pending_solve is not pending else None
    problem._pending_solve = pending
    try:
        resolve_deferred(problem)
    finally:
        problem._pending_solve = later
    problem._check_status_bits(status_word)
    # the status read here is that of the pass whose trial outputs the problem keeps (or
    # of a pass after it): the post-processing need not read it again
    problem._trial_checked = True
    return math.sqrt(sq)


def _norm_checked(problem, x, status):
    """||x|| and the status word of the constitutive pass that produced x, read in one
    device-to-host transfer; checks a deferred solve's report first, then the pass's status."""
    return _norm_wait(problem, _norm_queue(problem, x, status))


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


def linear_incremental_solver(problem, res_vec, A, dofs, solver_options, deferred=False):
    """``solver.py:213-237``."""
    b = torch.neg(res_vec)
    x0 = initial_increment(problem, dofs)
    inc = linear_solver(problem, A, b, x0, solver_options, deferred=deferred)
    if solver_options.get("line_search_flag", False):
        return line_search(problem, dofs, inc)
    out = dofs.clone()
    _capi.check(problem.lib.cpfem_axpy(out.numel(), 1.0, _dev_ptr(inc), _dev_ptr(out), _stream()))
    return out


def _defers(problem, solver_options):
    """Whether the Newton loop may defer the checks of its Krylov solves: the device
    BiCGSTAB without a line search (whose trial points would use the unchecked increment),
    unless the problem opts out (``problem.defer_krylov_checks = False``)."""
    if not getattr(problem, "defer_krylov_checks", True) or solver_options.get("line_search_flag", False):
        return False
    keys = solver_options.keys() & set(_KEYS)
    return not keys or keys == {"jax_solver"}


def _continues(history, limit):
    """Whether the Newton loop will almost surely go on after the iterate being formed: the
    quadratic model (``_expect_converged``) puts its residual above twice the stop limit, or
    there is no contraction rate yet."""
    if len(history) < 2 or not (history[-2] > 0.0 and history[-1] < history[-2]):
        return True
    return history[-1] ** 3 / history[-2] ** 2 > 2.0 * limit


def solver(problem, solver_options=None):
    """Row-elimination Newton solve; returns ``[sol (num_nodes, 3)]``.

    Each iteration's BiCGSTAB is deferred (``bicgstab(deferred=True)``): the host queues the
    next constitutive pass without waiting for the solve, and the solve's report is checked
    together with that pass's residual norm; an iteration whose solve fails the check is
    redone from its start with a checked solve, so the iterates and the result are those of
    the checked loop.  Where the loop will almost surely go on (``_continues``), the next
    iteration's solve is queued behind the residual norm's copy, before the host waits for
    it, so the device does not idle while the host reads the norm and decides
    (``problem.queue_next_solve = False`` turns this off); a solve so queued whose iteration
    never comes (the residual was below the limit after all) is dropped
    (``stats["solves_dropped"]``)."""
    solver_options = {} if solver_options is None else solver_options
    start = time.time()
    problem._pending_solve = None
    if solver_options.get("initial_guess") is not None:
        dofs = _flat(solver_options["initial_guess"], problem.device).clone()
    else:
        dofs = torch.zeros(problem.num_total_dofs_all_vars, dtype=torch.float64, device=problem.device)
    rel_tol = solver_options.get("rel_tol", 1e-8)
    tol = solver_options.get("tol", 1e-6)
    max_newton = solver_options.get("max_newton", 100)
    defer = _defers(problem, solver_options)
    ahead = defer and getattr(problem, "queue_next_solve", True)

    def tangent_pass(dofs, deferred, go_on):
        """The iterate's residual and tangent, and its norm read; with ``go_on`` the next
        iteration's solve is queued before the read (returned, else None)."""
        res_vec, A, status = _update_deferred(problem, dofs)
        if not (ahead and deferred and go_on):
            return res_vec, A, _norm_checked(problem, res_vec, status), None
        ticket = _norm_queue(problem, res_vec, status)
        queued = linear_incremental_solver(problem, res_vec, A, dofs, solver_options, deferred=True)
        return res_vec, A, _norm_wait(problem, ticket), queued

    res_vec, A, res_val, queued = tangent_pass(dofs, defer, True)
    res_val_initial = res_val
    rel_res_val = res_val / res_val_initial if res_val_initial > 0 else float("nan")
    history = [res_val]
    it = 0
    limit = max(tol, rel_tol * res_val_initial)
    skip = getattr(problem, "skip_final_tangent", True)

    def iteration(res_vec, A, dofs, deferred, queued):
        if queued is not None:
            dofs = queued    # this iteration's solve, queued behind the last norm
        else:
            dofs = linear_incremental_solver(problem, res_vec, A, dofs, solver_options, deferred=deferred)
        res_vec = None
        go_on = _continues(history, limit)
        if skip and _expect_converged(history, limit):
            # the last iterate needs no tangent: residual (and trial state) only, and the
            # tangent pass after all if the residual is not below the limit yet (its local
            # solves then start at their roots)
            res_vec, status = _residual_deferred(problem, dofs)
            res_val = _norm_checked(problem, res_vec, status)
            if (res_val / res_val_initial > rel_tol) and (res_val > tol):
                problem.stats["final_tangent_mispredicted"] = problem.stats.get("final_tangent_mispredicted", 0) + 1
                res_vec, go_on = None, True
            else:
                problem.stats["final_tangent_skipped"] = problem.stats.get("final_tangent_skipped", 0) + 1
        queued = None
        if res_vec is None:
            res_vec, A, res_val, queued = tangent_pass(dofs, deferred, go_on)
        return res_vec, A, dofs, res_val, queued

    while (rel_res_val > rel_tol) and (res_val > tol):
        if it >= max_newton:
            raise RuntimeError(f"global Newton did not converge in {max_newton} iterations (res = {res_val})")
        try:
            res_vec, A, dofs, res_val, queued = iteration(res_vec, A, dofs, defer, queued)
        except DeferredSolveFailed:
            # redo the iteration from its start with a checked solve: the system at the
            # iteration's start is formed again (its buffers now hold the failed iterate's);
            # a solve queued behind the failed check is dropped with it
            problem.stats["deferred_redone"] = problem.stats.get("deferred_redone", 0) + 1
            problem._pending_solve = None
            dofs_start = dofs
            res_vec, A, _, _ = tangent_pass(dofs_start, False, False)
            res_vec, A, dofs, res_val, queued = iteration(res_vec, A, dofs_start, False, None)
        rel_res_val = res_val / res_val_initial
        history.append(res_val)
        it += 1
    if queued is not None:
        problem.stats["solves_dropped"] = problem.stats.get("solves_dropped", 0) + 1
    problem._pending_solve = None
    if not math.isfinite(res_val):
        raise FloatingPointError("res_val contains NaN, stop the program!")
    problem.stats["newton_iters"] = it
    problem.stats["res_history"] = history
    problem.stats["solve_time"] = time.time() - start
    return problem.unflatten_fn_sol_list(dofs)


# ---------------------------------------------------------------------------------------
# BC helpers on device vectors (``solver.py:119-192``).  The Dirichlet dofs of a problem are
# unique (a dof named twice keeps its last value, as the reference's sequential .at[].set).
# ---------------------------------------------------------------------------------------
def _bc_index(problem):
    fe = problem.fes[0]
    return fe.bc_dofs.long(), fe.bc_vals


def assign_bc(dofs, problem):
    """``assign_bc``: a copy of dofs with the BC values on their dofs."""
    idx, vals = _bc_index(problem)
    out = _flat(dofs, problem.device).clone()
    out[idx] = vals
    return out


def assign_zeros_bc(dofs, problem):
    """``assign_zeros_bc``: a copy of dofs with zeros on the BC dofs."""
    idx, _ = _bc_index(problem)
    out = _flat(dofs, problem.device).clone()
    out[idx] = 0.0
    return out


def assign_ones_bc(dofs, problem):
    """``assign_ones_bc``: a copy of dofs with ones on the BC dofs."""
    idx, _ = _bc_index(problem)
    out = _flat(dofs, problem.device).clone()
    out[idx] = 1.0
    return out


def copy_bc(dofs, problem):
    """``copy_bc``: zeros except dofs' own values on the BC dofs."""
    idx, _ = _bc_index(problem)
    d = _flat(dofs, problem.device)
    out = torch.zeros_like(d)
    out[idx] = d[idx]
    return out


def apply_bc_vec(res_vec, dofs, problem, scale=1.0):
    """``apply_bc_vec``: BC rows of the residual become dofs - scale * value."""
    idx, vals = _bc_index(problem)
    out = _flat(res_vec, problem.device).clone()
    out[idx] = _flat(dofs, problem.device)[idx] - scale * vals
    return out


# ---------------------------------------------------------------------------------------
# Arc-length continuation (Crisfield's form) and dynamic relaxation (``solver.py:447-795``).
# The reference solves their linear systems with UMFPACK; here the device BiCGSTAB solves
# them to ``DIRECT_SOLVE`` (relative 1e-12) unless ``solver_options`` name another solver
# (``jax_solver`` options, or a ``custom_solver`` such as a host direct solver).  Neither
# routine commits internal variables: the caller does, between steps, as with ``solver``.
# ---------------------------------------------------------------------------------------
DIRECT_SOLVE = {"jax_solver": {"tol": 1e-12, "atol": 1e-30, "maxiter": 100000, "restart_on_breakdown": True}}


def _solve_to(problem, A, b, solver_options):
    """A^-1 b for the row-eliminated A, solved for b / |b| and scaled back (a direct solver's
    answer does not depend on the scale of b; the Krylov stop rule's absolute floor would).
    The start has the Dirichlet components of the answer (A's unit rows give them): a start
    of zero would make the first residual, and so BiCGSTAB's shadow vector, live on the
    Dirichlet dofs alone, orthogonal to every later residual (a breakdown at once when the
    right-hand side is u_b)."""
    opts = {k: (dict(v) if isinstance(v, dict) else v) for k, v in (solver_options or DIRECT_SOLVE).items()}
    nb = float(torch.linalg.vector_norm(b))
    if nb == 0.0:
        return torch.zeros_like(b)
    bn = (b / nb).contiguous()
    idx, _ = _bc_index(problem)
    x0 = torch.zeros_like(b)
    x0[idx] = bn[idx]
    x = linear_solver(problem, A, bn, x0, opts)
    return x * nb


def _tangent_bc(problem, dofs, scale=1.0):
    """Residual with BC rows dofs - scale * values and the row-eliminated tangent at dofs
    (``newton_update_helper`` of the arc-length solvers, ``solver.py:452-459``)."""
    res, values, status = problem.assemble(dofs, need_tangent=True)
    problem._check_status(status)
    problem.A_values = values
    res = res.reshape(-1)
    problem.apply_dirichlet(res, dofs, values)
    if scale != 1.0:
        idx, vals = _bc_index(problem)
        res.index_add_(0, idx, (1.0 - scale) * vals)
    return res.clone(), DeviceCSR(problem, values)


def _pick_lambda(a1, a2, a3, u, lam, prev_u, prev_lam, dub, dut, dir_u, dir_lam, w):
    """The two roots of the arc-length constraint and the one whose direction continues the
    previous increment (``solver.py:480-508``)."""
    disc = math.sqrt(a2 * a2 - 4.0 * a1 * a3) if a2 * a2 - 4.0 * a1 * a3 >= 0.0 else float("nan")
    l1 = (-a2 + disc) / (2.0 * a1)
    l2 = (-a2 - disc) / (2.0 * a1)
    if not (math.isfinite(l1) and math.isfinite(l2)):
        raise RuntimeError(f"no valid solutions for delta lambda, a1 = {a1}, a2 = {a2}, a3 = {a3}")
    base = u - prev_u
    dd = float(torch.dot(dir_u, base + dub))
    dt = float(torch.dot(dir_u, dut))
    d1 = dd + l1 * dt + w * dir_lam * (lam + l1 - prev_lam)
    d2 = dd + l2 * dt + w * dir_lam * (lam + l2 - prev_lam)
    if abs(d1) < 1e-10 and abs(d2) < 1e-10:
        return max(l1, l2)
    return l1 if d1 > d2 else l2


def _arc_length(problem, prev_u_vec, prev_lamda, prev_Delta_u_vec, prev_Delta_lamda, Delta_l, psi, tol,
                max_iter, solver_options, q_vec):
    dev = problem.device
    prev_u = _flat(prev_u_vec, dev).clone()
    u = prev_u.clone()
    lam = prev_lam = float(prev_lamda)
    dir_u = _flat(prev_Delta_u_vec, dev).clone()
    dir_lam = float(prev_Delta_lamda)
    if q_vec is None:
        drive = assign_bc(torch.zeros_like(u), problem)          # u_b
    else:
        drive = assign_zeros_bc(_flat(q_vec, dev), problem)      # q mapped
    w = psi ** 2 * float(torch.dot(drive, drive))
    res_val, it = 1.0, 0
    while res_val > tol:
        if it >= max_iter:
            raise RuntimeError(f"arc-length step did not converge in {max_iter} iterations (res = {res_val})")
        if q_vec is None:
            res, A = _tangent_bc(problem, u, lam)
            res_val = float(torch.linalg.vector_norm(res))
            dub = _solve_to(problem, A, torch.neg(res), solver_options)
            dut = _solve_to(problem, A, drive, solver_options)
        else:
            res, A = _tangent_bc(problem, u)
            rq = res + lam * drive
            res_val = float(torch.linalg.vector_norm(rq))
            dub = _solve_to(problem, A, torch.neg(rq), solver_options)
            dut = _solve_to(problem, A, torch.neg(drive), solver_options)
        Du, Dlam = u - prev_u, lam - prev_lam
        s = Du + dub
        a1 = float(torch.dot(dut, dut)) + w
        a2 = 2.0 * float(torch.dot(s, dut)) + 2.0 * w * Dlam
        a3 = float(torch.dot(s, s)) + w * Dlam ** 2 - Delta_l ** 2
        dl = _pick_lambda(a1, a2, a3, u, lam, prev_u, prev_lam, dub, dut, dir_u, dir_lam, w)
        lam = lam + dl
        u = u + dub + dl * dut
        dir_u, dir_lam = u - prev_u, lam - prev_lam
        it += 1
    problem.stats["arc_length_iters"] = it
    return u, lam, dir_u, dir_lam


def arc_length_solver_disp_driven(problem, prev_u_vec, prev_lamda, prev_Delta_u_vec, prev_Delta_lamda,
                                  Delta_l=0.1, psi=1.0, tol=1e-6, max_iter=100, solver_options=None):
    """``solver.py:447-517``: one arc-length step under displacement control -- the BC
    values scaled by lambda, constraint |Du|^2 + psi^2 Dlambda^2 |u_b|^2 = Delta_l^2.
    Returns (u_vec, lamda, Delta_u_vec, Delta_lamda), u_vec flat on the device.
    ``max_iter`` is a cap the reference does not have."""
    return _arc_length(problem, prev_u_vec, prev_lamda, prev_Delta_u_vec, prev_Delta_lamda, Delta_l, psi, tol,
                       max_iter, solver_options, None)


def arc_length_solver_force_driven(problem, prev_u_vec, prev_lamda, prev_Delta_u_vec, prev_Delta_lamda, q_vec,
                                   Delta_l=0.1, psi=1.0, tol=1e-6, max_iter=100, solver_options=None):
    """``solver.py:522-590``: one arc-length step under load control, equilibrium
    res(u) + lambda q = 0 with q's BC rows zeroed."""
    return _arc_length(problem, prev_u_vec, prev_lamda, prev_Delta_u_vec, prev_Delta_lamda, Delta_l, psi, tol,
                       max_iter, solver_options, q_vec)


def get_q_vec(problem):
    """``solver.py:593-602``: the residual at u = 0."""
    u = torch.zeros(problem.num_total_dofs_all_vars, dtype=torch.float64, device=problem.device)
    return problem.newton_update(problem.unflatten_fn_sol_list(u))[0].reshape(-1).clone()


def _row_abs_sum(problem, values):
    """sum_j |A_ij| of the device matrix (``np.absolute(KCSR).sum(axis=1)``)."""
    rows = problem._bufs.get("csr_rows")
    if rows is None:
        indptr, _ = problem.csr_arrays()
        rows = torch.from_numpy(np.repeat(np.arange(len(indptr) - 1), np.diff(indptr))).to(problem.device)
        problem._bufs["csr_rows"] = rows
    out = torch.zeros(problem.num_total_dofs_all_vars, dtype=torch.float64, device=problem.device)
    out.index_add_(0, rows, values[problem.csr_map()].abs())
    return out


def assembleCSR(problem, dofs):
    """``solver.py:607-623``: the tangent at dofs with unit BC rows (here on the device)."""
    _, A = _tangent_bc(problem, _flat(dofs, problem.device))
    return A


def calC(t, cmin, cmax):
    """``solver.py:626-634``: damping c = 2 sqrt(t) clipped to [cmin, cmax]."""
    t = max(t, 0.0)
    return min(max(2.0 * math.sqrt(t), cmin), cmax)


def dynamic_relax_solve(problem, tol=1e-6, nKMat=50, nPrint=500, info=True, info_force=True, initial_guess=None,
                        max_iter=1000000, solver_options=None):
    """``solver.py:656-795``: one linear step from u = 0, then damped explicit
    pseudo-dynamics with the lumped mass M = h~^2/4 sum_j |K_ij| until max|R| <= tol.  The
    reference's update sets qdot_old = qdot before qdotdot = qdot - qdot_old, so its
    pseudo-acceleration is zero and the mass is never re-formed; this keeps that order.
    Returns the (num_nodes, 3) solution; ``max_iter`` is a cap the reference does not have.
    Progress goes to the module logger every ``nPrint`` iterations."""
    import logging
    log = logging.getLogger(__name__)
    dev = problem.device
    n = problem.num_total_dofs_all_vars
    dofs = torch.zeros(n, dtype=torch.float64, device=dev)
    res, A = _tangent_bc(problem, dofs)
    x0 = initial_increment(problem, dofs).clone()
    opts = {k: (dict(v) if isinstance(v, dict) else v) for k, v in (solver_options or DIRECT_SOLVE).items()}
    dofs = dofs + linear_solver(problem, A, torch.neg(res), x0, opts)
    if initial_guess is not None:
        dofs = assign_bc(initial_guess, problem)
    cmin, cmax, h_tilde, h = 1e-3, 3.9, 1.1, 1.0
    idx, _ = _bc_index(problem)

    def vec(d):
        r, _, status = problem.assemble(d, need_tangent=False)
        problem._check_status(status)
        r = r.reshape(-1).clone()
        r[idx] = 0.0
        return r

    def mass(d):
        _, K = _tangent_bc(problem, d)
        return h_tilde * h_tilde / 4.0 * _row_abs_sum(problem, K.values)
    R = vec(dofs)
    M = mass(dofs)
    q = dofs.clone()
    qdot = -h / 2.0 * R / M
    qdot_old = torch.zeros_like(q)
    qdotdot = torch.zeros_like(q)
    qdotdot_old = torch.zeros_like(q)
    nIters = iKMat = 0
    error = float(R.abs().max())
    while error > tol:
        if nIters >= max_iter:
            raise RuntimeError(f"dynamic relaxation did not converge in {max_iter} iterations (max|R| = {error})")
        q_old, R_old = q.clone(), R
        q = q + h * qdot
        dofs = q.clone()
        R = vec(dofs)
        nIters += 1
        iKMat += 1
        S0 = torch.dot((R - R_old) / h, qdot)
        den = torch.dot(qdot * M, qdot)
        dq = q - q_old
        ratio = torch.where(dq != 0, (qdotdot - qdotdot_old) / torch.where(dq != 0, dq, torch.ones_like(dq)),
                            torch.zeros_like(dq))
        stats = torch.stack([R.abs().max(), S0, den, ratio.abs().max()]).cpu().numpy()
        error = float(stats[0])
        t = float(stats[1] / stats[2])
        c = calC(t, cmin, cmax)
        if h_tilde * h_tilde / 4.0 * float(stats[3]) > 1 and iKMat > nKMat:
            iKMat = 0
            M = mass(dofs)
        qdot_old = qdot.clone()
        qdotdot_old = qdotdot.clone()
        qdot = (2.0 - c * h) / (2.0 + c * h) * qdot_old - 2.0 * h / (2.0 + c * h) * R / M
        qdot_old = qdot.clone()
        qdotdot = qdot - qdot_old
        if (info or info_force) and nIters % nPrint == 1:
            log.info("DR iteration %d: max force (residual) %g (tol %g), damping t %g, c %g", nIters, error, tol, t, c)
    if not math.isfinite(error):
        raise FloatingPointError("dynamic relaxation produced a non-finite residual")
    problem.stats["dr_iters"] = nIters
    return problem.unflatten_fn_sol_list(dofs)[0]
