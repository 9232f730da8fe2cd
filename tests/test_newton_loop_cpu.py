"""The global Newton loop's control flow (``crystal_plasticity_OR_design/solver.py:310-437``)
and the checks of deferred Krylov solves, on the CPU: the device passes are replaced by a
diagonal stand-in system f(u) = u^3 + u - c, so the loop's decisions (stop rule, the
residual-only last pass, the next solve queued ahead of the norm read, the redo of an
iteration whose deferred solve fails its check, the iteration limit, the load step's
predictor fallback) run as they do on the GPU."""
import ctypes
import importlib
import math

import pytest
import torch


@pytest.fixture(scope="module")
def solver_mod(pkg):
    return importlib.import_module("jax-cpfem_gb300.solver")


@pytest.fixture(scope="module")
def capi(pkg):
    return importlib.import_module("jax-cpfem_gb300._capi")


C = torch.tensor([2.0, 10.0, -3.0], dtype=torch.float64)


class StandIn:
    """What the Newton loop reads of a problem, with a log of the passes it asks for."""

    def __init__(self, fail_solves=(), queue_next_solve=True):
        self.num_total_dofs_all_vars = 3
        self.num_nodes = 1
        self.device = torch.device("cpu")
        self.stats = {"krylov_iters": []}
        self._pending_solve = None
        self.queue_next_solve = queue_next_solve
        self.fail_solves = set(fail_solves)
        self.solves = []          # the deferred flag of every linear solve
        self.log = []             # "tangent", "residual", "solve", "wait" in the order asked for

    def unflatten_fn_sol_list(self, dofs):
        return [dofs.reshape(self.num_nodes, 3)]

    def _check_status_bits(self, word):
        assert word == 0


def _f(u):
    return u ** 3 + u - C


@pytest.fixture
def stand_in(solver_mod, monkeypatch):
    def update(problem, dofs):
        problem.log.append("tangent")
        return _f(dofs), 3.0 * dofs ** 2 + 1.0, None

    def residual(problem, dofs):
        problem.log.append("residual")
        return _f(dofs), None

    class NormCopy:
        """The norm's copy to the host; the value is ready at once on the CPU."""

        def __init__(self, problem, x, status):
            self.problem, self.sq = problem, float(x @ x)

        def wait(self):
            self.problem.log.append("wait")
            return self.sq, 0

    def resolve(problem):
        # the report of the deferred solve this norm follows
        p = problem._pending_solve
        if p is None:
            return
        problem._pending_solve = None
        if p["fail"]:
            raise solver_mod.DeferredSolveFailed("planted")
        problem.stats["krylov_iters"].append(p["n"])

    def incremental(problem, res_vec, A, dofs, solver_options, deferred=False):
        problem.solves.append(deferred)
        problem.log.append("solve")
        n = len(problem.solves)
        if deferred:
            problem._pending_solve = {"fail": n in problem.fail_solves, "n": n}
            if n in problem.fail_solves:
                return dofs + 100.0      # what a failed solve leaves must not survive
        return dofs - res_vec / A

    monkeypatch.setattr(solver_mod, "_update_deferred", update)
    monkeypatch.setattr(solver_mod, "_residual_deferred", residual)
    monkeypatch.setattr(solver_mod, "_NormCopy", NormCopy)
    monkeypatch.setattr(solver_mod, "resolve_deferred", resolve)
    monkeypatch.setattr(solver_mod, "linear_incremental_solver", incremental)
    return solver_mod


def _reference_newton(tol, rel_tol):
    """The reference loop written out: iterate while both stop tests fail."""
    u = torch.zeros(3, dtype=torch.float64)
    r0 = float(torch.linalg.norm(_f(u)))
    r, it = r0, 0
    while r / r0 > rel_tol and r > tol:
        u = u - _f(u) / (3.0 * u ** 2 + 1.0)
        r = float(torch.linalg.norm(_f(u)))
        it += 1
    return u, it


@pytest.mark.parametrize("ahead", [True, False])
def test_loop_matches_the_reference_iteration(stand_in, ahead):
    prob = StandIn(queue_next_solve=ahead)
    sol = stand_in.solver(prob, {"tol": 1e-10, "rel_tol": 1e-14})[0].reshape(-1)
    u, it = _reference_newton(1e-10, 1e-14)
    assert torch.equal(sol, u)
    assert prob.stats["newton_iters"] == it
    assert all(prob.solves) and len(prob.solves) == it   # every solve deferred, none dropped
    assert prob.stats["krylov_iters"] == list(range(1, it + 1))   # every report read, in order
    # the last iterate, predicted converged, gets a residual-only pass
    assert prob.stats.get("final_tangent_skipped", 0) == 1 and prob.log.count("residual") == 1
    assert prob.log.count("tangent") == it                # the first system and every iterate but the last
    assert prob.stats["res_history"][-1] < 1e-10
    # ahead: each tangent pass queues the next solve before its norm is read
    pattern = ["tangent", "solve", "wait"] if ahead else ["tangent", "wait", "solve"]
    tp = [i for i, e in enumerate(prob.log) if e == "tangent"]
    assert all(prob.log[i:i + 3] == pattern for i in tp)
    assert "solves_dropped" not in prob.stats and prob._pending_solve is None


def test_unexpected_convergence_drops_the_queued_solve(stand_in):
    """A guess that already meets the limit: the solve queued behind the first norm is
    dropped, and the guess is returned."""
    prob = StandIn()
    sol = stand_in.solver(prob, {"tol": 20.0, "rel_tol": 1e-14})[0].reshape(-1)
    assert torch.equal(sol, torch.zeros(3, dtype=torch.float64)) and prob.stats["newton_iters"] == 0
    assert prob.stats["solves_dropped"] == 1 and prob.solves == [True] and prob.stats["krylov_iters"] == []
    assert prob._pending_solve is None


@pytest.mark.parametrize("ahead", [True, False])
@pytest.mark.parametrize("fail", [1, 2, 3])
def test_failed_deferred_solve_redoes_the_iteration(stand_in, ahead, fail):
    clean = StandIn()
    ref = stand_in.solver(clean, {"tol": 1e-10, "rel_tol": 1e-14})[0]
    prob = StandIn(fail_solves={fail}, queue_next_solve=ahead)
    sol = stand_in.solver(prob, {"tol": 1e-10, "rel_tol": 1e-14})[0]
    assert torch.equal(sol, ref)                          # the failed increment left no trace
    assert prob.stats["deferred_redone"] == 1
    assert prob.stats["newton_iters"] == clean.stats["newton_iters"]
    assert prob.solves.count(False) == 1                  # the redo is a checked solve
    assert prob.solves[fail - 1] is True
    # the failed solve and (ahead) the one queued behind it are never counted
    assert fail not in prob.stats["krylov_iters"]
    assert len(prob.stats["krylov_iters"]) == clean.stats["newton_iters"] - 1


def test_iteration_limit(stand_in):
    with pytest.raises(RuntimeError, match="did not converge"):
        stand_in.solver(StandIn(), {"tol": 1e-30, "rel_tol": 1e-30, "max_newton": 3})


def test_defers_only_the_plain_device_solve(solver_mod):
    class P:
        pass

    p = P()
    assert solver_mod._defers(p, {})
    assert solver_mod._defers(p, {"jax_solver": {}})
    assert not solver_mod._defers(p, {"jax_solver": {}, "line_search_flag": True})
    assert not solver_mod._defers(p, {"custom_solver": lambda *a: None})
    p.defer_krylov_checks = False
    assert not solver_mod._defers(p, {})


def _report(capi, monkeypatch, solver_mod, **fields):
    buf = torch.zeros(ctypes.sizeof(capi.SolveReport), dtype=torch.uint8)
    r = capi.SolveReport.from_address(buf.data_ptr())
    for k, v in dict(k=7, error=0, rs=1e-22, atol2=1e-20, true_rs=1e-22, bb=1.0).items():
        setattr(r, k, fields.get(k, v))
    monkeypatch.setattr(solver_mod, "_report_buffer", lambda problem, slot=0: buf)


def _pending(fp32):
    class P:
        pass

    p = P()
    p.stats = {"krylov_iters": []}
    p._pending_solve = {"fp32": fp32, "tol": 1e-4, "atol": 1e-10}
    return p


def test_resolve_deferred_accepts_a_converged_report(solver_mod, capi, monkeypatch):
    _report(capi, monkeypatch, solver_mod)
    p = _pending(True)
    solver_mod.resolve_deferred(p)
    assert p.stats["krylov_iters"] == [7] and p._pending_solve is None
    solver_mod.resolve_deferred(p)                        # nothing pending: no second count
    assert p.stats["krylov_iters"] == [7]


@pytest.mark.parametrize("fields, fp32, fallback", [
    ({"error": 1}, False, False),                         # a grid barrier timed out
    ({"true_rs": 0.04}, False, False),                    # ||b - Ax|| = 0.2 fails jax_solve's 0.1
    ({"true_rs": -1.0}, False, False),                    # no true residual (NaN)
    ({"rs": 1e-18}, True, True),                          # FP32 V-cycle: not converged
    ({"true_rs": 1e-4}, True, True),                      # FP32 V-cycle: true residual off the stop rule
])
def test_resolve_deferred_rejects(solver_mod, capi, monkeypatch, fields, fp32, fallback):
    _report(capi, monkeypatch, solver_mod, **fields)
    p = _pending(fp32)
    with pytest.raises(solver_mod.DeferredSolveFailed):
        solver_mod.resolve_deferred(p)
    assert p._pending_solve is None and p.stats["krylov_iters"] == []
    assert getattr(p, "mg_fp64_only", False) == fallback


def test_fp32_stop_rule(solver_mod):
    ok = solver_mod._fp32_solve_ok
    assert ok(True, 1e-5, 1.0, 1e-4, 1e-10)                # within the factor 10 of tol*||b||
    assert not ok(True, 2e-3, 1.0, 1e-4, 1e-10)
    assert not ok(False, 1e-9, 1.0, 1e-4, 1e-10)
    assert not ok(True, math.nan, 1.0, 1e-4, 1e-10)
    assert ok(True, 5e-10, 0.0, 1e-4, 1e-10)               # b = 0: the absolute limit


def test_predictor_fallback(pkg):
    """A load step whose solve fails from the extrapolated guess is solved again from the
    last solution; a failure from the last solution itself is raised."""
    workloads = importlib.import_module("jax-cpfem_gb300.workloads")

    class Solver:
        def __init__(self, bad):
            self.bad, self.starts = bad, []

        def solver(self, problem, opts):
            g = opts["initial_guess"][0]
            self.starts.append(g)
            if any(g.data_ptr() == b.data_ptr() for b in self.bad):
                raise RuntimeError("global Newton did not converge")
            return [g + 1.0]

    last = torch.zeros(2, 3, dtype=torch.float64)
    guess = torch.ones(2, 3, dtype=torch.float64)
    prob = StandIn()
    s = Solver(bad=[guess])
    out = workloads.solve_with_fallback(s, prob, {"tol": 1e-8}, guess, last)
    assert torch.equal(out, last + 1.0) and prob.stats["predictor_fallbacks"] == 1
    assert len(s.starts) == 2 and s.starts[1].data_ptr() == last.data_ptr()
    prob = StandIn()
    out = workloads.solve_with_fallback(Solver(bad=[]), prob, {}, guess, last)
    assert torch.equal(out, guess + 1.0) and "predictor_fallbacks" not in prob.stats
    with pytest.raises(RuntimeError):
        workloads.solve_with_fallback(Solver(bad=[last]), StandIn(), {}, last, last)
