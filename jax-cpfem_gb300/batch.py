"""Ragged batches of independent RVEs solved together.

Many RVEs (a UQ or calibration sweep: different sizes, grain maps and Kalidindi
parameters) run as one problem on the concatenated mesh: one constitutive launch over
every Gauss point of every instance (per-instance parameters through the parameter-index
table), one element-assembly launch, a block-diagonal matrix, and a batched BiCGSTAB that
gives every instance its own scalars and stop test (a team of blocks per instance, sized
by the instance's nodes times its last Krylov count).  Each instance keeps the reference's global-Newton
semantics (``crystal_plasticity_OR_design/solver.py:407``): it stops iterating when its own
``rel_res <= rel_tol or res <= tol``; converged instances get a zero increment.
"""
from __future__ import annotations

import contextlib
import dataclasses
import math
import time

import numpy as np
import torch

from . import _capi
from .material import MaterialSpec, random_quaternions
from .mesh import Mesh, box_mesh, face_nodes, voronoi_grains
from .problem import CrystalPlasticity, DeviceCSR, _stream
from . import solver as _solver
from .workloads import solve_with_fallback as _solve_with_fallback


@dataclasses.dataclass
class Instance:
    edge: int
    grains: int
    seed: int
    material: MaterialSpec


def sample_instances(count, base: MaterialSpec, seed=0, edges=(8, 12, 16, 20, 24), grains=(8, 64), spread=0.2):
    """The batch of the benchmark configuration: edge uniform in ``edges``, grain count
    uniform in [grains], every Kalidindi parameter scaled by U(1-spread, 1+spread)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        f = rng.uniform(1 - spread, 1 + spread, size=5)
        mat = base.replace(h=base.h * f[0], gss_initial=base.gss_initial * f[1], t_sat=base.t_sat * f[2],
                           gss_a=base.gss_a * f[3], xm=base.xm * f[4])
        out.append(Instance(int(rng.choice(edges)), int(rng.integers(grains[0], grains[1] + 1)),
                            int(rng.integers(0, 2 ** 31 - 1)), mat))
    return out


def build_instance(inst: Instance):
    mesh = box_mesh(inst.edge, inst.edge, inst.edge)
    ori, rng = voronoi_grains(mesh, inst.grains, inst.seed)
    quat = random_quaternions(rng, inst.grains)
    return mesh, quat, ori


class Batch:
    """All instances on one concatenated mesh."""

    def __init__(self, instances, device=None):
        self.instances = list(instances)
        base = self.instances[0].material
        for it in self.instances:
            if (it.material.slip, it.material.C11, it.material.C12, it.material.C44, it.material.coplanar_q) != \
                    (base.slip, base.C11, base.C12, base.C44, base.coplanar_q):
                raise ValueError("instances of one batch share the slip systems and elastic constants")
        pts, cells, quats, oris = [], [], [], []
        node_off, cell_off, grain_off = [0], [0], 0
        self.meshes = []
        for it in self.instances:
            mesh, quat, ori = build_instance(it)
            self.meshes.append((mesh, quat, ori))
            pts.append(mesh.points)
            cells.append(mesh.cells + node_off[-1])
            quats.append(quat)
            oris.append(ori + grain_off)
            grain_off += quat.shape[0]
            node_off.append(node_off[-1] + mesh.points.shape[0])
            cell_off.append(cell_off[-1] + mesh.cells.shape[0])
        self.mesh = Mesh(np.concatenate(pts), np.concatenate(cells))
        self.problem = CrystalPlasticity(self.mesh, additional_info=(np.concatenate(quats), np.concatenate(oris)),
                                         material=base, device=device)
        p = self.problem
        dev = p.device
        self.n = len(self.instances)
        self.node_off_np = np.asarray(node_off, dtype=np.int64)
        self.cell_off_np = np.asarray(cell_off, dtype=np.int64)
        self.node_off = torch.tensor(node_off, dtype=torch.int32, device=dev)
        self.dof_off = torch.tensor(3 * self.node_off_np, dtype=torch.int64, device=dev)
        # per-instance Kalidindi parameters and initial slip resistance
        p.param_table = torch.tensor(np.stack([it.material.param_row() for it in self.instances]),
                                     dtype=torch.float64, device=dev)
        inst_of_cell = np.repeat(np.arange(self.n), np.diff(self.cell_off_np))
        p.param_idx = torch.tensor(np.repeat(inst_of_cell, 8), dtype=torch.int32, device=dev)
        g0 = torch.tensor([it.material.gss_initial for it in self.instances], dtype=torch.float64, device=dev)
        p.g = g0[p.param_idx.long()].expand(p.num_slip, -1).contiguous()
        p._views = None
        self.inst_of_cell = torch.tensor(inst_of_cell, dtype=torch.int64, device=dev)
        self.cells_per_inst = torch.tensor(np.diff(self.cell_off_np), dtype=torch.float64, device=dev)
        # Dirichlet faces of every unit-cube instance (rollers + pulled top)
        self.faces = []
        for k, (mesh, _, _) in enumerate(self.meshes):
            o = self.node_off_np[k]
            P = mesh.points
            self.faces.append([face_nodes(P, 0, 0.0) + o, face_nodes(P, 1, 0.0) + o, face_nodes(P, 2, 0.0) + o,
                               face_nodes(P, 2, 1.0) + o])
        self.order = np.argsort(-np.diff(self.node_off_np), kind="stable")   # largest first
        self.sol = torch.zeros(p.num_total_dofs_all_vars, dtype=torch.float64, device=dev)
        self.prev = None
        # the initial guess of each step's Newton solve: the last solution ("previous", the
        # reference driver's) or 2 u_n - u_(n-1) ("linear", as workloads.LoadStepper)
        self.predictor = "previous"
        self.params = p.internal_vars
        self.stats = {"newton_iters": [], "krylov_iters": []}
        self.host_s = {}
        self._last_iters = np.zeros(self.n, dtype=np.float64)

    @contextlib.contextmanager
    def _phase(self, name):
        """Wall-clock time of a solve phase (synchronised) when the problem is timing."""
        if not self.problem.timing:
            yield
            return
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        yield
        torch.cuda.synchronize()
        self.host_s[name] = self.host_s.get(name, 0.0) + time.perf_counter() - t0

    def set_bcs(self, disp):
        nodes, comps, vals = [], [], []
        for f in self.faces:
            nodes += f
            comps += [0, 1, 2, 2]
            vals += [0.0, 0.0, 0.0, disp]
        self.problem.fes[0].set_dirichlet_lists(nodes, comps, vals)

    def _assemble(self, dofs, trial, cells=None):
        """Residual and BC-eliminated tangent at dofs; with ``cells`` only those cells'
        GPs are re-evaluated (the others keep their outputs in the persistent buffers)."""
        p = self.problem
        res, values, status = p.assemble(dofs, need_tangent=True, cell_list=cells, trial=trial)
        p._check_status(status)
        p.A_values = values
        res = res.reshape(-1)
        p.apply_dirichlet(res, dofs, values)
        return res, DeviceCSR(p, values)

    def _cells_of(self, inst):
        c = np.concatenate([np.arange(self.cell_off_np[i], self.cell_off_np[i + 1], dtype=np.int32)
                            for i in np.sort(inst)])
        return torch.from_numpy(c).to(self.problem.device)

    def _norms(self, res):
        p = self.problem
        out = torch.empty(self.n, dtype=torch.float64, device=p.device)
        _capi.check(p.lib.cpfem_segmented_dot(self.n, self.dof_off.data_ptr(), res.data_ptr(), res.data_ptr(),
                                              out.data_ptr(), _stream()))
        return torch.sqrt(out).cpu().numpy()

    def solve(self, **options):
        """Batched global Newton for the current BCs, dt and state (options of
        ``_solve_from``), from the extrapolated guess under the ``"linear"`` predictor; if
        that fails (an instance's extrapolation overshot into a state a local solve cannot
        reach), again from the last solution, the reference driver's guess."""
        # as workloads.LoadStepper: under the extrapolated guess, local starts are predicted
        # from the second Newton pass of a step on
        self.problem.predict_from_pass = 1 if self.predictor == "linear" else 2
        if self.predictor == "linear" and self.prev is not None:
            try:
                return self._solve_from(2.0 * self.sol - self.prev, **options)
            except (RuntimeError, FloatingPointError):
                self.stats["predictor_fallbacks"] = self.stats.get("predictor_fallbacks", 0) + 1
        return self._solve_from(self.sol.clone(), **options)

    def _solve_from(self, dofs, rel_tol=1e-8, tol=1e-6, precond=1, ktol=1e-10, katol=1e-10, maxiter=10000,
                    max_newton=100):
        p = self.problem
        lib = p.lib
        trial = p.new_trial()
        with self._phase("assemble"):
            res, A = self._assemble(dofs, trial)
            r0 = self._norms(res)
        rn = r0.copy()
        with np.errstate(invalid="ignore", divide="ignore"):
            active = (rn / r0 > rel_tol) & (rn > tol)
        nws = int(lib.cpfem_bicgstab_batched_workspace_bytes(p.num_nodes))
        ws = p._buf("batched_ws", (nws // 8 + 64,))
        info = np.zeros(2 * self.n, dtype=np.int32)
        node_off = np.ascontiguousarray(self.node_off_np, dtype=np.int32)
        nodes = np.diff(self.node_off_np).astype(np.float64)
        its = 0
        newton_count = np.zeros(self.n, dtype=np.int64)
        while active.any():
            if its >= max_newton:
                raise RuntimeError("batched global Newton did not converge")
            act = np.ascontiguousarray(self.order[active[self.order]], dtype=np.int32)
            # work estimate per instance: nodes x its last Krylov count (nodes^(4/3) before any)
            wts = np.ascontiguousarray(nodes[act] * np.where(self._last_iters[act] > 0, self._last_iters[act],
                                                             nodes[act] ** (1.0 / 3.0)))
            b = torch.neg(res)
            x = _solver.initial_increment(p, dofs).clone()
            with self._phase("krylov"), p.region("bicgstab_batched"):
                _capi.check(lib.cpfem_bicgstab_batched(p.sell, A.values.data_ptr(), b.data_ptr(), x.data_ptr(),
                                                       int(precond), float(ktol), float(katol), int(maxiter),
                                                       self.n, node_off.ctypes.data, int(act.size), act.ctypes.data,
                                                       wts.ctypes.data, ws.data_ptr(), info.ctypes.data, _stream()))
            inf = info.reshape(self.n, 2)
            self._last_iters[act] = np.maximum(inf[act, 0], 1)
            if not inf[act, 1].all():
                raise RuntimeError("a batched linear solve did not converge")
            self.stats["krylov_iters"].append(inf[act, 0].copy())
            _capi.check(lib.cpfem_axpy(dofs.numel(), 1.0, x.data_ptr(), dofs.data_ptr(), _stream()))
            newton_count[act] += 1
            with self._phase("assemble"):
                # converged instances keep their state: only the active ones are re-evaluated
                cells = None if act.size == self.n else self._cells_of(act)
                res, A = self._assemble(dofs, trial, cells)
                rn = self._norms(res)
            if not np.isfinite(rn[active]).all():
                raise FloatingPointError("non-finite residual in the batch")
            active = active & (rn / r0 > rel_tol) & (rn > tol)
            its += 1
        self.stats["newton_iters"].append(newton_count)
        return dofs

    def step(self, disp, dt, **solve_options):
        """One load step of every instance; returns the per-instance mean cell sigma_zz.
        ``solve_options`` go to ``solve`` (rel_tol, tol, ktol, ...)."""
        p = self.problem
        p.dt = float(dt)
        with self._phase("bcs"):
            self.set_bcs(disp)
            p.set_params(self.params)
        sol = self.solve(**solve_options)
        with self._phase("post"):
            sig = p.compute_avg_stress(sol.reshape(-1, 3), self.params)
            self.params = p.update_int_vars_gp(sol.reshape(-1, 3), self.params)
        self.prev, self.sol = self.sol, sol
        szz = torch.zeros(self.n, dtype=torch.float64, device=p.device)
        szz.index_add_(0, self.inst_of_cell, sig[:, 2, 2])
        return szz / self.cells_per_inst


def build_serial(instances, device=None):
    """One plain drop-in problem per RVE (the set-up half of ``run_serial``)."""
    out = []
    for it in instances:
        mesh, quat, ori = build_instance(it)
        p = CrystalPlasticity(mesh, additional_info=(quat, ori), material=it.material, device=device)
        P = mesh.points
        out.append((p, [face_nodes(P, 0, 0.0), face_nodes(P, 1, 0.0), face_nodes(P, 2, 0.0), face_nodes(P, 2, 1.0)]))
    return out


def run_serial(instances, disps, dt, device=None, prepared=None, solver_options=None, predictor="previous"):
    """The same RVEs one at a time through the plain drop-in path (``prepared`` from
    ``build_serial`` keeps the problem set-up out of a timed region); ``solver_options`` and
    ``predictor`` as the batch uses them."""
    prepared = prepared if prepared is not None else build_serial(instances, device)
    out = np.zeros((len(prepared), len(disps)))
    base = dict(solver_options or {"jax_solver": {}})
    for k, (p, nodes) in enumerate(prepared):
        params = p.internal_vars
        sol = torch.zeros(p.num_total_dofs_all_vars, dtype=torch.float64, device=p.device)
        prev = None
        p.reset_local_start()
        p.predict_from_pass = 1 if predictor == "linear" else 2
        for i, d in enumerate(disps):
            p.dt = float(dt)
            p.fes[0].set_dirichlet_lists(nodes, [0, 1, 2, 2], [0.0, 0.0, 0.0, float(d)])
            p.set_params(params)
            guess = 2.0 * sol - prev if (predictor == "linear" and prev is not None) else sol
            prev = sol
            sol = _solve_with_fallback(_solver, p, base, guess, sol).reshape(-1)
            sig = p.compute_avg_stress(sol.reshape(-1, 3), params)
            params = p.update_int_vars_gp(sol.reshape(-1, 3), params)
            out[k, i] = float(sig[:, 2, 2].mean())
    return out
