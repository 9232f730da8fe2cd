"""The drop-in boundary as the reference drivers use it.

``test_copper_driver_loop`` runs the load loop of ``singlecrystal_copper/singlecrystal_copper.py``
(:153-233) as written there: the problem is built with ``dirichlet_bc_info`` location and
value functions that take a point, the top displacement function is replaced in the list
and ``fes[0].update_Dirichlet_boundary_conditions`` is called every step, ``solver`` gets
``{'jax_solver': {}, 'initial_guess': sol_list}``, and the driver reads
``compute_avg_stress``, ``update_int_vars_gp`` and ``inspect_interval_vars``.  The only
changes are the imports (the driver's model module and JAX-FEM's ``solver``) and a box mesh
in place of its Neper file.  The stress curve and the displacements are checked against
the oracle on the same mesh and load.

``test_custom_solver_hook`` routes the Newton systems through the ``custom_solver`` hook
of ``crystal_plasticity_OR_design/solver.py:106-109`` with ``GpuBicgstab`` (the binding a
host JAX-FEM driver would add), and ``test_custom_solver_on_host_csr`` gives it a host
scipy CSR matrix as JAX-FEM would.
"""
import importlib

import numpy as onp
import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch

from oracle import cpfem_oracle as O
from tests.common import oracle_problem

pytestmark = pytest.mark.gpu


def _driver(pkg, problem_mod, solver, nsteps, solver_options=None):
    """singlecrystal_copper.py:66-233, with a 4x4x4 box of side 0.1 mm for its Neper mesh."""
    CrystalPlasticity = problem_mod.CrystalPlasticity       # models_copper.CrystalPlasticity
    mesh = pkg.box_mesh(4, 4, 4, 0.1, 0.1, 0.1)
    cell_ori_inds = onp.zeros(mesh.cells.shape[0], dtype=onp.int64)
    quat = onp.array([[1, 0., 0., 0.]])
    Lx = np.max(mesh.points[:, 0])
    Lz = np.max(mesh.points[:, 2])
    disps = np.linspace(0., 0.05 * Lx, 51)
    ts = np.linspace(0., 0.5, 51)

    def bottom(point):
        return np.isclose(point[2], 0., atol=1e-5)

    def top(point):
        return np.isclose(point[2], Lz, atol=1e-5)

    def zero_dirichlet_val(point):
        return 0.

    def get_dirichlet_top(disp):
        def val_fn(point):
            return disp
        return val_fn

    dirichlet_bc_info = [[bottom, bottom, bottom, top, top, top],
                         [0, 1, 2, 0, 1, 2],
                         [zero_dirichlet_val, zero_dirichlet_val, zero_dirichlet_val, zero_dirichlet_val,
                          zero_dirichlet_val, get_dirichlet_top(disps[0])]]
    problem = CrystalPlasticity(mesh, vec=3, dim=3, ele_type='HEX8',
                                dirichlet_bc_info=dirichlet_bc_info, additional_info=(quat, cell_ori_inds))
    sol_list = [np.zeros((problem.fes[0].num_total_nodes, problem.fes[0].vec))]
    params = problem.internal_vars
    stress_zz_plot = np.array([])
    for i in range(nsteps):
        problem.dt = ts[i + 1] - ts[i]
        dirichlet_bc_info[-1][-1] = get_dirichlet_top(disps[i + 1])
        problem.fes[0].update_Dirichlet_boundary_conditions(dirichlet_bc_info)
        problem.set_params(params)
        opts = {'jax_solver': {}, 'initial_guess': sol_list} if solver_options is None else \
            dict(solver_options, initial_guess=sol_list)
        sol_list = solver(problem, solver_options=opts)
        sigma_cell_data = problem.compute_avg_stress(sol_list[0], params)[:, :, :]
        sigma_cell_zz = sigma_cell_data[:, 2, 2]
        stress_zz_plot = np.append(stress_zz_plot, float(sigma_cell_zz.mean()))
        params = problem.update_int_vars_gp(sol_list[0], params)
        F_p_zz, slip_resistance_0, slip_0 = problem.inspect_interval_vars(params)
    return mesh, quat, cell_ori_inds, disps, ts, stress_zz_plot, sol_list[0], problem


def _oracle(pkg, mesh, quat, ori, disps, ts, nsteps):
    spec = pkg.material.COPPER
    orc = oracle_problem(spec, mesh, quat, ori)
    p = mesh.points
    bot, top = O.face_nodes(p, 2, 0.0), O.face_nodes(p, 2, 0.1)
    bcf = lambda d: [(bot, 0, 0.0), (bot, 1, 0.0), (bot, 2, 0.0), (top, 0, 0.0), (top, 1, 0.0), (top, 2, d)]
    sig, u = O.run_load_steps(orc, disps[:nsteps + 1], ts[:nsteps + 1], bcf)
    return sig[:, :, 2, 2].mean(1), u


def test_copper_driver_loop(pkg, gpu):
    problem_mod, solver_mod = gpu
    nsteps = 6
    mesh, quat, ori, disps, ts, szz, sol, problem = _driver(pkg, problem_mod, solver_mod.solver, nsteps)
    szz_o, u_o = _oracle(pkg, mesh, quat, ori, disps, ts, nsteps)
    assert np.abs(szz - szz_o).max() / np.abs(szz_o).max() < 1e-8, (szz, szz_o)
    u = sol.reshape(-1).cpu().numpy()
    assert np.abs(u - u_o).max() / np.abs(u_o).max() < 1e-8
    # the constructor's dirichlet_bc_info reached the device: bottom (3 comps) + top (3 comps)
    n_face = 25
    assert problem.fes[0].bc_dofs.numel() == 6 * n_face


def test_custom_solver_hook(pkg, gpu):
    problem_mod, solver_mod = gpu
    cs = importlib.import_module("jax-cpfem_gb300.custom_solver")
    hook = cs.GpuBicgstab()
    nsteps = 3
    *_, szz_ref, sol_ref, _ = _driver(pkg, problem_mod, solver_mod.solver, nsteps)
    *_, szz, sol, problem = _driver(pkg, problem_mod, solver_mod.solver, nsteps, {'custom_solver': hook})
    assert hook.last_iterations is not None and hook.last_iterations >= 0
    assert np.abs(szz - szz_ref).max() / np.abs(szz_ref).max() < 1e-9
    assert float((sol - sol_ref).abs().max() / sol_ref.abs().max()) < 1e-9


def test_custom_solver_on_host_csr(pkg, gpu):
    """A host scipy CSR Newton matrix (what JAX-FEM's get_A builds) solved on the device,
    against a host direct solve; a non-block pattern is refused."""
    problem_mod, solver_mod = gpu
    cs = importlib.import_module("jax-cpfem_gb300.custom_solver")
    spec = pkg.material.BENCH_STEEL
    mesh = pkg.box_mesh(5, 5, 5)
    ori, rng = pkg.mesh.voronoi_grains(mesh, 4, 3)
    quat = pkg.material.random_quaternions(rng, 4)
    orc = oracle_problem(spec, mesh, quat, ori, bcs=[(O.face_nodes(mesh.points, 2, 0.0), 0, 0.0),
                                                      (O.face_nodes(mesh.points, 2, 0.0), 1, 0.0),
                                                      (O.face_nodes(mesh.points, 2, 0.0), 2, 0.0),
                                                      (O.face_nodes(mesh.points, 2, 1.0), 2, 1e-3)])
    orc.dt = 0.1
    u = np.zeros(orc.ndof)
    u[2::3] = 2e-3 * mesh.points[:, 2]
    res, A = orc.newton_update(u)
    A = O.apply_bc_rows(A, orc.bc_dofs_vals()[0])
    b = -res
    x_ref = spla.spsolve(A.tocsc(), b)
    hook = cs.GpuBicgstab()
    x = hook(A, b, np.zeros_like(b), {})
    assert isinstance(x, np.ndarray)
    assert np.abs(x - x_ref).max() / np.abs(x_ref).max() < 1e-7
    x2 = hook(A, 2.0 * b, np.zeros_like(b), {})     # same pattern: the layout is reused
    assert np.abs(x2 - 2.0 * x_ref).max() / np.abs(x_ref).max() < 1e-7
    with pytest.raises(ValueError):
        hook(sp.random(9, 9, density=0.5, format="csr", random_state=0) + sp.eye(9), np.ones(9), np.zeros(9), {})
