"""Arc-length continuation and dynamic relaxation (``crystal_plasticity_OR_design/solver.py:
447-795``) on the GPU against the oracle's restatement of the same algorithms (scipy's sparse
LU standing in for UMFPACK on the oracle side, the device BiCGSTAB to 1e-12 on the GPU
side).  A 2^3 polycrystal of the steel-like FCC material with 3 grains, states committed
between steps as a driver would; compared per step: u and lambda (arc length), and the final
solution and iteration count (dynamic relaxation)."""
import numpy as np
import pytest
import torch

from oracle import cpfem_oracle as O
from tests.common import gpu_problem, oracle_problem, roller_bcs

pytestmark = pytest.mark.gpu


def _case(pkg):
    spec = pkg.material.BENCH_STEEL
    mesh = pkg.box_mesh(2, 2, 2)
    ori, rng = pkg.mesh.voronoi_grains(mesh, 3, 7)
    quat = pkg.material.random_quaternions(rng, 3)
    return spec, mesh, quat, ori


def _pair(pkg, gpu, bcs):
    problem_mod, _ = gpu
    spec, mesh, quat, ori = _case(pkg)
    prob = gpu_problem(pkg, problem_mod, spec, mesh, quat, ori, bcs)
    orc = oracle_problem(spec, mesh, quat, ori, bcs)
    prob.dt = orc.dt = 0.1
    return prob, orc, mesh


def _rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    return float(np.abs(a - b).max() / np.abs(b).max())


def _steps(prob, orc, solver_mod, n, gpu_step, orc_step):
    """n continuation steps on both sides, each followed by a state commit."""
    z = np.zeros(orc.ndof)
    uo, lo, duo, dlo = z, 0.0, z, 0.0
    ug = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64, device=prob.device)
    lg, dug, dlg = 0.0, ug.clone(), 0.0
    pg, po = prob.internal_vars, orc.internal_vars
    out = []
    for _ in range(n):
        prob.set_params(pg)
        orc.set_params(po)
        ug, lg, dug, dlg = gpu_step(ug, lg, dug, dlg)
        uo, lo, duo, dlo = orc_step(uo, lo, duo, dlo)
        out.append((_rel(ug, uo), abs(lg - lo) / abs(lo)))
        pg = prob.update_int_vars_gp(ug.reshape(-1, 3), pg)
        po = orc.update_int_vars_gp(uo, po)
    return out, po


def test_arc_length_displacement_control(pkg, gpu):
    _, solver_mod = gpu
    spec, mesh, _, _ = _case(pkg)
    prob, orc, mesh = _pair(pkg, gpu, roller_bcs(pkg.mesh, mesh.points, 2e-3))
    nb = float(np.linalg.norm(O._bc_vector(orc, orc.ndof)))
    dl = 0.4 * nb
    errs, po = _steps(prob, orc, solver_mod, 4,
                      lambda u, l, du, dlm: solver_mod.arc_length_solver_disp_driven(prob, u, l, du, dlm, dl,
                                                                                     tol=1e-8),
                      lambda u, l, du, dlm: O.arc_length_disp(orc, u, l, du, dlm, dl, tol=1e-8))
    assert po[1].max() > spec.gss_initial * 1.001   # the steps reach the plastic range
    for eu, el in errs:
        assert eu < 1e-8 and el < 1e-9, errs


def test_arc_length_load_control(pkg, gpu):
    _, solver_mod = gpu
    spec, mesh, _, _ = _case(pkg)
    P = mesh.points
    fn = pkg.mesh.face_nodes
    bcs = [(fn(P, 0, 0.0), 0, 0.0), (fn(P, 1, 0.0), 1, 0.0), (fn(P, 2, 0.0), 2, 0.0)]
    prob, orc, mesh = _pair(pkg, gpu, bcs)
    # a unit total pull on the top face, as consistent nodal forces of uniform traction
    cnt = np.zeros(P.shape[0])
    for c in mesh.cells:
        on = [n for n in c if abs(P[n, 2] - 1.0) < 1e-9]
        if len(on) == 4:
            cnt[on] += 1
    q = np.zeros(orc.ndof)
    q[3 * np.arange(P.shape[0]) + 2] = -cnt / cnt.sum()
    qg = torch.tensor(q, device=prob.device)
    dl = 70.0 * float(np.linalg.norm(q))
    errs, po = _steps(prob, orc, solver_mod, 4,
                      lambda u, l, du, dlm: solver_mod.arc_length_solver_force_driven(prob, u, l, du, dlm, qg, dl,
                                                                                      tol=1e-8),
                      lambda u, l, du, dlm: O.arc_length_force(orc, u, l, du, dlm, q, dl, tol=1e-8))
    assert po[1].max() > spec.gss_initial * 1.001
    for eu, el in errs:
        assert eu < 1e-8 and el < 1e-9, errs


@pytest.mark.parametrize("disp", [1e-3, 2.5e-3])
def test_dynamic_relaxation(pkg, gpu, disp):
    _, solver_mod = gpu
    _, mesh, _, _ = _case(pkg)
    prob, orc, mesh = _pair(pkg, gpu, roller_bcs(pkg.mesh, mesh.points, disp))
    ug = solver_mod.dynamic_relax_solve(prob, tol=1e-7, info=False, info_force=False)
    uo, its = O.dynamic_relax(orc, tol=1e-7)
    assert abs(prob.stats["dr_iters"] - its) <= 1
    assert _rel(ug.reshape(-1), uo) < 1e-8
    # and it is the equilibrium the Newton solver finds, to the residual tolerance's effect
    un, _ = O.solver(orc, {"tol": 1e-10, "rel_tol": 1e-14})
    assert _rel(ug.reshape(-1), un) < 1e-6
