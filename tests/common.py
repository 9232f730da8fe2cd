"""Shared set-up for the parity tests: the same seeded case built for the GPU problem
class and for the CPU oracle."""
import numpy as np

from oracle import cpfem_oracle as O

ORACLE_SLIP = {"fcc12": O.FCC12, "bcc12": O.BCC12, "bcc24": O.BCC24}


def roller_bcs(mesh_pkg, points, disp, L=1.0):
    fn = mesh_pkg.face_nodes
    return [(fn(points, 0, 0.0), 0, 0.0), (fn(points, 1, 0.0), 1, 0.0),
            (fn(points, 2, 0.0), 2, 0.0), (fn(points, 2, L), 2, disp)]


def corner_bcs(mesh_pkg, points, disp, L=1.0):
    c = mesh_pkg.corner_nodes(points, (0.0, 0.0, 0.0))
    return [(c, 0, 0.0), (c, 1, 0.0), (mesh_pkg.face_nodes(points, 2, 0.0), 2, 0.0),
            (mesh_pkg.face_nodes(points, 2, L), 2, disp)]


def oracle_problem(spec, mesh, quat, ori, bcs=()):
    return O.OracleProblem(mesh.points, mesh.cells, ORACLE_SLIP[spec.slip], spec.C11, spec.C12, spec.C44,
                           quat, ori, gss_initial=spec.gss_initial, h=spec.h, t_sat=spec.t_sat,
                           gss_a=spec.gss_a, xm=spec.xm, r=spec.r, ao=spec.ao, coplanar=spec.coplanar_q,
                           local_tol=spec.local_tol, max_sub_step=spec.max_sub_step, bcs=bcs)


def gpu_problem(pkg, problem_mod, spec, mesh, quat, ori, bcs=()):
    p = problem_mod.CrystalPlasticity(mesh, additional_info=(quat, ori), material=spec)
    if bcs:
        p.fes[0].set_dirichlet_lists([b[0] for b in bcs], [b[1] for b in bcs], [b[2] for b in bcs])
    return p


def random_gp_inputs(rng, n, N, strain=1e-3, plastic=True):
    """Random per-GP inputs of one load increment: tension-like F near I with noise,
    a mildly deformed Fp^-1, slip resistances around the flow stress, rotations."""
    ug = np.zeros((n, 3, 3))
    ug[:, 2, 2] = strain
    ug[:, 0, 0] = ug[:, 1, 1] = -0.3 * strain
    ug += 0.3 * strain * rng.normal(size=(n, 3, 3))
    fpi = np.eye(3) + (2e-4 * rng.normal(size=(n, 3, 3)) if plastic else np.zeros((n, 3, 3)))
    g = rng.uniform(60.0, 160.0, size=(n, N))
    slip = rng.normal(scale=1e-3, size=(n, N))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    R = O.rot_mat(q)
    return ug, fpi, g, slip, R


def fast_oracle_problem(spec, mesh, quat, ori, bcs=()):
    """The compiled oracle (same algorithm as ``oracle_problem``, for the large cases)."""
    from oracle import coracle as C
    return C.FastOracleProblem(mesh.points, mesh.cells, ORACLE_SLIP[spec.slip], spec.C11, spec.C12, spec.C44,
                               quat, ori, gss_initial=spec.gss_initial, h=spec.h, t_sat=spec.t_sat,
                               gss_a=spec.gss_a, xm=spec.xm, r=spec.r, ao=spec.ao, coplanar=spec.coplanar_q,
                               local_tol=spec.local_tol, max_sub_step=spec.max_sub_step, bcs=bcs)


def oracle_history(orc, workload, steps, solver_options=None):
    """The reference driver loop on the oracle (``singlecrystal_copper.py:179-233``): per
    step the volume-averaged Cauchy stress (3,3), the solution, and Newton / Krylov counts;
    the final internal variables."""
    sol = np.zeros(orc.ndof)
    params = orc.internal_vars
    vol = orc.jxw.sum(1)
    sig, us, info = [], [], []
    for i in range(steps):
        orc.dt = workload.dt
        orc.set_bcs(workload.bc_triples(workload.strain_step * (i + 1)))
        orc.set_params(params)
        opts = dict(solver_options or {})
        opts["initial_guess"] = sol
        sol, inf = O.solver(orc, opts)
        s = orc.compute_avg_stress(sol, params)
        sig.append(np.einsum("eij,e->ij", s, vol) / vol.sum())
        us.append(sol.copy())
        info.append(inf)
        params = orc.update_int_vars_gp(sol, params)
    return np.array(sig), np.array(us), params, info
