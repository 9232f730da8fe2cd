"""CPU checks of the oracle itself: the reference's golden curves, FD of the tangent,
the BiCGSTAB restatement, rotation conventions."""
import os

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from oracle import cpfem_oracle as O

GOLD = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))


def _one_element(table, C, params, coplanar, tol_local, max_sub):
    pts, cells = O.box_mesh(1, 1, 1)
    return pts, O.OracleProblem(pts, cells, table, *C, [[1, 0, 0, 0]], np.zeros(1, int), coplanar=coplanar,
                                local_tol=tol_local, max_sub_step=max_sub, **params)


def _corner_bcs(pts):
    c = O.corner_nodes(pts, (0, 0, 0))
    return lambda d: [(c, 0, 0.0), (c, 1, 0.0), (O.face_nodes(pts, 2, 0.0), 2, 0.0),
                      (O.face_nodes(pts, 2, 1.0), 2, d)]


def test_golden_case1_copper():
    """calibration_case1: 1-element copper, 20 steps of 1.25e-3, dt 0.125, tol 1e-7."""
    pts, prob = _one_element(O.FCC12, (1.684e5, 1.214e5, 0.754e5),
                             dict(gss_initial=60.8, h=541.5, t_sat=109.8, gss_a=2.5, xm=0.1, r=1.0),
                             False, 1e-8, 5)
    s, _ = O.run_load_steps(prob, np.linspace(0, 0.025, 21), np.linspace(0, 2.5, 21), _corner_bcs(pts),
                            {"tol": 1e-7}, stress_fn=lambda sg: sg[0, 2, 2])
    gold = GOLD["case1_szz"][:20]
    rel = np.abs(s - gold) / np.abs(gold)
    assert rel.max() < 1e-8, rel


def test_golden_case2_tantalum():
    """calibration_case2: 1-element Ta (BCC12), compression 40 steps, global line search."""
    pts, prob = _one_element(O.BCC12, (2.670e5, 1.610e5, 0.825e5),
                             dict(gss_initial=67.4641, h=1959.1320, t_sat=7295.1754, gss_a=200.0,
                                  xm=1.0 / 45.2726, r=1.0), False, 1e-8, 5)
    s, _ = O.run_load_steps(prob, np.linspace(0, -0.10, 41), np.linspace(0, 10.0, 41), _corner_bcs(pts),
                            {"tol": 1e-7, "line_search_flag": True}, stress_fn=lambda sg: sg[0, 2, 2])
    gold = GOLD["case2_szz"][:40]
    rel = np.abs(s - gold) / np.abs(gold)
    assert rel.max() < 1e-10, rel


def _batch(rng, n, table=O.FCC12, plastic=True):
    N = table.shape[0]
    ug = 3e-3 * rng.normal(size=(n, 3, 3))
    fpi = np.eye(3) + (5e-3 * rng.normal(size=(n, 3, 3)) if plastic else 0.0)
    g = rng.uniform(40.0, 160.0, size=(n, N))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    R = O.rot_mat(q)
    P = O.schmid_tensors(table)
    Pr = np.einsum("gia,gjb,kab->gkij", R, R, P)
    Cr = O.rotate_rank4(R, O.cubic_stiffness(168.4e3, 121.4e3, 75.4e3))
    return lambda F: O.GPBatch(F, fpi, g, Pr, Cr, 0.05 * np.ones(n), 1e-3, 0.1), np.eye(3) + ug


def test_tangent_matches_central_differences():
    rng = np.random.default_rng(1)
    mk, F = _batch(rng, 6)
    b = mk(F)
    S, _, ok = O.local_newton(b, 1e-10, 5)
    assert ok.all()
    D = O.tangent(b, S).reshape(-1, 9, 9)
    h = 1e-6
    Dfd = np.empty_like(D)
    for kl in range(9):
        E = np.zeros(9)
        E[kl] = h
        Fp, Fm = F + E.reshape(3, 3), F - E.reshape(3, 3)
        bp, bm = mk(Fp), mk(Fm)
        Sp = O.local_newton(bp, 1e-10, 5)[0]
        Sm = O.local_newton(bm, 1e-10, 5)[0]
        Dfd[:, :, kl] = ((O.first_pk_stress(bp, Sp) - O.first_pk_stress(bm, Sm)) / (2 * h)).reshape(-1, 9)
    rel = np.abs(D - Dfd).max() / np.abs(D).max()
    assert rel < 1e-5, rel


def test_local_newton_zero_strain_gives_zero_stress():
    rng = np.random.default_rng(2)
    mk, F = _batch(rng, 4, plastic=False)
    b = mk(np.broadcast_to(np.eye(3), (4, 3, 3)).copy())
    S, its, ok = O.local_newton(b, 1e-8, 5)
    assert ok.all() and (its == 0).all() and np.abs(S).max() == 0.0


def test_bicgstab_restatement_solves_nonsymmetric_system():
    rng = np.random.default_rng(3)
    n = 60
    A = sp.random(n, n, density=0.1, random_state=4) + sp.eye(n) * 4.0
    A = A.tocsr()
    b = rng.normal(size=n)
    diag = A.diagonal()
    x, k = O.bicgstab(A, b, np.zeros(n), lambda v: v / diag)
    assert k > 0
    x_ref = spla.spsolve(A.tocsc(), b)
    assert np.abs(x - x_ref).max() / np.abs(x_ref).max() < 1e-8


def test_euler_zyx_matches_scipy(pkg):
    from scipy.spatial.transform import Rotation
    ang = np.random.default_rng(5).uniform(-180, 180, size=(7, 3))
    R = pkg.material.euler_zyx_deg(ang)
    R_ref = Rotation.from_euler("zyx", ang, degrees=True).as_matrix()
    assert np.abs(R - R_ref).max() < 1e-14


def test_q_matrix_semantics():
    q = O.q_matrix(12, 1.4, coplanar=True)
    assert q[0, 0] == 1.0 and q[0, 2] == 1.0 and q[0, 3] == 1.4 and q[5, 3] == 1.0 and q[5, 6] == 1.4
    assert (O.q_matrix(12, 1.4, coplanar=False) == 1.4).all()


def test_slip_tables_agree_with_package(pkg):
    for name, tab in (("fcc12", O.FCC12), ("bcc12", O.BCC12), ("bcc24", O.BCC24)):
        assert np.array_equal(np.asarray(pkg.material.SLIP_SYSTEMS[name], float), tab)


def test_box_mesh_matches_package(pkg):
    pts, cells = O.box_mesh(3, 2, 4, 1.0, 2.0, 3.0)
    m = pkg.box_mesh(3, 2, 4, 1.0, 2.0, 3.0)
    assert np.array_equal(pts, m.points) and np.array_equal(cells, m.cells)
    sg, jxw = O.shape_grads_and_jxw(pts, cells)
    sg2, jxw2 = pkg.mesh.shape_grads_jxw(m)
    assert np.abs(sg - sg2).max() < 1e-14 and np.abs(jxw - jxw2).max() < 1e-15
    assert abs(jxw.sum() - 6.0) < 1e-12


def test_euler_generators_match_finite_differences(pkg):
    from importlib import import_module
    adj = import_module("jax-cpfem_gb300.adjoint")
    ang = np.random.default_rng(9).uniform(-90, 90, size=(4, 3))
    W = adj._euler_generators(ang)
    R0 = pkg.material.euler_zyx_deg(ang)
    for k in range(3):
        d = np.zeros(3)
        d[k] = 1e-5
        dR = (pkg.material.euler_zyx_deg(ang + d) - pkg.material.euler_zyx_deg(ang - d)) / 2e-5
        Wfd = dR @ np.swapaxes(R0, -1, -2)
        w = W[:, k]
        skew = np.zeros((4, 3, 3))
        skew[:, 0, 1], skew[:, 0, 2], skew[:, 1, 2] = -w[:, 2], w[:, 1], -w[:, 0]
        skew = skew - np.swapaxes(skew, -1, -2)
        assert np.abs(skew - Wfd).max() < 1e-8


@pytest.mark.parametrize("slip,coplanar", [("fcc12", True), ("bcc24", False)])
def test_compiled_oracle_matches_numpy_oracle(slip, coplanar):
    """The compiled oracle (cpfem_oracle_c.c, the large-case checker and the timed CPU
    baseline) against the numpy oracle it restates: per-GP outputs, the assembled residual
    and CSR tangent (pattern exact), and three load steps of a 3^3 polycrystal."""
    from oracle import coracle as C
    table = {"fcc12": O.FCC12, "bcc24": O.BCC24}[slip]
    pts, cells = O.box_mesh(3, 3, 3)
    rng = np.random.default_rng(5)
    quat = rng.normal(size=(4, 4))
    quat /= np.linalg.norm(quat, axis=1)[:, None]
    ori = rng.integers(0, 4, size=cells.shape[0])
    kw = dict(gss_initial=90.0, h=200.0, t_sat=300.0, gss_a=2.0, xm=0.05, r=1.4, coplanar=coplanar)
    mats = (204.6e3, 137.7e3, 126.2e3)
    a = O.OracleProblem(pts, cells, table, *mats, quat, ori, **kw)
    b = C.FastOracleProblem(pts, cells, table, *mats, quat, ori, **kw)
    for p in (a, b):
        p.dt = 0.1
    u = np.zeros(a.ndof)
    u[2::3] = 3e-3 * pts[:, 2]
    u += 2e-4 * rng.normal(size=u.size)
    r1, A1 = a.newton_update(u)
    r2, A2 = b.newton_update(u)
    A2 = A2.tocsr()
    assert np.array_equal(A1.indptr, A2.indptr) and np.array_equal(A1.indices, A2.indices)
    assert np.abs(r1 - r2).max() < 1e-11 * np.abs(r1).max()
    assert np.abs(A1.data - A2.data).max() < 1e-11 * np.abs(A1.data).max()
    new_a = a.update_int_vars_gp(u, a.internal_vars)
    new_b = b.update_int_vars_gp(u, b.internal_vars)
    for x, y in zip(new_a[:3], new_b[:3]):
        assert np.abs(x - y).max() < 1e-12 * np.abs(x).max()
    sa, sb = a.compute_avg_stress(u, a.internal_vars), b.compute_avg_stress(u, b.internal_vars)
    assert np.abs(sa - sb).max() < 1e-11 * np.abs(sa).max()

    def bcs(d):
        return [(O.face_nodes(pts, 0, 0.0), 0, 0.0), (O.face_nodes(pts, 1, 0.0), 1, 0.0),
                (O.face_nodes(pts, 2, 0.0), 2, 0.0), (O.face_nodes(pts, 2, 1.0), 2, d)]
    ts, disps = 0.1 * np.arange(4), 1e-3 * np.arange(4)
    s1, u1 = O.run_load_steps(a, disps, ts, bcs)
    s2, u2 = O.run_load_steps(b, disps, ts, bcs)
    assert np.abs(s1 - s2).max() < 1e-10 * np.abs(s1).max()
    assert np.abs(u1 - u2).max() < 1e-10 * np.abs(u1).max()


def test_compiled_bicgstab_matches_restatement():
    """The compiled BiCGSTAB runs the numpy restatement's recurrences: same iteration count
    and iterate on a non-symmetric system."""
    from oracle import coracle as C
    rng = np.random.default_rng(3)
    n = 300
    A = sp.random(n, n, density=0.03, random_state=4, format="csr") + sp.diags(4.0 + rng.random(n))
    A = sp.csr_array(A)
    A.sort_indices()
    b = rng.normal(size=n)
    x_ref, k_ref = O.bicgstab(A, b, np.zeros(n), lambda v: v / A.diagonal())
    M = C.CSR(A.indptr.astype(np.int64), A.indices.astype(np.int32), A.data.copy(), n)
    x = np.zeros(n)
    k = np.zeros(1, dtype=np.int32)
    minv = 1.0 / A.diagonal()
    C.load().orc_bicgstab(n, M.indptr.ctypes.data, M.indices.ctypes.data, M.data.ctypes.data, b.ctypes.data,
                          x.ctypes.data, minv.ctypes.data, 1e-10, 1e-10, 10000, k.ctypes.data)
    assert int(k[0]) == k_ref
    assert np.abs(x - x_ref).max() < 1e-9 * np.abs(x_ref).max()


def test_complex_step_history_derivative_matches_central_differences():
    """The oracle's complex-step derivative of a load history (the independent check of the
    GPU adjoint) against central differences of the same oracle, on 2 cells and 2 steps."""
    pts, cells = O.box_mesh(2, 1, 1)
    rng = np.random.default_rng(4)
    q = rng.normal(size=(2, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    ori = np.array([0, 1])
    theta = np.array([200.0, 90.0, 300.0, 2.0, 0.05])
    euler = rng.uniform(-20, 20, size=(2, 3))
    disps, ts = 1e-3 * np.arange(3), 0.1 * np.arange(3)

    def bcs(d):
        return [(O.face_nodes(pts, 0, 0.0), 0, 0.0), (O.face_nodes(pts, 1, 0.0), 1, 0.0),
                (O.face_nodes(pts, 2, 0.0), 2, 0.0), (O.face_nodes(pts, 2, 1.0), 2, d)]

    def f(th, eu):
        return O.history_stress(pts, cells, O.FCC12, (204.6e3, 137.7e3, 126.2e3), q, ori, th, eu, disps, ts, bcs,
                                local_tol=1e-10, solver_options={"tol": 1e-10, "rel_tol": 1e-13,
                                                                 "max_newton": 40})[:, 2, 2]
    for k in (1, 4):                       # g0 and m
        d = np.eye(5)[k]
        cs = O.complex_step(lambda th: f(th, euler), theta, d)
        h = 1e-6 * theta[k]
        fd = (f(theta + h * d, euler) - f(theta - h * d, euler)) / (2 * h)
        assert np.abs(cs - fd).max() < 1e-5 * np.abs(cs).max(), (k, cs, fd)
    d = np.zeros_like(euler)
    d[1, 0] = 1.0
    cs = O.complex_step(lambda eu: f(theta, eu), euler, d)
    fd = (f(theta, euler + 1e-4 * d) - f(theta, euler - 1e-4 * d)) / 2e-4
    assert np.abs(cs - fd).max() < 1e-5 * np.abs(cs).max(), (cs, fd)


def _continuation_case(disp=2e-3):
    pts, cells = O.box_mesh(2, 2, 2)
    q = np.array([[0.9, 0.1, -0.3, 0.2]])
    q /= np.linalg.norm(q)
    prob = O.OracleProblem(pts, cells, O.FCC12, 204.6e3, 137.7e3, 126.2e3, q, np.zeros(8, int), gss_initial=90.0,
                           h=500.0, t_sat=250.0, gss_a=2.25, xm=0.05, r=1.4, coplanar=True)
    prob.dt = 0.1
    prob.set_bcs([(O.face_nodes(pts, 0, 0.0), 0, 0.0), (O.face_nodes(pts, 1, 0.0), 1, 0.0),
                  (O.face_nodes(pts, 2, 0.0), 2, 0.0), (O.face_nodes(pts, 2, 1.0), 2, disp)])
    return prob


def test_oracle_arc_length_step():
    """Displacement-controlled arc-length steps (``solver.py:447-517``).  The loop tests the
    residual of the iterate before its update, so a step started from an equilibrium makes
    one update (the tangent predictor, sized by the constraint) and stops; a step started
    off equilibrium iterates until the residual it starts an update from is below tol.
    Each returned increment satisfies the arc-length constraint, and the BC rows follow
    lambda."""
    prob = _continuation_case()
    ub = O._bc_vector(prob, prob.ndof)
    dl = 0.4 * np.linalg.norm(ub)
    bc_dofs, bc_vals = prob.bc_dofs_vals()
    z = np.zeros(prob.ndof)
    u, lam, du, dlam = O.arc_length_disp(prob, z, 0.0, z, 0.0, Delta_l=dl, tol=1e-8)
    assert abs(np.sum(du ** 2) + dlam ** 2 * np.sum(ub ** 2) - dl ** 2) < 1e-10 * dl ** 2
    assert np.abs(u[bc_dofs] - lam * bc_vals).max() < 1e-12
    # the second step starts off equilibrium (the first was a predictor only) and corrects
    calls = []
    orig = prob.newton_update
    prob.newton_update = lambda d, *a, **k: calls.append(1) or orig(d, *a, **k)
    u2, lam2, du2, dlam2 = O.arc_length_disp(prob, u, lam, du, dlam, Delta_l=dl, tol=1e-8)
    prob.newton_update = orig
    assert len(calls) > 1 and lam2 > lam > 0
    assert abs(np.sum(du2 ** 2) + dlam2 ** 2 * np.sum(ub ** 2) - dl ** 2) < 1e-10 * dl ** 2
    assert np.abs(u2[bc_dofs] - lam2 * bc_vals).max() < 1e-12


def test_oracle_dynamic_relaxation():
    """Dynamic relaxation (``solver.py:656-795``) ends at the Newton solver's equilibrium,
    to the effect of its max|R| tolerance."""
    prob = _continuation_case(1e-3)
    ud, its = O.dynamic_relax(prob, tol=1e-7)
    assert its > 0
    un, _ = O.solver(prob, {"tol": 1e-10, "rel_tol": 1e-14})
    assert np.abs(ud - un).max() < 1e-6 * np.abs(un).max()
    assert O.dr_damping(-1.0, 1e-3, 3.9) == 1e-3 and O.dr_damping(100.0, 1e-3, 3.9) == 3.9
