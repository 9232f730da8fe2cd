"""CPU FP64 oracle for the CPFEM hot path -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.

Results of the CUDA path are checked against it.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
legs of ``bench.py`` (``cpu_baseline`` and ``--impl reference``) may import it; the
product package never does, and it is never the thing measured as the GPU result.

It is a plain numpy/scipy restatement of the reference algorithm, written so that each
step can be read side by side with the reference source (paths relative to the
reference project root):

* per-Gauss-point Kalidindi update, S-based implicit local Newton with the cut-half
  line search, linearised Fp^-1 update and explicit hardening:
  ``singlecrystal_copper/models_copper.py:155-249`` (plain model) and
  ``crystal_plasticity_OR_design/models_sens_rot.py:143-259`` (per-GP parameters);
* the implicit-function tangent of the local solve (``custom_jvp`` ``f_jvp``,
  ``models_copper.py:251-259``) -- here written out analytically;
* HEX8 / 2x2x2 Gauss element residual ``int P : grad v`` and its tangent -- the
  un-vendored JAX-FEM ``Problem`` kernels, restated from finite-element first principles
  (call sites ``models_copper.py:277-278,315`` and ``crystal_plasticity_OR_design/solver.py:392``);
* COO -> CSR with summed duplicates and sorted columns, row elimination of Dirichlet
  rows (``solver.py:119-133,279-304``);
* BiCGSTAB with the Jacobi preconditioner, tol = atol = 1e-10 (``solver.py:19-48``),
  restating ``jax.scipy.sparse.linalg.bicgstab`` of JAX 0.4.x (the third-party
  dependency; no version is pinned in the reference beyond a comment naming 0.4.13,
  ``models_copper.py:206``);
* the global Newton loop with its optional 3-halving line search (``solver.py:213-276,
  310-437``);
* ``compute_avg_stress`` / ``update_int_vars_gp`` (``models_copper.py:273-319``).

Parity pins: the reference's own golden sigma_zz curves
(``calibration/data/csv/calibration_case1/stress_strain_curve_copper.txt`` and
``calibration/data/csv/calibration_case2/ss_curve_e-2.txt``), copied as fixtures under
``tests/golden/`` by ``tests/golden/make_golden.py``.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp

# ----------------------------------------------------------------------------------
# Slip-system tables: rows are ``normal(3) direction(3)``, in the reference files' order
# (``singlecrystal_copper/data/csv/input_slip_sys.txt``,
#  ``polycrystal_DPsteel/data/csv/input_slip_sys_bcc12.txt``,
#  ``polycrystal_DPsteel/data/csv/input_slip_sys_bcc24.txt``).  The order matters: the
# latent-hardening matrix groups rows by the index rule 3*floor(i/3).
# ----------------------------------------------------------------------------------
FCC12 = np.array([
    [1, 1, -1, 0, 1, 1], [1, 1, -1, 1, 0, 1], [1, 1, -1, 1, -1, 0],
    [1, -1, -1, 0, 1, -1], [1, -1, -1, 1, 0, 1], [1, -1, -1, 1, 1, 0],
    [1, -1, 1, 0, 1, 1], [1, -1, 1, 1, 0, -1], [1, -1, 1, 1, 1, 0],
    [1, 1, 1, 0, 1, -1], [1, 1, 1, 1, 0, -1], [1, 1, 1, 1, -1, 0]], dtype=np.float64)

BCC12 = np.array([
    [1, 1, 0, -1, 1, 1], [1, 1, 0, 1, -1, 1], [1, -1, 0, 1, 1, 1], [1, -1, 0, 1, 1, -1],
    [1, 0, 1, 1, 1, -1], [1, 0, 1, -1, 1, 1], [1, 0, -1, 1, 1, 1], [1, 0, -1, 1, -1, 1],
    [0, 1, 1, 1, 1, -1], [0, 1, 1, 1, -1, 1], [0, 1, -1, 1, 1, 1], [0, 1, -1, -1, 1, 1]],
    dtype=np.float64)

BCC24 = np.concatenate([BCC12, np.array([
    [1, 1, 2, 1, 1, -1], [-1, 1, 2, 1, -1, 1], [1, -1, 2, -1, 1, 1], [1, 1, -2, 1, 1, 1],
    [1, 2, 1, 1, -1, 1], [-1, 2, 1, 1, 1, -1], [1, -2, 1, 1, 1, 1], [1, 2, -1, -1, 1, 1],
    [2, 1, 1, -1, 1, 1], [-2, 1, 1, 1, 1, 1], [2, -1, 1, 1, 1, -1], [2, 1, -1, 1, -1, 1]],
    dtype=np.float64)])

SLIP_TABLES = {"fcc12": FCC12, "bcc12": BCC12, "bcc24": BCC24}


def schmid_tensors(table):
    """P_a = d_a (x) n_a with both vectors normalised (``models_copper.py:59-69``)."""
    n = table[:, :3] / np.linalg.norm(table[:, :3], axis=1)[:, None]
    d = table[:, 3:] / np.linalg.norm(table[:, 3:], axis=1)[:, None]
    return np.einsum("ai,aj->aij", d, n)


def q_matrix(num_slip, r, coplanar=True):
    """Latent-hardening matrix.  ``coplanar=True`` follows ``models_copper.py:71-76``
    (q = r, with ones on the 3-blocks given by 3*floor(i/3)); ``coplanar=False`` follows
    ``models_sens_rot.py:170-175`` where the ``.at[].set`` result is discarded so q = r."""
    q = r * np.ones((num_slip, num_slip))
    if coplanar:
        for i in range(num_slip):
            for j in range(3):
                q[i, i // 3 * 3 + j] = 1.0
    return q


def rot_mat(quat):
    """Quaternion (scalar first, not normalised) -> rotation matrix (``models_copper.py:37-48``)."""
    q = np.asarray(quat, dtype=np.float64)
    q0, q1, q2, q3 = q[..., 0], q[..., 1], q[..., 2], q[..., 3]
    R = np.empty(q.shape[:-1] + (3, 3))
    R[..., 0, 0] = q0 * q0 + q1 * q1 - q2 * q2 - q3 * q3
    R[..., 0, 1] = 2 * q1 * q2 - 2 * q0 * q3
    R[..., 0, 2] = 2 * q1 * q3 + 2 * q0 * q2
    R[..., 1, 0] = 2 * q1 * q2 + 2 * q0 * q3
    R[..., 1, 1] = q0 * q0 - q1 * q1 + q2 * q2 - q3 * q3
    R[..., 1, 2] = 2 * q2 * q3 - 2 * q0 * q1
    R[..., 2, 0] = 2 * q1 * q3 - 2 * q0 * q2
    R[..., 2, 1] = 2 * q2 * q3 + 2 * q0 * q1
    R[..., 2, 2] = q0 * q0 - q1 * q1 - q2 * q2 + q3 * q3
    return R


def cubic_stiffness(C11, C12, C44):
    """Fourth-order cubic stiffness with minor symmetries (``models_copper.py:92-130``)."""
    C = np.zeros((3, 3, 3, 3))
    for i in range(3):
        C[i, i, i, i] = C11
        for j in range(3):
            if i != j:
                C[i, i, j, j] = C12
                C[i, j, i, j] = C44
                C[i, j, j, i] = C44
    return C


def rotate_rank2(R, T):
    """R T R^T for a stack of tensors (``models_copper.py:29-32``)."""
    return np.einsum("...ia,...jb,...ab->...ij", R, R, T)


def rotate_rank4(R, C):
    """C'_ijkl = R_ia R_jb R_kc R_ld C_abcd (``models_copper.py:21-26``)."""
    return np.einsum("...ia,...jb,...kc,...ld,abcd->...ijkl", R, R, R, R, C)


# ----------------------------------------------------------------------------------
# Per-GP constitutive update (vectorised over a batch of Gauss points)
# ----------------------------------------------------------------------------------
class GPBatch:
    """Inputs of the local problem for G Gauss points.

    Pr: (G,N,3,3) rotated Schmid tensors, Cr: (G,3,3,3,3) rotated stiffness,
    Fpi: (G,3,3) old Fp^-1, g: (G,N) old slip resistance, xm: (G,) rate exponent m,
    ao: reference slip rate, dt: time increment.
    """

    def __init__(self, F, Fpi, g, Pr, Cr, xm, ao, dt):
        self.F, self.Fpi, self.g, self.Pr, self.Cr = F, Fpi, g, Pr, Cr
        xm = np.asarray(xm)
        self.xm = np.broadcast_to(xm.astype(np.result_type(xm, np.float64)), (F.shape[0],))
        self.ao, self.dt = ao, dt
        self.A = F @ Fpi

    def subset(self, idx):
        return GPBatch(self.F[idx], self.Fpi[idx], self.g[idx], self.Pr[idx], self.Cr[idx],
                       self.xm[idx], self.ao, self.dt)


def _sign(x):
    """np.sign of the real part: the branch, which a complex-step perturbation never flips."""
    return np.sign(np.real(x))


def _abs(x):
    """|x|, continued analytically for complex-step derivatives (x sign(Re x))."""
    return x * _sign(x) if np.iscomplexobj(x) else np.abs(x)


def _slip_increment(b, S):
    """tau, Delta gamma and d(Delta gamma)/d tau (``models_copper.py:173-174``)."""
    tau = np.einsum("gij,gaij->ga", S, b.Pr)
    x = tau / b.g
    p = 1.0 / b.xm[:, None]
    ax = _abs(x)
    dgam = b.ao * b.dt * ax ** p * _sign(tau)
    # derivative as JAX differentiates |x|**p * sign(tau): p |x|^(p-1) sign(x) sign(tau) / g
    with np.errstate(divide="ignore", invalid="ignore"):
        kd = np.where(np.real(ax) > 0, b.ao * b.dt * p * ax ** (p - 1.0) / b.g * _sign(x) * _sign(tau), 0.0)
    return tau, dgam, kd


def _kinematics(b, dgam):
    """L_p increment, linearised Fp^-1 update and Fe (``models_copper.py:188-191``)."""
    L = np.einsum("ga,gaij->gij", dgam, b.Pr)
    Fpi_new = b.Fpi @ (np.eye(3) - L)
    Fe = b.F @ Fpi_new
    return Fpi_new, Fe


def residual(b, S):
    """r(S) = S - C' : (Fe^T Fe - I)/2 (``models_copper.py:195-201``).  S: (G,3,3)."""
    _, dgam, _ = _slip_increment(b, S)
    _, Fe = _kinematics(b, dgam)
    E = 0.5 * (np.einsum("gki,gkj->gij", Fe, Fe) - np.eye(3))
    return S - np.einsum("gijkl,gkl->gij", b.Cr, E)


def jacobian(b, S):
    """dr/dS (G,9,9), the quantity ``jax.jacfwd`` evaluates at ``models_copper.py:226``."""
    _, dgam, kd = _slip_increment(b, S)
    _, Fe = _kinematics(b, dgam)
    dFe = -np.einsum("gij,gajk->gaik", b.A, b.Pr)             # dFe/dL contracted per system
    Nsym = np.einsum("gki,gakj->gaij", Fe, dFe)
    Nsym = 0.5 * (Nsym + np.swapaxes(Nsym, -1, -2))
    CN = np.einsum("gijkl,gakl->gaij", b.Cr, Nsym)
    J = -np.einsum("ga,gaij,gakl->gijkl", kd, CN, b.Pr).reshape(-1, 9, 9)
    J += np.eye(9)
    return J


def local_newton(b, tol, max_sub_step, max_it=200):
    """Local Newton on S from y0 = 0 with the cut-half line search, per lane exactly as
    the batched ``lax.while_loop`` of ``models_copper.py:204-249`` behaves.

    Returns S (G,3,3), iteration counts (G,), converged mask (G,).  ``max_it`` is a
    safety cap the reference does not have; lanes that hit it report not-converged.
    """
    G = b.F.shape[0]
    y = np.zeros((G, 3, 3), dtype=np.result_type(b.F, b.Fpi, b.g, b.Pr, b.Cr, b.xm))
    r = residual(b, y)
    rn = np.linalg.norm(r.reshape(G, 9), axis=1)
    its = np.zeros(G, dtype=np.int64)
    active = rn > tol
    while active.any():
        idx = np.nonzero(active & (its < max_it))[0]
        if idx.size == 0:
            break
        bs = b.subset(idx)
        ys, rs, rn0 = y[idx], r[idx], rn[idx]
        J = jacobian(bs, ys)
        dy = np.linalg.solve(J, -rs.reshape(-1, 9)[..., None])[..., 0].reshape(-1, 3, 3)
        relax = np.ones(idx.size)
        sub = np.zeros(idx.size, dtype=np.int64)
        r_try, rn_try = rs.copy(), rn0.copy()
        searching = (rn_try >= rn0) & (sub < max_sub_step)
        while searching.any():
            s = np.nonzero(searching)[0]
            rt = residual(bs.subset(s), ys[s] + relax[s, None, None] * dy[s])
            r_try[s] = rt
            rn_try[s] = np.linalg.norm(rt.reshape(-1, 9), axis=1)
            relax[s] *= 0.5
            sub[s] += 1
            searching = (rn_try >= rn0) & (sub < max_sub_step)
        y[idx] = ys + 2.0 * relax[:, None, None] * dy
        r[idx], rn[idx] = r_try, rn_try
        its[idx] += 1
        active = rn > tol
    return y, its, ~(rn > tol)


def first_pk_stress(b, S):
    """sigma = Fe S Fe^T / det Fe ; P = det F sigma F^-T (``models_copper.py:155-162``)."""
    _, dgam, _ = _slip_increment(b, S)
    _, Fe = _kinematics(b, dgam)
    sigma = (Fe @ S @ np.swapaxes(Fe, -1, -2)) / np.linalg.det(Fe)[:, None, None]
    return np.linalg.det(b.F)[:, None, None] * sigma @ np.swapaxes(np.linalg.inv(b.F), -1, -2)


def tangent(b, S):
    """Consistent tangent dP/dF (G,3,3,3,3) at the converged S, via the implicit-function
    theorem of ``f_jvp`` (``models_copper.py:251-259``): dS = -J_S^-1 (dr/dF) dF.

    P = F X with X = Fp^-1 S Fp^-T / det(Fp^-1) (algebraically the reference P), and
    Fp^-1 = Fp^-1_old (I - L(S)).
    """
    G = S.shape[0]
    _, dgam, kd = _slip_increment(b, S)
    Fpi_new, Fe = _kinematics(b, dgam)
    I3 = np.eye(3)
    # dr/dF_kl = -C' : sym(Fe^T e_k e_l^T Fpi_new)
    T = np.einsum("gkm,gln->gklmn", Fe, Fpi_new)                  # (Fe^T e_k e_l^T Fpi)_mn
    T = 0.5 * (T + np.swapaxes(T, -1, -2))
    drdF = -np.einsum("gijmn,gklmn->gijkl", b.Cr, T).reshape(G, 9, 9)
    J = jacobian(b, S)
    dSdF = np.linalg.solve(J, -drdF)                               # (G, 9 [ij], 9 [kl])
    detFpi = np.linalg.det(Fpi_new)
    X = Fpi_new @ S @ np.swapaxes(Fpi_new, -1, -2) / detFpi[:, None, None]
    # explicit part: dP_ij/dF_kl = delta_ik X_lj
    D = np.einsum("ik,glj->gijkl", I3, X).reshape(G, 9, 9)
    # dP/dS for the 9 basis directions e_mn of S
    Finv_pi = np.linalg.inv(Fpi_new)
    dPdS = np.empty((G, 9, 9), dtype=X.dtype)
    for m in range(3):
        for n in range(3):
            dL = np.einsum("ga,ga,gaij->gij", kd, b.Pr[:, :, m, n], b.Pr)
            dFpi = -b.Fpi @ dL
            E = np.zeros((3, 3))
            E[m, n] = 1.0
            dX = (dFpi @ S @ np.swapaxes(Fpi_new, -1, -2) + Fpi_new @ E @ np.swapaxes(Fpi_new, -1, -2)
                  + Fpi_new @ S @ np.swapaxes(dFpi, -1, -2)) / detFpi[:, None, None]
            dX -= X * np.einsum("gij,gji->g", Finv_pi, dFpi)[:, None, None]
            dPdS[:, :, 3 * m + n] = (b.F @ dX).reshape(G, 9)
    D = D + dPdS @ dSdF
    return D.reshape(G, 3, 3, 3, 3)


def hardening_update(S, b, g, slip, h, t_sat, gss_a, r, coplanar):
    """Explicit state update after the local solve (``models_copper.py:176-187``,
    per-GP parameters as in ``models_sens_rot.py:168-193``)."""
    _, dgam, _ = _slip_increment(b, S)
    Fpi_new, _ = _kinematics(b, dgam)
    ratio = 1.0 - g / t_sat[:, None]
    tmp = h[:, None] * _abs(dgam) * _abs(ratio) ** gss_a[:, None] * _sign(ratio)
    N = g.shape[1]
    qs = np.stack([q_matrix(N, ri, coplanar) for ri in np.unique(r)])
    ridx = np.searchsorted(np.unique(r), r)
    g_inc = np.einsum("gab,gb->ga", qs[ridx], tmp)
    return Fpi_new, g + g_inc, slip + dgam


def _bincount(idx, w, n):
    """np.bincount with weights, for real or complex weights."""
    if np.iscomplexobj(w):
        return np.bincount(idx, weights=w.real, minlength=n) + 1j * np.bincount(idx, weights=w.imag, minlength=n)
    return np.bincount(idx, weights=w, minlength=n)


# ----------------------------------------------------------------------------------
# HEX8 element and mesh helpers (restated from FE first principles)
# ----------------------------------------------------------------------------------
HEX8_NODES = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                       [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)
_g = 1.0 / np.sqrt(3.0)
HEX8_QUADS = np.array([[a, b, c] for c in (-_g, _g) for b in (-_g, _g) for a in (-_g, _g)])


def hex8_dN_dxi(xi):
    """dN_a/dxi_J at a point of the reference cube [-1,1]^3, gmsh node order."""
    s = HEX8_NODES
    t = 1.0 + s * xi[None, :]
    d = np.empty((8, 3))
    d[:, 0] = 0.125 * s[:, 0] * t[:, 1] * t[:, 2]
    d[:, 1] = 0.125 * s[:, 1] * t[:, 0] * t[:, 2]
    d[:, 2] = 0.125 * s[:, 2] * t[:, 0] * t[:, 1]
    return d


def shape_grads_and_jxw(points, cells):
    """Physical shape-function gradients (E,8 quads,8 nodes,3) and JxW (E,8)."""
    X = points[cells]                                              # (E,8,3)
    E = cells.shape[0]
    sg = np.empty((E, 8, 8, 3))
    jxw = np.empty((E, 8))
    for q, xi in enumerate(HEX8_QUADS):
        dN = hex8_dN_dxi(xi)                                       # (8,3)
        Jm = np.einsum("eai,aj->eij", X, dN)                       # dx_i/dxi_j
        Jinv = np.linalg.inv(Jm)
        sg[:, q] = np.einsum("aj,eji->eai", dN, Jinv)
        jxw[:, q] = np.linalg.det(Jm) * 1.0                        # Gauss weight 1
    return sg, jxw


def box_mesh(nx, ny, nz, Lx=1.0, Ly=1.0, Lz=1.0):
    """Structured hex8 box, nodes x-fastest, gmsh-ordered connectivity."""
    xs, ys, zs = (np.linspace(0, L, n + 1) for L, n in ((Lx, nx), (Ly, ny), (Lz, nz)))
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    points = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    nid = lambda i, j, k: i + (nx + 1) * (j + (ny + 1) * k)
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    cells = np.stack([nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                      nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1),
                      nid(i, j + 1, k + 1)], axis=1).astype(np.int64)
    return points, cells


# ----------------------------------------------------------------------------------
# Problem: internal variables, assembly, solver
# ----------------------------------------------------------------------------------
class OracleProblem:
    """Restates the ``CrystalPlasticity(Problem)`` data model of the parameterised models
    (``models_sens_rot.py:52-139``): internal_vars =
    [Fp_inv (E,Q,3,3), g (E,Q,N), slip (E,Q,N), rot (E,Q,3,3), gss_a, h, t_sat, xm, r (E,Q)]."""

    def __init__(self, points, cells, slip_table, C11, C12, C44, quat, cell_ori_inds,
                 gss_initial, h, t_sat, gss_a, xm, r, ao=1e-3, coplanar=False,
                 local_tol=1e-8, max_sub_step=5, bcs=()):
        self.points, self.cells = np.asarray(points, np.float64), np.asarray(cells, np.int64)
        self.E = self.cells.shape[0]
        self.n_nodes = self.points.shape[0]
        self.ndof = 3 * self.n_nodes
        self.schmid = schmid_tensors(np.asarray(slip_table, np.float64))
        self.N = self.schmid.shape[0]
        self.C = cubic_stiffness(C11, C12, C44)
        self.ao, self.coplanar = ao, coplanar
        self.local_tol, self.max_sub_step = local_tol, max_sub_step
        self.sg, self.jxw = shape_grads_and_jxw(self.points, self.cells)
        rots = rot_mat(np.asarray(quat, np.float64))[np.asarray(cell_ori_inds)]
        E, Q, N = self.E, 8, self.N
        ones = np.ones((E, Q))
        self.internal_vars = [
            np.broadcast_to(np.eye(3), (E, Q, 3, 3)).copy(),
            gss_initial * np.ones((E, Q, N)),
            np.zeros((E, Q, N)),
            np.repeat(rots[:, None], Q, axis=1),
            gss_a * ones, h * ones, t_sat * ones, xm * ones, r * ones]
        self.dt = 1.0
        self.set_bcs(bcs)

    # --- Dirichlet data: list of (node_inds, component, value) -------------------
    def set_bcs(self, bcs):
        self.bcs = [(np.asarray(n, np.int64), int(c), float(v)) for n, c, v in bcs]

    def bc_dofs_vals(self):
        dofs = np.concatenate([3 * n + c for n, c, _ in self.bcs]) if self.bcs else np.zeros(0, np.int64)
        vals = np.concatenate([np.full(n.size, v) for n, _, v in self.bcs]) if self.bcs else np.zeros(0)
        return dofs, vals

    # --- per-GP batch ---------------------------------------------------------------
    def u_grads(self, sol):
        """u_grad (E,Q,3,3) = sum_a u_a (x) dN_a/dX (``models_copper.py:277-278``)."""
        return np.einsum("eai,eqaj->eqij", sol.reshape(-1, 3)[self.cells], self.sg)

    def gp_batch(self, sol, params):
        Fpi, g, _, rot = params[:4]
        xm = params[7]
        G = self.E * 8
        F = (self.u_grads(sol) + np.eye(3)).reshape(G, 3, 3)
        R = rot.reshape(G, 3, 3)
        # the rotated tables only depend on the rotation: compute once per distinct R
        Ru, inv = np.unique(R.reshape(G, 9), axis=0, return_inverse=True)
        Ru = Ru.reshape(-1, 3, 3)
        Pr_u = np.einsum("uia,ujb,kab->ukij", Ru, Ru, self.schmid)
        Cr_u = rotate_rank4(Ru, self.C)
        inv = inv.reshape(-1)
        return GPBatch(F, Fpi.reshape(G, 3, 3), g.reshape(G, self.N), Pr_u[inv], Cr_u[inv],
                       xm.reshape(G), self.ao, self.dt)

    def solve_gps(self, b):
        S, its, ok = local_newton(b, self.local_tol, self.max_sub_step)
        if not ok.all():
            raise RuntimeError("oracle local Newton did not converge")
        return S, its

    # --- assembly ------------------------------------------------------------------
    def newton_update(self, sol, params=None, need_tangent=True):
        """Residual (ndof,) and, if asked, the CSR tangent with summed duplicates
        (what JAX-FEM's newton_update + ``solver.py:279-282`` produce)."""
        params = self.internal_vars if params is None else params
        b = self.gp_batch(sol, params)
        S, its = self.solve_gps(b)
        self.last_local_its = its
        E = self.E
        P = first_pk_stress(b, S).reshape(E, 8, 3, 3)
        res_e = np.einsum("eqij,eqaj,eq->eai", P, self.sg, self.jxw)
        dof = (3 * self.cells[:, :, None] + np.arange(3)[None, None, :]).reshape(E, 24)
        res = _bincount(dof.ravel(), res_e.ravel(), self.ndof)
        if not need_tangent:
            return res, None
        D = tangent(b, S).reshape(E, 8, 3, 3, 3, 3)
        Ke = np.einsum("eqaj,eqijkl,eqbl,eq->eaibk", self.sg, D, self.sg, self.jxw).reshape(E, 24, 24)
        I = np.repeat(dof[:, :, None], 24, axis=2).ravel()
        J = np.repeat(dof[:, None, :], 24, axis=1).ravel()
        A = sp.csr_array((Ke.ravel(), (I, J)), shape=(self.ndof, self.ndof))
        A.sum_duplicates()
        A.sort_indices()
        return res, A

    def compute_residual(self, sol, params=None):
        return self.newton_update(sol, params, need_tangent=False)[0]

    # --- post-processing / state update -------------------------------------------
    def compute_avg_stress(self, sol, params):
        """Per-cell JxW-weighted Cauchy stress (``models_copper.py:297-319``)."""
        b = self.gp_batch(sol, params)
        S, _ = self.solve_gps(b)
        P = first_pk_stress(b, S)
        sigma = P @ np.swapaxes(b.F, -1, -2) / np.linalg.det(b.F)[:, None, None]
        sigma = sigma.reshape(self.E, 8, 3, 3)
        return np.einsum("eqij,eq->eij", sigma, self.jxw) / self.jxw.sum(1)[:, None, None]

    def update_int_vars_gp(self, sol, params):
        """New internal variables at the converged solution (``models_copper.py:273-282``)."""
        b = self.gp_batch(sol, params)
        S, _ = self.solve_gps(b)
        G, E, N = S.shape[0], self.E, self.N
        gss_a, h, t_sat, xm, r = (p.reshape(G) for p in params[4:9])
        Fpi_new, g_new, slip_new = hardening_update(
            S, b, params[1].reshape(G, N), params[2].reshape(G, N), h, t_sat, gss_a, r, self.coplanar)
        return [Fpi_new.reshape(E, 8, 3, 3), g_new.reshape(E, 8, N), slip_new.reshape(E, 8, N)] + \
            [p.copy() for p in params[3:]]

    def set_params(self, params):
        self.internal_vars = params


# ----------------------------------------------------------------------------------
# Linear solver and global Newton (``solver.py``)
# ----------------------------------------------------------------------------------
def bicgstab(A, b, x0, M, tol=1e-10, atol=1e-10, maxiter=10000):
    """BiCGSTAB as ``jax.scipy.sparse.linalg.bicgstab`` (JAX 0.4.x) runs it: stop on
    ||r||^2 <= max(tol^2 ||b||^2, atol^2) of the true residual, early exit on ||s||,
    breakdown codes -10 (rho = 0) / -11 (alpha or omega = 0).  Returns (x, iterations)."""
    atol2 = max(tol * tol * float(b @ b), atol * atol)
    x = x0.copy()
    r = b - A @ x
    rhat, p, q = r.copy(), r.copy(), r.copy()
    rho = alpha = omega = 1.0
    k = 0
    while float(r @ r) > atol2 and 0 <= k < maxiter:
        rho_ = float(rhat @ r)
        beta = rho_ / rho * alpha / omega
        p = r + beta * (p - omega * q)
        phat = M(p)
        q = A @ phat
        alpha = rho_ / float(rhat @ q)
        s = r - alpha * q
        exit_early = float(s @ s) < atol2
        shat = M(s)
        t = A @ shat
        omega = float(t @ s) / float(t @ t)
        if exit_early:
            x = x + alpha * phat
            r = s
        else:
            x = x + (alpha * phat + omega * shat)
            r = s - omega * t
        k = -11 if (omega == 0 or alpha == 0) else k + 1
        k = -10 if rho_ == 0 else k
        rho = rho_
    return x, k


def apply_bc_rows(A, bc_dofs):
    """PETSc ``zeroRows``: BC rows become unit rows (``solver.py:290-293``)."""
    A = A.tolil() if False else A.copy()
    A = A.tocsr()
    rows = np.unique(bc_dofs)
    mask = np.zeros(A.shape[0], dtype=bool)
    mask[rows] = True
    row_of = np.repeat(np.arange(A.shape[0]), np.diff(A.indptr))
    A.data[mask[row_of]] = 0.0
    diag_pos = mask[row_of] & (A.indices == row_of)
    A.data[diag_pos] = 1.0
    return A


def solver(problem, solver_options=None):
    """Global Newton with row elimination (``solver.py:310-437``).

    Returns (dofs, info) with info = {newton_iters, krylov_iters: [...]}.
    """
    opts = dict(solver_options or {})
    rel_tol = opts.get("rel_tol", 1e-8)
    tol = opts.get("tol", 1e-6)
    ls_flag = opts.get("line_search_flag", False)
    guess = opts.get("initial_guess")
    dofs = np.array(guess, dtype=np.result_type(guess, np.float64)).reshape(-1) if guess is not None \
        else np.zeros(problem.ndof)
    bc_dofs, bc_vals = problem.bc_dofs_vals()

    def res_bc(d, res):
        res = res.copy()
        res[bc_dofs] = d[bc_dofs]
        res[bc_dofs] -= bc_vals
        return res

    # a problem may bring compiled row elimination and BiCGSTAB (coracle.FastOracleProblem)
    zero_rows = getattr(problem, "zero_rows", apply_bc_rows)

    def helper(d):
        res, A = problem.newton_update(d)
        return res_bc(d, res), zero_rows(A, bc_dofs)

    res, A = helper(dofs)
    rv = np.linalg.norm(res)
    r0 = rv
    info = {"newton_iters": 0, "krylov_iters": [], "res_history": [rv]}
    max_newton = opts.get("max_newton", 100)     # a safety cap the reference does not have
    while (rv / r0 > rel_tol if r0 > 0 else False) and rv > tol:
        if info["newton_iters"] >= max_newton:
            raise RuntimeError(f"oracle Newton did not converge in {max_newton} iterations (res = {rv})")
        x0 = np.zeros(problem.ndof, dtype=np.result_type(dofs, res))
        x0[bc_dofs] = bc_vals
        x0[bc_dofs] -= dofs[bc_dofs]
        if hasattr(problem, "linear_solve"):
            inc, kk = problem.linear_solve(A, -res, x0)
        else:
            diag = A.diagonal()
            inc, kk = bicgstab(A, -res, x0, lambda v: v * (1.0 / diag))
        err = np.linalg.norm(A @ inc + res)
        if not err < 0.1:
            raise RuntimeError(f"oracle linear solver failed, err={err}")
        info["krylov_iters"].append(kk)
        if ls_flag:
            dofs = _line_search(problem, dofs, inc, res_bc)
        else:
            dofs = dofs + inc
        res, A = helper(dofs)
        rv = np.linalg.norm(res)
        info["newton_iters"] += 1
        info["res_history"].append(rv)
    if not (np.isfinite(rv) and np.all(np.isfinite(dofs))):
        raise RuntimeError("oracle Newton produced non-finite values")
    return dofs, info


def _line_search(problem, dofs, inc, res_bc):
    """Three halvings, keep the last improving alpha (``solver.py:240-276``)."""
    def res_norm(alpha):
        d = dofs + alpha * inc
        return np.linalg.norm(res_bc(d, problem.compute_residual(d)))
    alpha = 1.0
    rn = res_norm(alpha)
    for _ in range(3):
        alpha *= 0.5
        rh = res_norm(alpha)
        if rh > rn:
            alpha *= 2.0
            break
        rn = rh
    return dofs + alpha * inc


def face_nodes(points, axis, value, atol=1e-5):
    return np.nonzero(np.isclose(points[:, axis], value, atol=atol))[0]


def corner_nodes(points, xyz, atol=1e-5):
    m = np.ones(points.shape[0], dtype=bool)
    for a, v in enumerate(xyz):
        m &= np.isclose(points[:, a], v, atol=atol)
    return np.nonzero(m)[0]


def run_load_steps(problem, disps, ts, make_bcs, solver_options=None, stress_fn=None):
    """Driver loop of ``calibration_case1_singleCrystalCopper_GB.py:270-292``: per step
    set dt and the top displacement, solve, record the stress, commit the state."""
    sol = np.zeros(problem.ndof)
    out = []
    params = problem.internal_vars
    for i in range(len(ts) - 1):
        problem.dt = float(ts[i + 1] - ts[i])
        problem.set_bcs(make_bcs(float(disps[i + 1])))
        problem.set_params(params)
        opts = dict(solver_options or {})
        opts["initial_guess"] = sol
        sol, _ = solver(problem, opts)
        sig = problem.compute_avg_stress(sol, params)
        out.append(stress_fn(sig) if stress_fn else sig)
        params = problem.update_int_vars_gp(sol, params)
    problem.set_params(params)
    return np.array(out), sol


# ----------------------------------------------------------------------------------
# Derivatives of a load history (the quantity the reference differentiates with jax.grad
# through ad_wrapper / implicit_vjp, ``crystal_plasticity_OR_design/solver.py:801-874``,
# in the calibration and orientation-design drivers)
# ----------------------------------------------------------------------------------
def euler_zyx_deg(angles):
    """Lowercase 'zyx' Euler angles in degrees, i.e. extrinsic rotations about z, then y,
    then x: R = Rx(c) Ry(b) Rz(a) -- what ``Rotation.from_euler('zyx', ..., degrees=True)``
    returns at ``poly_sensitivity_rot_mesh2.py:41-55``; written out so that complex angles
    (complex-step derivatives) pass through."""
    ang = np.asarray(angles) * (np.pi / 180.0)
    a, b, c = ang[..., 0], ang[..., 1], ang[..., 2]
    ca, sa, cb, sb, cc, sc = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    z, o = np.zeros_like(a), np.ones_like(a)
    Rz = np.stack([ca, -sa, z, sa, ca, z, z, z, o], -1).reshape(ang.shape[:-1] + (3, 3))
    Ry = np.stack([cb, z, sb, z, o, z, -sb, z, cb], -1).reshape(ang.shape[:-1] + (3, 3))
    Rx = np.stack([o, z, z, z, cc, -sc, z, sc, cc], -1).reshape(ang.shape[:-1] + (3, 3))
    return Rx @ Ry @ Rz


def history_stress(points, cells, slip_table, C, grain_quat, cell_grain, theta, euler, disps, ts, make_bcs,
                   r=1.4, coplanar=True, ao=1e-3, local_tol=1e-8, max_sub_step=5, solver_options=None):
    """Per-step mean cell Cauchy stress (n_steps, 3, 3) of a load history as a function of
    the Kalidindi parameters theta = (h0, g0, gs, a, m) and per-grain Euler angles
    (degrees, 'zyx', composed as R = R_euler R_quat, ``poly_sensitivity_rot_mesh2.py:41-65,
    186-203``).  Complex theta / euler give complex-step derivatives: every operation on the
    path is complex-analytic on the branch the real iterate takes, the local and global
    Newton solves use their exact complex Jacobians, and the linear solves are direct, so
    Im(f(x + i h d)) / h is the directional derivative of the discrete load history to
    rounding."""
    h0, g0, gs, a, m = theta
    R = euler_zyx_deg(euler) @ rot_mat(grain_quat)
    prob = OracleProblem(points, cells, slip_table, *C, grain_quat, cell_grain, gss_initial=1.0, h=1.0,
                         t_sat=1.0, gss_a=1.0, xm=1.0, r=r, ao=ao, coplanar=coplanar, local_tol=local_tol,
                         max_sub_step=max_sub_step)
    E, N = prob.E, prob.N
    ones = np.ones((E, 8))
    rot = np.repeat(R[np.asarray(cell_grain)][:, None], 8, axis=1)
    prob.internal_vars = [np.broadcast_to(np.eye(3), (E, 8, 3, 3)).astype(rot.dtype), g0 * np.ones((E, 8, N)),
                          np.zeros((E, 8, N)), rot, a * ones, h0 * ones, gs * ones, m * ones, r * ones]

    def direct(A, b, x0):
        import scipy.sparse.linalg as spla
        return spla.spsolve(sp.csc_matrix(A), b), 0
    prob.linear_solve = direct
    sig, _ = run_load_steps(prob, disps, ts, make_bcs, solver_options)
    return sig.mean(axis=1)


def complex_step(fn, x, d, h=1e-30):
    """Directional derivative Im(fn(x + i h d)) / h of a real function (no cancellation)."""
    return np.imag(fn(np.asarray(x, dtype=np.complex128) + 1j * h * np.asarray(d))) / h


# ----------------------------------------------------------------------------------
# Arc-length continuation and dynamic relaxation (``crystal_plasticity_OR_design/solver.py:
# 447-795``).  The reference solves their linear systems with UMFPACK; here scipy's sparse
# LU stands in for it.  Neither routine updates internal variables: a caller commits the
# state between steps (``update_int_vars_gp``), as with the Newton solver.
# ----------------------------------------------------------------------------------
def _direct(A, b):
    import scipy.sparse.linalg as spla
    return spla.spsolve(sp.csc_matrix(A), b)


def _bc_vector(problem, n):
    """``assign_bc(zeros)`` (``solver.py:137-145``): the BC values on their dofs."""
    dofs, vals = problem.bc_dofs_vals()
    u = np.zeros(n)
    u[dofs] = vals
    return u


def _arc_length_lambda(a1, a2, a3, u, lam, prev_u, prev_lam, dub, dut, dir_u, dir_lam, psi2_w):
    """The constraint's two roots and the one whose direction continues the previous
    increment (``solver.py:480-508``); returns delta_lambda."""
    disc = np.sqrt(a2 ** 2 - 4.0 * a1 * a3)
    l1 = (-a2 + disc) / (2.0 * a1)
    l2 = (-a2 - disc) / (2.0 * a1)
    if not (np.isfinite(l1) and np.isfinite(l2)):
        raise RuntimeError(f"no valid delta lambda: a1 = {a1}, a2 = {a2}, a3 = {a3}")

    def dot(du1, dl1, du2, dl2):
        return np.sum(du1 * du2) + psi2_w * dl1 * dl2
    d1 = dot(dir_u, dir_lam, u + dub + l1 * dut - prev_u, lam + l1 - prev_lam)
    d2 = dot(dir_u, dir_lam, u + dub + l2 * dut - prev_u, lam + l2 - prev_lam)
    if abs(d1) < 1e-10 and abs(d2) < 1e-10:
        return max(l1, l2)
    return l1 if d1 > d2 else l2


def arc_length_disp(problem, prev_u, prev_lam, prev_Du, prev_Dlam, Delta_l=0.1, psi=1.0, tol=1e-6,
                    max_iter=100):
    """Crisfield's arc length under displacement control (``solver.py:447-517``): the BC
    values are scaled by lambda, the residual's BC rows are u - lambda * u_b.  Returns
    (u, lambda, Delta u, Delta lambda) of the step.  ``max_iter`` is a cap the reference
    does not have."""
    bc_dofs, bc_vals = problem.bc_dofs_vals()
    u = np.array(prev_u, dtype=np.float64)
    lam = float(prev_lam)
    u_b = _bc_vector(problem, problem.ndof)
    w = psi ** 2 * np.sum(u_b ** 2)
    dir_u, dir_lam = np.array(prev_Du, dtype=np.float64), float(prev_Dlam)
    res_val, it = 1.0, 0
    while res_val > tol:
        if it >= max_iter:
            raise RuntimeError(f"arc-length step did not converge in {max_iter} iterations")
        res, A = problem.newton_update(u)
        res = res.copy()
        res[bc_dofs] = u[bc_dofs]
        res[bc_dofs] -= bc_vals * lam
        A = apply_bc_rows(A, bc_dofs)
        res_val = np.linalg.norm(res)
        dub = _direct(A, -res)
        dut = _direct(A, u_b)
        Du, Dlam = u - prev_u, lam - prev_lam
        a1 = np.sum(dut ** 2) + w
        a2 = 2.0 * np.sum((Du + dub) * dut) + 2.0 * w * Dlam
        a3 = np.sum((Du + dub) ** 2) + w * Dlam ** 2 - Delta_l ** 2
        dl = _arc_length_lambda(a1, a2, a3, u, lam, prev_u, prev_lam, dub, dut, dir_u, dir_lam, w)
        lam = lam + dl
        u = u + dub + dl * dut
        dir_u, dir_lam = u - prev_u, lam - prev_lam
        it += 1
    return u, lam, dir_u, dir_lam


def arc_length_force(problem, prev_u, prev_lam, prev_Du, prev_Dlam, q_vec, Delta_l=0.1, psi=1.0, tol=1e-6,
                     max_iter=100):
    """Crisfield's arc length under load control (``solver.py:522-590``): equilibrium
    res(u) + lambda q = 0 with q's BC rows zeroed."""
    bc_dofs, bc_vals = problem.bc_dofs_vals()
    u = np.array(prev_u, dtype=np.float64)
    lam = float(prev_lam)
    q = np.array(q_vec, dtype=np.float64).copy()
    q[bc_dofs] = 0.0
    w = psi ** 2 * np.sum(q ** 2)
    dir_u, dir_lam = np.array(prev_Du, dtype=np.float64), float(prev_Dlam)
    res_val, it = 1.0, 0
    while res_val > tol:
        if it >= max_iter:
            raise RuntimeError(f"arc-length step did not converge in {max_iter} iterations")
        res, A = problem.newton_update(u)
        res = res.copy()
        res[bc_dofs] = u[bc_dofs]
        res[bc_dofs] -= bc_vals
        A = apply_bc_rows(A, bc_dofs)
        res_val = np.linalg.norm(res + lam * q)
        dub = _direct(A, -(res + lam * q))
        dut = _direct(A, -q)
        Du, Dlam = u - prev_u, lam - prev_lam
        a1 = np.sum(dut ** 2) + w
        a2 = 2.0 * np.sum((Du + dub) * dut) + 2.0 * w * Dlam
        a3 = np.sum((Du + dub) ** 2) + w * Dlam ** 2 - Delta_l ** 2
        dl = _arc_length_lambda(a1, a2, a3, u, lam, prev_u, prev_lam, dub, dut, dir_u, dir_lam, w)
        lam = lam + dl
        u = u + dub + dl * dut
        dir_u, dir_lam = u - prev_u, lam - prev_lam
        it += 1
    return u, lam, dir_u, dir_lam


def get_q_vec(problem):
    """The residual at u = 0 (``solver.py:593-602``)."""
    return problem.compute_residual(np.zeros(problem.ndof))


def dr_damping(t, cmin, cmax):
    """``calC`` (``solver.py:626-634``): c = 2 sqrt(t) clipped to [cmin, cmax]."""
    t = max(t, 0.0)
    return min(max(2.0 * np.sqrt(t), cmin), cmax)


def dynamic_relax(problem, tol=1e-6, nKMat=50, initial_guess=None, max_iter=100000):
    """Dynamic relaxation (``solver.py:656-795``): one linear step from u = 0, then explicit
    damped pseudo-dynamics with the lumped mass M = h~^2/4 rowsum|K| until max|R| <= tol.
    The reference's update sets qdot_old = qdot before qdotdot = qdot - qdot_old, so the
    pseudo-acceleration is zero and the stiffness is never re-formed after the first; this
    keeps that order.  ``max_iter`` is a cap the reference does not have.
    Returns (dofs, iterations)."""
    bc_dofs, bc_vals = problem.bc_dofs_vals()
    n = problem.ndof
    dofs = np.zeros(n)
    res, A = problem.newton_update(dofs)
    res = res.copy()
    res[bc_dofs] = dofs[bc_dofs]
    res[bc_dofs] -= bc_vals
    A = apply_bc_rows(A, bc_dofs)
    x0 = np.zeros(n)
    x0[bc_dofs] = bc_vals
    dofs = dofs + _direct(A, -res)
    if initial_guess is not None:
        dofs = np.array(initial_guess, dtype=np.float64).reshape(-1).copy()
        dofs[bc_dofs] = bc_vals
    cmin, cmax, h_tilde, h = 1e-3, 3.9, 1.1, 1.0

    def vec(d):
        r = problem.compute_residual(d).copy()
        r[bc_dofs] = 0.0
        return r

    def mass(d):
        _, K = problem.newton_update(d)
        K = apply_bc_rows(K, bc_dofs)
        return h_tilde * h_tilde / 4.0 * np.asarray(abs(K).sum(axis=1)).reshape(-1)
    qdot_old, qdotdot, qdotdot_old = np.zeros(n), np.zeros(n), np.zeros(n)
    R = vec(dofs)
    M = mass(dofs)
    q = dofs.copy()
    qdot = -h / 2.0 * R / M
    nIters = iKMat = 0
    error = np.max(np.abs(R))
    while error > tol:
        if nIters >= max_iter:
            raise RuntimeError(f"dynamic relaxation did not converge in {max_iter} iterations")
        q_old, R_old = q.copy(), R
        q = q + h * qdot
        dofs = q.copy()
        R = vec(dofs)
        nIters += 1
        iKMat += 1
        error = np.max(np.abs(R))
        S0 = np.dot((R - R_old) / h, qdot)
        t = S0 / np.einsum("i,i,i", qdot, M, qdot)
        c = dr_damping(t, cmin, cmax)
        dq = q - q_old
        ratio = np.divide(qdotdot - qdotdot_old, dq, out=np.zeros(n), where=dq != 0)
        eps = h_tilde * h_tilde / 4.0 * np.abs(ratio)
        if np.max(eps) > 1 and iKMat > nKMat:
            iKMat = 0
            M = mass(dofs)
        qdot_old, qdotdot_old = qdot.copy(), qdotdot.copy()
        qdot = (2.0 - c * h) / (2.0 + c * h) * qdot_old - 2.0 * h / (2.0 + c * h) * R / M
        qdot_old = qdot.copy()
        qdotdot = qdot - qdot_old
    return dofs, nIters
