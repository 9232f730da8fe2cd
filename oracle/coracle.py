"""Compiled CPU oracle -- TEST INFRASTRUCTURE, NOT PRODUCT CODE.

``FastOracleProblem`` is ``cpfem_oracle.OracleProblem`` with its per-Gauss-point pass,
element assembly, row elimination and BiCGSTAB running in ``cpfem_oracle_c.c`` (plain C,
OpenMP over the host cores) instead of numpy.  The algorithm, the unknowns and the
control flow are the numpy oracle's (``cpfem_oracle.solver`` drives both); the CPU test
suite checks the two against each other on small cases, and the numpy oracle is pinned to
the reference's golden curves.  It exists for the sizes numpy cannot reach in a test: the
32^3 load steps of the parity tests and the timed CPU baseline of ``bench.py``.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py`` import it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np
import scipy.sparse as sp

from . import cpfem_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpfem_oracle_c.c")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcpfem_oracle.so")

_lib = None


def build(force=False):
    """gcc -O3 -fopenmp; no -march, no fused multiply-add contraction (the same results on
    x86-64 and aarch64 hosts)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", "-o", LIB, SRC, "-lm"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return LIB


def load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(LIB)
    P, L, I, D = ctypes.c_void_p, ctypes.c_long, ctypes.c_int, ctypes.c_double
    lib.orc_num_threads.restype = I
    lib.orc_set_threads.argtypes = [I]
    lib.orc_deformation.argtypes = [L, P, P, P, P]
    lib.orc_gp_pass.restype = L
    lib.orc_gp_pass.argtypes = [L, I, P, P, P, P, P, P, P, P, I, D, D, D, I, I, P, P, P, P, P, P, P]
    lib.orc_element.argtypes = [L, P, P, P, P, P, P]
    lib.orc_gather.argtypes = [L, P, P, P, P]
    lib.orc_zero_rows.argtypes = [L, P, P, P, P]
    lib.orc_spmv.argtypes = [L, P, P, P, P, P]
    lib.orc_bicgstab.restype = I
    lib.orc_bicgstab.argtypes = [L, P, P, P, P, P, P, D, D, I, P]
    _lib = lib
    return lib


def num_threads():
    return int(load().orc_num_threads())


def set_threads(n):
    load().orc_set_threads(int(n))


def _p(a):
    return None if a is None else a.ctypes.data


def _c(a, dtype=np.float64):
    return np.ascontiguousarray(a, dtype=dtype)


class CSR:
    """Scalar CSR matrix with int64 row pointers (what the C routines take); ``tocsr()``
    gives the scipy matrix."""

    def __init__(self, indptr, indices, data, n):
        self.indptr, self.indices, self.data, self.shape = indptr, indices, data, (n, n)

    def tocsr(self):
        return sp.csr_array((self.data, self.indices, self.indptr), shape=self.shape)

    def __matmul__(self, x):
        x = _c(x)
        y = np.empty(self.shape[0])
        load().orc_spmv(self.shape[0], _p(self.indptr), _p(self.indices), _p(self.data), _p(x), _p(y))
        return y

    def diagonal(self):
        return self.tocsr().diagonal()

    def copy(self):
        return CSR(self.indptr, self.indices, self.data.copy(), self.shape[0])


class FastOracleProblem(O.OracleProblem):
    """``OracleProblem`` with the compiled passes (same constructor and data model)."""

    max_local_it = 200

    def __init__(self, *args, **kw):
        super().__init__(*args, **kw)
        self.lib = load()
        E = self.E
        dof = (3 * self.cells[:, :, None] + np.arange(3)[None, None, :]).reshape(E, 24)
        self._dof = dof
        I = np.repeat(dof[:, :, None], 24, axis=2).ravel()
        J = np.repeat(dof[:, None, :], 24, axis=1).ravel()
        key = I * self.ndof + J
        ukeys, inv = np.unique(key, return_inverse=True)        # scipy's summed, sorted pattern
        del I, J, key
        rows = ukeys // self.ndof
        self.indices = (ukeys % self.ndof).astype(np.int32)
        self.indptr = np.concatenate([[0], np.cumsum(np.bincount(rows, minlength=self.ndof))]).astype(np.int64)
        inv = inv.reshape(-1)
        self.gather_idx = np.argsort(inv, kind="stable").astype(np.int64)   # element order per value
        self.gather_ptr = np.concatenate([[0], np.cumsum(np.bincount(inv, minlength=ukeys.size))]).astype(np.int64)
        self.nnz = int(ukeys.size)
        self.sg_c = _c(self.sg)
        self.jxw_c = _c(self.jxw)
        self.cells_c = _c(self.cells, np.int64)
        self._rot_key = None

    # --- per-GP inputs --------------------------------------------------------------
    def _tables(self, params):
        """Rotation index per GP and the rotated Schmid / stiffness tables of the distinct
        rotations (the rotated tables depend on the rotation only)."""
        if self._rot_key is not params[3]:
            G = self.E * 8
            R = np.asarray(params[3], np.float64).reshape(G, 9)
            Ru, inv = np.unique(R, axis=0, return_inverse=True)
            Ru = Ru.reshape(-1, 3, 3)
            self._Pr = _c(np.einsum("uia,ujb,kab->ukij", Ru, Ru, self.schmid))
            self._Cr = _c(O.rotate_rank4(Ru, self.C))
            self._rot_idx = _c(inv.reshape(-1), np.int32)
            self._rot_key = params[3]
        return self._rot_idx, self._Pr, self._Cr

    def _gp(self, sol, params, P=False, D=False, sigma=False, state=False):
        G, N = self.E * 8, self.N
        lib = self.lib
        F = np.empty((G, 9))
        u = _c(sol).reshape(-1)
        lib.orc_deformation(self.E, _p(self.cells_c), _p(self.sg_c), _p(u), _p(F))
        ridx, Pr, Cr = self._tables(params)
        Fpi = _c(params[0]).reshape(G, 9)
        g = _c(params[1]).reshape(G, N)
        slip = _c(params[2]).reshape(G, N)
        prm = _c(np.stack([np.broadcast_to(np.asarray(params[k], np.float64), (self.E, 8)).reshape(G)
                           for k in range(4, 9)], axis=1))
        out = {"F": F, "its": np.empty(G, dtype=np.int32)}
        out["P"] = np.empty((G, 9)) if P else None
        out["D"] = np.empty((G, 81)) if D else None
        out["sigma"] = np.empty((G, 9)) if sigma else None
        for k, w in (("Fpi_new", 9), ("g_new", N), ("slip_new", N)):
            out[k] = np.empty((G, w)) if state else None
        bad = lib.orc_gp_pass(G, N, _p(F), _p(Fpi), _p(g), _p(slip), _p(ridx), _p(Pr), _p(Cr), _p(prm),
                              1 if self.coplanar else 0, float(self.ao), float(self.dt), float(self.local_tol),
                              int(self.max_sub_step), int(self.max_local_it), _p(out["P"]), _p(out["D"]),
                              _p(out["sigma"]), _p(out["Fpi_new"]), _p(out["g_new"]), _p(out["slip_new"]),
                              _p(out["its"]))
        if bad:
            raise RuntimeError(f"oracle local Newton did not converge at {bad} Gauss points")
        self.last_local_its = out["its"]
        return out

    # --- assembly ---------------------------------------------------------------------
    def newton_update(self, sol, params=None, need_tangent=True):
        params = self.internal_vars if params is None else params
        o = self._gp(sol, params, P=True, D=need_tangent)
        E = self.E
        re = np.empty((E, 24))
        ke = np.empty((E, 576)) if need_tangent else None
        self.lib.orc_element(E, _p(self.sg_c), _p(self.jxw_c), _p(o["P"]), _p(o["D"]), _p(re), _p(ke))
        res = np.bincount(self._dof.ravel(), weights=re.ravel(), minlength=self.ndof)
        if not need_tangent:
            return res, None
        data = np.empty(self.nnz)
        self.lib.orc_gather(self.nnz, _p(self.gather_ptr), _p(self.gather_idx), _p(ke), _p(data))
        return res, CSR(self.indptr, self.indices, data, self.ndof)

    # --- solver hooks (cpfem_oracle.solver calls them when present) --------------------
    def zero_rows(self, A, bc_dofs):
        rows = _c(np.unique(bc_dofs), np.int64)
        self.lib.orc_zero_rows(rows.size, _p(rows), _p(A.indptr), _p(A.indices), _p(A.data))
        return A

    def linear_solve(self, A, b, x0):
        x = _c(x0).copy()
        b = _c(b)
        minv = 1.0 / A.diagonal()
        k = np.zeros(1, dtype=np.int32)
        rc = self.lib.orc_bicgstab(A.shape[0], _p(A.indptr), _p(A.indices), _p(A.data), _p(b), _p(x), _p(minv),
                                   1e-10, 1e-10, 10000, _p(k))
        if rc:
            raise MemoryError("oracle BiCGSTAB workspace")
        return x, int(k[0])

    # --- post-processing / state update ---------------------------------------------
    def compute_avg_stress(self, sol, params):
        o = self._gp(sol, params, sigma=True)
        sig = o["sigma"].reshape(self.E, 8, 3, 3)
        return np.einsum("eqij,eq->eij", sig, self.jxw) / self.jxw.sum(1)[:, None, None]

    def update_int_vars_gp(self, sol, params):
        o = self._gp(sol, params, state=True)
        E, N = self.E, self.N
        return [o["Fpi_new"].reshape(E, 8, 3, 3), o["g_new"].reshape(E, 8, N), o["slip_new"].reshape(E, 8, N)] + \
            [p.copy() for p in params[3:]]

    def gp_outputs(self, sol, params):
        """P, dP/dF and the new state at every GP (for per-GP comparisons)."""
        return self._gp(sol, params, P=True, D=True, state=True)
