"""Crystal data and material specifications.

Slip systems are listed in the order of the reference data files, because the
latent-hardening matrix groups rows by the index rule 3*floor(i/3)
(``singlecrystal_copper/models_copper.py:71-76``):

* FCC {111}<110>, 12 systems: ``singlecrystal_copper/data/csv/input_slip_sys.txt``
* BCC {110}<111>, 12 systems: ``polycrystal_DPsteel/data/csv/input_slip_sys_bcc12.txt``
* BCC {110}<111> + {112}<111>, 24 systems: ``polycrystal_DPsteel/data/csv/input_slip_sys_bcc24.txt``

Each row is ``plane normal (3), slip direction (3)``; both are normalised when used
(``models_copper.py:59-66``).
"""
from __future__ import annotations

import dataclasses

import numpy as np

from . import _capi

FCC12 = ((1, 1, -1, 0, 1, 1), (1, 1, -1, 1, 0, 1), (1, 1, -1, 1, -1, 0),
         (1, -1, -1, 0, 1, -1), (1, -1, -1, 1, 0, 1), (1, -1, -1, 1, 1, 0),
         (1, -1, 1, 0, 1, 1), (1, -1, 1, 1, 0, -1), (1, -1, 1, 1, 1, 0),
         (1, 1, 1, 0, 1, -1), (1, 1, 1, 1, 0, -1), (1, 1, 1, 1, -1, 0))

BCC12 = ((1, 1, 0, -1, 1, 1), (1, 1, 0, 1, -1, 1), (1, -1, 0, 1, 1, 1), (1, -1, 0, 1, 1, -1),
         (1, 0, 1, 1, 1, -1), (1, 0, 1, -1, 1, 1), (1, 0, -1, 1, 1, 1), (1, 0, -1, 1, -1, 1),
         (0, 1, 1, 1, 1, -1), (0, 1, 1, 1, -1, 1), (0, 1, -1, 1, 1, 1), (0, 1, -1, -1, 1, 1))

BCC24 = BCC12 + ((1, 1, 2, 1, 1, -1), (-1, 1, 2, 1, -1, 1), (1, -1, 2, -1, 1, 1), (1, 1, -2, 1, 1, 1),
                 (1, 2, 1, 1, -1, 1), (-1, 2, 1, 1, 1, -1), (1, -2, 1, 1, 1, 1), (1, 2, -1, -1, 1, 1),
                 (2, 1, 1, -1, 1, 1), (-2, 1, 1, 1, 1, 1), (2, -1, 1, 1, 1, -1), (2, 1, -1, 1, -1, 1))

SLIP_SYSTEMS = {"fcc12": FCC12, "bcc12": BCC12, "bcc24": BCC24}


@dataclasses.dataclass
class MaterialSpec:
    """Constants a reference ``custom_init`` / ``get_maps`` hard-codes.

    ``coplanar_q`` selects the latent-hardening matrix: True builds q = r with ones on
    the coplanar 3-blocks (``models_copper.py:71-76``); False is q = r everywhere, which
    is what the parameterised models compute because their ``q.at[].set`` result is
    discarded (``crystal_plasticity_OR_design/models_sens_rot.py:170-175``).
    ``per_gp_params`` selects the internal-variable layout: False gives the 4-entry
    list of the plain models, True the 9-entry list of the parameterised ones.
    ``phases`` makes a multi-phase material (``polycrystal_DPsteel/models_DPsteel_inhomo.py``):
    one spec per phase supplies that phase's elastic constants, initial slip resistance
    and Kalidindi parameters, each cell belongs to one phase, and the internal variables
    are the 10-entry list of that model (the 9 entries plus the lattice-frame stiffness
    C per GP, ``models_DPsteel_inhomo.py:229``).  ``phase1_fraction`` is the volume
    fraction of phase 1 when the cells' phases are drawn the way that model draws them.
    """
    C11: float
    C12: float
    C44: float
    gss_initial: float
    h: float
    t_sat: float
    gss_a: float
    xm: float
    r: float = 1.0
    ao: float = 1e-3
    slip: str = "fcc12"
    coplanar_q: bool = True
    per_gp_params: bool = False
    local_tol: float = 1e-8
    max_sub_step: int = 5
    max_iter: int = 300
    phases: tuple = ()
    phase1_fraction: float = 0.4

    def replace(self, **kw):
        return dataclasses.replace(self, **kw)

    def slip_vectors(self):
        t = np.asarray(SLIP_SYSTEMS[self.slip], dtype=np.float64)
        n = t[:, :3] / np.linalg.norm(t[:, :3], axis=1)[:, None]
        d = t[:, 3:] / np.linalg.norm(t[:, 3:], axis=1)[:, None]
        return d, n

    @property
    def num_slip(self):
        return len(SLIP_SYSTEMS[self.slip])

    def to_ctypes(self):
        m = _capi.Material()
        d, n = self.slip_vectors()
        m.num_slip = d.shape[0]
        m.qmode = 1 if self.coplanar_q else 0
        m.max_sub_step = int(self.max_sub_step)
        m.max_iter = int(self.max_iter)
        m.local_tol = float(self.local_tol)
        m.ao = float(self.ao)
        m.C11, m.C12, m.C44 = float(self.C11), float(self.C12), float(self.C44)
        for a in range(d.shape[0]):
            for i in range(3):
                m.slip_d[a][i] = d[a, i]
                m.slip_n[a][i] = n[a, i]
        return m

    def param_row(self):
        """(gss_a, h, t_sat, xm, r) -- the order of the parameterised internal variables."""
        return np.array([self.gss_a, self.h, self.t_sat, self.xm, self.r], dtype=np.float64)

    def elastic_row(self):
        return np.array([self.C11, self.C12, self.C44], dtype=np.float64)

    @property
    def num_internal_vars(self):
        return 10 if self.phases else (9 if self.per_gp_params else 4)


# Constants of the reference models (file:line of each ``custom_init`` / ``get_maps``).
COPPER = MaterialSpec(  # singlecrystal_copper/models_copper.py:55-56,94-96,141-149
    C11=1.684e5, C12=1.214e5, C44=0.754e5, gss_initial=60.8, h=541.5, t_sat=109.8, gss_a=2.5,
    xm=0.1, r=1.0, slip="fcc12", coplanar_q=True, local_tol=1e-8, max_sub_step=5)
CALIB_CASE1 = COPPER.replace(coplanar_q=False, per_gp_params=True)  # calibration/case1.py
CALIB_CASE2 = MaterialSpec(  # calibration/case2.py (Ta, BCC12)
    C11=2.670e5, C12=1.610e5, C44=0.825e5, gss_initial=67.4641, h=1959.1320, t_sat=7295.1754,
    gss_a=200.0, xm=1.0 / 45.2726, r=1.0, slip="bcc12", coplanar_q=False, per_gp_params=True,
    local_tol=1e-8, max_sub_step=5)
CALIB_CASE4 = MaterialSpec(  # calibration/case4.py (304 steel, FCC)
    C11=2.622e5, C12=1.120e5, C44=0.746e5, gss_initial=90.0, h=392.9772, t_sat=7295.1754,
    gss_a=8.0, xm=1.0 / 120.0, r=1.0, slip="fcc12", coplanar_q=False, per_gp_params=True,
    local_tol=1e-8, max_sub_step=8)
SENS_ROT = COPPER.replace(coplanar_q=False, per_gp_params=True, local_tol=1e-6, max_sub_step=10)
STEEL304 = CALIB_CASE4.replace(coplanar_q=True, per_gp_params=False)   # polycrystal_304steel/models_304steel.py
TANTALUM = CALIB_CASE2.replace(coplanar_q=True, per_gp_params=False)   # singlecrystal_tantalum/models_tantalum.py

# The benchmark configurations (GPa in the specification, MPa here).
BENCH_COPPER = MaterialSpec(
    C11=168.4e3, C12=121.4e3, C44=75.4e3, gss_initial=16.0, h=250.0, t_sat=190.0, gss_a=2.25,
    xm=0.05, r=1.4, slip="fcc12", coplanar_q=True)
BENCH_STEEL = MaterialSpec(
    C11=204.6e3, C12=137.7e3, C44=126.2e3, gss_initial=90.0, h=200.0, t_sat=300.0, gss_a=2.0,
    xm=0.05, r=1.4, slip="fcc12", coplanar_q=True)
BENCH_TANTALUM = MaterialSpec(
    C11=267.0e3, C12=161.0e3, C44=82.5e3, gss_initial=160.0, h=150.0, t_sat=300.0, gss_a=1.5,
    xm=0.05, r=1.4, slip="bcc24", coplanar_q=True)

# Dual-phase steel, ferrite (phase 0) + martensite (phase 1), BCC24 with the coplanar
# 3-block q (polycrystal_DPsteel/models_DPsteel_inhomo.py:55-100,145-179,257-266).
DP_FERRITE = MaterialSpec(
    C11=2.314e5, C12=1.347e5, C44=1.164e5, gss_initial=170.0, h=400.0, t_sat=2500.0, gss_a=4.0,
    xm=0.05, r=1.0, slip="bcc24", coplanar_q=True, per_gp_params=True, local_tol=1e-8, max_sub_step=5)
DP_MARTENSITE = DP_FERRITE.replace(C11=4.174e5, C12=2.424e5, C44=2.111e5, gss_initial=435.0, h=950.0,
                                   t_sat=5300.0)
DP_STEEL = DP_FERRITE.replace(phases=(DP_FERRITE, DP_MARTENSITE), phase1_fraction=0.4)


def rot_mat(quat):
    """Quaternion (scalar first, used as given) -> rotation matrix
    (``models_copper.py:37-48``)."""
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


def euler_zyx_deg(angles):
    """Rotation matrices of lowercase 'zyx' Euler angles in degrees, i.e. extrinsic
    rotations about z, then y, then x: R = Rx(c) Ry(b) Rz(a) for angles (a, b, c) --
    ``scipy.spatial.transform.Rotation.from_euler('zyx', ..., degrees=True)`` as used at
    ``crystal_plasticity_OR_design/poly_sensitivity_rot_mesh2.py:41-55``."""
    ang = np.deg2rad(np.asarray(angles, dtype=np.float64))
    a, b, c = ang[..., 0], ang[..., 1], ang[..., 2]
    ca, sa, cb, sb, cc, sc = np.cos(a), np.sin(a), np.cos(b), np.sin(b), np.cos(c), np.sin(c)
    z = np.zeros_like(a)
    o = np.ones_like(a)
    Rz = np.stack([ca, -sa, z, sa, ca, z, z, z, o], -1).reshape(ang.shape[:-1] + (3, 3))
    Ry = np.stack([cb, z, sb, z, o, z, -sb, z, cb], -1).reshape(ang.shape[:-1] + (3, 3))
    Rx = np.stack([o, z, z, z, cc, -sc, z, sc, cc], -1).reshape(ang.shape[:-1] + (3, 3))
    return Rx @ Ry @ Rz


def cubic_tensor(rows):
    """(..., 3) rows of (C11, C12, C44) -> (..., 3, 3, 3, 3) cubic stiffness in the lattice
    frame, as the reference fills C (``models_copper.py:92-130``)."""
    rows = np.asarray(rows, dtype=np.float64)
    C = np.zeros(rows.shape[:-1] + (3, 3, 3, 3))
    for i in range(3):
        for j in range(3):
            C[..., i, i, j, j] = rows[..., 0] if i == j else rows[..., 1]
            if i != j:
                C[..., i, j, i, j] = rows[..., 2]
                C[..., i, j, j, i] = rows[..., 2]
    return C


def cubic_constants(C, tol=1e-9):
    """Inverse of ``cubic_tensor`` for (..., 3, 3, 3, 3) arrays; raises unless C has the
    cubic form (the constitutive kernel stores three constants per stiffness)."""
    C = np.asarray(C, dtype=np.float64)
    rows = np.stack([C[..., 0, 0, 0, 0], C[..., 0, 0, 1, 1], C[..., 1, 2, 1, 2]], -1)
    scale = max(float(np.abs(C).max()) if C.size else 1.0, 1e-300)
    if C.size and float(np.abs(cubic_tensor(rows) - C).max()) > tol * scale:
        raise ValueError("per-GP stiffness must have the cubic form (C11, C12, C44) in the lattice frame")
    return rows


def random_quaternions(rng, n):
    """Uniform orientations on SO(3): normalised Gaussian quaternions."""
    q = rng.normal(size=(n, 4))
    return q / np.linalg.norm(q, axis=1)[:, None]


def check_orthonormal(R, tol=1e-10):
    """The lattice-frame local solve needs proper orthonormal rotations."""
    R = np.asarray(R, dtype=np.float64).reshape(-1, 3, 3)
    err = np.abs(np.einsum("gki,gkj->gij", R, R) - np.eye(3)).max() if R.size else 0.0
    det = np.linalg.det(R) if R.size else np.ones(1)
    if err > tol or np.abs(det - 1.0).max() > tol:
        raise ValueError(f"rotations must be orthonormal with det +1 (max |R^T R - I| = {err:.3e}); "
                         "normalise the quaternions")
    return R


__all__ = ["MaterialSpec", "FCC12", "BCC12", "BCC24", "SLIP_SYSTEMS", "rot_mat", "euler_zyx_deg",
           "random_quaternions", "check_orthonormal", "COPPER", "CALIB_CASE1", "CALIB_CASE2",
           "CALIB_CASE4", "SENS_ROT", "STEEL304", "TANTALUM", "BENCH_COPPER", "BENCH_STEEL", "BENCH_TANTALUM",
           "DP_FERRITE", "DP_MARTENSITE", "DP_STEEL", "cubic_tensor", "cubic_constants"]
