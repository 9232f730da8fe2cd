"""Regenerate the golden fixtures of this directory from the reference checkout.

Reads (paths relative to the reference project root):
  calibration/data/csv/calibration_case1/stress_strain_curve_copper.txt  sigma_zz, 1-element copper
  calibration/data/csv/calibration_case2/ss_curve_e-2.txt                sigma_zz, 1-element Ta (BCC12)
  calibration/data/csv/calibration_case4/UQ/stress_zz_curve_scenario0.txt  mean sigma_zz, 20^3, 50 grains
  calibration/data/csv/calibration_case4/UQ/stress_xx_curve_scenario1.txt  mean sigma_xx, x-loaded twin
  calibration/data/csv/calibration_case4/quat.txt                         orientations (rows 0..49)
  calibration/data/neper/calibration_case4/UQ/n50-id0.msh                 grain of every voxel cell
  polycrystal_304steel/data/vtk/polycrystal_304steel/u_000..015.vtu     per-cell stresses, 16^3, 8 grains
  polycrystal_304steel/data/csv/polycrystal_304steel/quat.txt            its orientations
  singlecrystal_tantalum/data/vtk/singlecrystal_tantalum/u_000..049.vtu  per-cell stresses, 10^3 single crystal
  polycrystal_DPsteel/data/vtk/polycrystal_DPsteel/u_inhomo_000..049.vtu  per-cell stresses, phases and
                                                                          orientation indices, 10^3 DP steel
  polycrystal_DPsteel/data/csv/polycrystal_DPsteel/quat.txt              its orientations (8 rows)
and writes ``golden.npz``.  The Neper meshes (20^3 of case 4, 16^3 of the 304-steel VTUs,
10^3 of the tantalum VTUs) are checked to be structured boxes with x-fastest node
numbering, so only per-cell grain ids are stored.  The VTU fields are float32 (meshio).

The Neper mesh is read with the package's own gmsh 2.2 reader (``mesh.read_gmsh22``).

Usage: python tests/golden/make_golden.py REFERENCE_ROOT
       (or set CPFEM_REFERENCE_ROOT to the reference checkout)
"""
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))


def reference_root():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CPFEM_REFERENCE_ROOT")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py REFERENCE_ROOT (or set CPFEM_REFERENCE_ROOT): the reference checkout")
    return ref


def main():
    REF = reference_root()
    mesh_mod = importlib.import_module("jax-cpfem_gb300.mesh")
    c = os.path.join(REF, "calibration/data/csv")
    case1 = np.loadtxt(os.path.join(c, "calibration_case1/stress_strain_curve_copper.txt"))
    case2 = np.loadtxt(os.path.join(c, "calibration_case2/ss_curve_e-2.txt"))
    c4zz = np.loadtxt(os.path.join(c, "calibration_case4/UQ/stress_zz_curve_scenario0.txt"))
    c4xx = np.loadtxt(os.path.join(c, "calibration_case4/UQ/stress_xx_curve_scenario1.txt"))
    quat = np.loadtxt(os.path.join(c, "calibration_case4/quat.txt"))[:50, 1:]
    msh, grains = mesh_mod.read_gmsh22(os.path.join(REF, "calibration/data/neper/calibration_case4/UQ/n50-id0.msh"))
    pts, cells = msh.points, msh.cells
    from oracle.cpfem_oracle import box_mesh
    bp, bc = box_mesh(20, 20, 20, 0.0295, 0.0295, 0.0295)
    assert np.abs(bp - pts).max() < 1e-9, "case4 mesh is not the structured box"
    assert (bc == cells).all(), "case4 connectivity differs from the structured box"
    vtu = importlib.import_module("jax-cpfem_gb300.vtu")
    vdir = os.path.join(REF, "polycrystal_304steel/data/vtk/polycrystal_304steel")
    st = [vtu.read_vtu(os.path.join(vdir, f"u_{i:03d}.vtu")) for i in range(16)]
    bp, bc = box_mesh(16, 16, 16, 0.016, 0.016, 0.016)
    assert np.abs(bp - st[0]["points"]).max() < 1e-12 and (bc == st[0]["cells"]).all()
    steel_sig = np.stack([np.stack([r["cell_data"][f"sigma_{c}"] for c in ("xx", "yy", "zz")]) for r in st])
    steel_ori = st[0]["cell_data"]["cell_ori_inds"].astype(np.int16)
    steel_quat = np.loadtxt(os.path.join(REF, "polycrystal_304steel/data/csv/polycrystal_304steel/quat.txt"))[:8, 1:]
    tdir = os.path.join(REF, "singlecrystal_tantalum/data/vtk/singlecrystal_tantalum")
    ta = [vtu.read_vtu(os.path.join(tdir, f"u_{i:03d}.vtu")) for i in range(50)]
    L = ta[0]["points"].max()
    bp, bc = box_mesh(10, 10, 10, L, L, L)
    assert np.abs(bp - ta[0]["points"]).max() < 1e-12 and (bc == ta[0]["cells"]).all()
    ta_szz = np.stack([r["cell_data"]["sigma_zz"] for r in ta])
    ddir = os.path.join(REF, "polycrystal_DPsteel/data/vtk/polycrystal_DPsteel")
    dp = [vtu.read_vtu(os.path.join(ddir, f"u_inhomo_{i:03d}.vtu")) for i in range(50)]
    bp, bc = box_mesh(10, 10, 10, 2.0, 2.0, 2.0)
    assert np.abs(bp - dp[0]["points"]).max() < 1e-12 and (bc == dp[0]["cells"]).all()
    # The files were written by a run whose two phases had their elastic constants
    # exchanged relative to their Kalidindi parameters: the saved C11/C12/C44 fields carry
    # the martensite constants on the cells whose saved phase_inds is 0 (ferrite
    # parameters) and the ferrite constants on the others.  Both maps are kept: the phase
    # of the plastic parameters (phase_inds) and the phase of the stiffness (from C11).
    c11 = dp[0]["cell_data"]["C11"]
    assert set(np.unique(c11).tolist()) == {231400.0, 417400.0}
    dp_phase = dp[0]["cell_data"]["phase_inds"].astype(np.int8)
    dp_stiff_phase = (c11 > 3.0e5).astype(np.int8)
    assert (dp_stiff_phase == 1 - dp_phase).all()
    dp_ori = dp[0]["cell_data"]["cell_ori_inds"].astype(np.int16)
    assert all((r["cell_data"]["phase_inds"] == dp[0]["cell_data"]["phase_inds"]).all() for r in dp)
    dp_sig = np.stack([np.stack([r["cell_data"][f"sigma_{c}"] for c in ("xx", "yy", "zz")]) for r in dp])
    dp_quat = np.loadtxt(os.path.join(REF, "polycrystal_DPsteel/data/csv/polycrystal_DPsteel/quat.txt"))[:20, 1:]
    np.savez_compressed(os.path.join(HERE, "golden.npz"), case1_szz=case1, case2_szz=case2,
                        case4_szz=c4zz, case4_sxx=c4xx, case4_quat=quat,
                        case4_grain=grains.astype(np.int16), steel_sig=steel_sig, steel_ori=steel_ori,
                        steel_quat=steel_quat, ta_szz=ta_szz, ta_L=np.array(L), dp_sig=dp_sig,
                        dp_phase=dp_phase, dp_stiff_phase=dp_stiff_phase, dp_ori=dp_ori, dp_quat=dp_quat)
    print("wrote golden.npz", case1.shape, case2.shape, c4zz.shape, c4xx.shape, quat.shape, grains.shape)


if __name__ == "__main__":
    main()
