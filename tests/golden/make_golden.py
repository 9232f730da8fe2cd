"""Regenerate the golden fixtures of this directory from the reference checkout.

Reads (paths relative to the reference project root):
  calibration/data/csv/calibration_case1/stress_strain_curve_copper.txt  sigma_zz, 1-element copper
  calibration/data/csv/calibration_case2/ss_curve_e-2.txt                sigma_zz, 1-element Ta (BCC12)
  calibration/data/csv/calibration_case4/UQ/stress_zz_curve_scenario0.txt  mean sigma_zz, 20^3, 50 grains
  calibration/data/csv/calibration_case4/UQ/stress_xx_curve_scenario1.txt  mean sigma_xx, x-loaded twin
  calibration/data/csv/calibration_case4/quat.txt                         orientations (rows 0..49)
  calibration/data/neper/calibration_case4/UQ/n50-id0.msh                 grain of every voxel cell
and writes ``golden.npz``.  The 20^3 Neper mesh is checked to be the structured box of
side 0.0295 with x-fastest node numbering, so only its per-cell grain ids are stored.

Usage: python tests/golden/make_golden.py [reference_root]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"


def read_msh(path):
    lines = open(path).read().split("\n")
    i = lines.index("$Nodes")
    n = int(lines[i + 1])
    pts = np.array([[float(v) for v in lines[i + 2 + k].split()[1:4]] for k in range(n)])
    i = lines.index("$Elements")
    m = int(lines[i + 1])
    cells, tags = [], []
    for k in range(m):
        p = [int(v) for v in lines[i + 2 + k].split()]
        if p[1] == 5:
            tags.append(p[3])
            cells.append(p[3 + p[2]:3 + p[2] + 8])
    return pts, np.array(cells) - 1, np.array(tags) - 1


def main():
    c = os.path.join(REF, "calibration/data/csv")
    case1 = np.loadtxt(os.path.join(c, "calibration_case1/stress_strain_curve_copper.txt"))
    case2 = np.loadtxt(os.path.join(c, "calibration_case2/ss_curve_e-2.txt"))
    c4zz = np.loadtxt(os.path.join(c, "calibration_case4/UQ/stress_zz_curve_scenario0.txt"))
    c4xx = np.loadtxt(os.path.join(c, "calibration_case4/UQ/stress_xx_curve_scenario1.txt"))
    quat = np.loadtxt(os.path.join(c, "calibration_case4/quat.txt"))[:50, 1:]
    pts, cells, grains = read_msh(os.path.join(REF, "calibration/data/neper/calibration_case4/UQ/n50-id0.msh"))
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    from oracle.cpfem_oracle import box_mesh
    bp, bc = box_mesh(20, 20, 20, 0.0295, 0.0295, 0.0295)
    assert np.abs(bp - pts).max() < 1e-9, "case4 mesh is not the structured box"
    assert (bc == cells).all(), "case4 connectivity differs from the structured box"
    np.savez_compressed(os.path.join(HERE, "golden.npz"), case1_szz=case1, case2_szz=case2,
                        case4_szz=c4zz, case4_sxx=c4xx, case4_quat=quat,
                        case4_grain=grains.astype(np.int16))
    print("wrote golden.npz", case1.shape, case2.shape, c4zz.shape, c4xx.shape, quat.shape, grains.shape)


if __name__ == "__main__":
    main()
