"""HEX8 meshes: structured boxes, Voronoi grain maps, gmsh 2.2 files and the
shape-function gradients / JxW that JAX-FEM's ``FiniteElement`` provides
(``fes[0].shape_grads``, ``fes[0].JxW``; used at ``singlecrystal_copper/models_copper.py:277,315``).

Element: trilinear HEX8, gmsh node order, 2x2x2 Gauss points at +-1/sqrt(3), weight 1.
"""
from __future__ import annotations

import dataclasses

import numpy as np

_REF_NODES = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                       [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], dtype=np.float64)
_GP = 1.0 / np.sqrt(3.0)
QUAD_POINTS = np.array([[x, y, z] for z in (-_GP, _GP) for y in (-_GP, _GP) for x in (-_GP, _GP)])


@dataclasses.dataclass
class Mesh:
    """Same fields as ``jax_fem.generate_mesh.Mesh``: points (n,3) and cells (E,8)."""
    points: np.ndarray
    cells: np.ndarray

    def __post_init__(self):
        self.points = np.ascontiguousarray(self.points, dtype=np.float64)
        self.cells = np.ascontiguousarray(self.cells, dtype=np.int64)


def box_mesh(nx, ny, nz, Lx=1.0, Ly=1.0, Lz=1.0):
    """Structured box: node (i,j,k) has id i + (nx+1)(j + (ny+1)k) (x fastest, like the
    Neper/gmsh files the reference reads), cells in gmsh HEX8 order."""
    xs = np.linspace(0.0, Lx, nx + 1)
    ys = np.linspace(0.0, Ly, ny + 1)
    zs = np.linspace(0.0, Lz, nz + 1)
    Z, Y, X = np.meshgrid(zs, ys, xs, indexing="ij")
    points = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
    k, j, i = (a.ravel() for a in np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij"))

    def nid(ii, jj, kk):
        return ii + (nx + 1) * (jj + (ny + 1) * kk)

    cells = np.stack([nid(i, j, k), nid(i + 1, j, k), nid(i + 1, j + 1, k), nid(i, j + 1, k),
                      nid(i, j, k + 1), nid(i + 1, j, k + 1), nid(i + 1, j + 1, k + 1),
                      nid(i, j + 1, k + 1)], axis=1)
    return Mesh(points, cells)


def structured_dims(points, rtol=1e-9):
    """Node counts (nx, ny, nz) per direction when the points are a tensor grid numbered
    x fastest (box meshes, the reference's Neper voxel meshes), else None."""
    P = np.asarray(points, dtype=np.float64)
    if P.ndim != 2 or P.shape[1] != 3 or P.shape[0] == 0:
        return None
    span = max(float(np.ptp(P, axis=0).max()), 1e-300)
    tol = rtol * span
    # the first row (x fastest) ends where y first changes, the first plane where z does
    row = np.nonzero(np.abs(P[:, 1] - P[0, 1]) > tol)[0]
    nx = int(row[0]) if row.size else P.shape[0]
    plane = np.nonzero(np.abs(P[:, 2] - P[0, 2]) > tol)[0]
    nxy = int(plane[0]) if plane.size else P.shape[0]
    if nx < 1 or nxy % nx or P.shape[0] % nxy:
        return None
    ny, nz = nxy // nx, P.shape[0] // nxy
    gx, gy, gz = P[:nx, 0], P[:nxy:nx, 1], P[::nxy, 2]
    grid = np.stack(np.meshgrid(gz, gy, gx, indexing="ij")[::-1], axis=-1).reshape(-1, 3)
    if np.abs(grid - P).max() > tol:
        return None
    return nx, ny, nz


def voronoi_grains(mesh, num_grains, seed):
    """Grain id per cell: seeds uniform in the bounding box from ``default_rng(seed)``,
    each cell assigned to the seed nearest its centroid (Euclidean, non-periodic)."""
    rng = np.random.default_rng(seed)
    lo, hi = mesh.points.min(0), mesh.points.max(0)
    seeds = lo + rng.uniform(0.0, 1.0, (num_grains, 3)) * (hi - lo)
    cent = mesh.points[mesh.cells].mean(axis=1)
    out = np.empty(cent.shape[0], dtype=np.int64)
    for s in range(0, cent.shape[0], 65536):
        c = cent[s:s + 65536]
        d2 = ((c[:, None, :] - seeds[None, :, :]) ** 2).sum(-1)
        out[s:s + 65536] = d2.argmin(1)
    return out, rng


def _dN_dxi(xi):
    t = 1.0 + _REF_NODES * xi[None, :]
    d = np.empty((8, 3))
    d[:, 0] = 0.125 * _REF_NODES[:, 0] * t[:, 1] * t[:, 2]
    d[:, 1] = 0.125 * _REF_NODES[:, 1] * t[:, 0] * t[:, 2]
    d[:, 2] = 0.125 * _REF_NODES[:, 2] * t[:, 0] * t[:, 1]
    return d


def shape_grads_jxw(mesh, chunk=131072):
    """dN_a/dX at every quad point, (E, 8 quads, 8 nodes, 3), and JxW (E, 8)."""
    E = mesh.cells.shape[0]
    sg = np.empty((E, 8, 8, 3))
    jxw = np.empty((E, 8))
    dNs = [_dN_dxi(xi) for xi in QUAD_POINTS]
    for s in range(0, E, chunk):
        X = mesh.points[mesh.cells[s:s + chunk]]
        for q, dN in enumerate(dNs):
            J = np.einsum("eai,aj->eij", X, dN)
            sg[s:s + chunk, q] = np.einsum("aj,eji->eai", dN, np.linalg.inv(J))
            jxw[s:s + chunk, q] = np.linalg.det(J)
    if (jxw <= 0).any():
        raise ValueError("inverted or degenerate HEX8 cell")
    return sg, jxw


def read_gmsh22(path):
    """Minimal gmsh 2.2 ASCII reader for Neper HEX8 output: returns (Mesh, grain id per
    cell) with the grain taken from the first (physical) tag minus one, as
    ``meshio_mesh.cell_data['gmsh:physical'][0] - 1`` gives it
    (``calibration/calibration_case4_UQ_polyCrystalSteel_1D_GB.py:116``)."""
    with open(path) as f:
        lines = f.read().split("\n")
    i = lines.index("$Nodes")
    n = int(lines[i + 1])
    ids = np.empty(n, dtype=np.int64)
    pts = np.empty((n, 3))
    for k in range(n):
        parts = lines[i + 2 + k].split()
        ids[k] = int(parts[0])
        pts[k] = [float(v) for v in parts[1:4]]
    remap = np.full(ids.max() + 1, -1, dtype=np.int64)
    remap[ids] = np.arange(n)
    i = lines.index("$Elements")
    m = int(lines[i + 1])
    cells, tags = [], []
    for k in range(m):
        parts = [int(v) for v in lines[i + 2 + k].split()]
        if parts[1] != 5:
            continue
        ntag = parts[2]
        tags.append(parts[3])
        cells.append(parts[3 + ntag:3 + ntag + 8])
    cells = remap[np.asarray(cells, dtype=np.int64)]
    return Mesh(pts, cells), np.asarray(tags, dtype=np.int64) - 1


def nodes_where(points, fn):
    """Indices of nodes for which ``fn(point)`` is true (a reference ``location_fn``)."""
    return np.nonzero(np.asarray([bool(fn(p)) for p in points]))[0]


def face_nodes(points, axis, value, atol=1e-5):
    return np.nonzero(np.isclose(points[:, axis], value, atol=atol))[0]


def corner_nodes(points, xyz, atol=1e-5):
    m = np.ones(points.shape[0], dtype=bool)
    for a, v in enumerate(xyz):
        m &= np.isclose(points[:, a], v, atol=atol)
    return np.nonzero(m)[0]
