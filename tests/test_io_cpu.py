"""Mesh and result file formats on the host: the gmsh 2.2 reader (Neper voxel meshes) and
the VTU writer/reader (meshio's inline-binary layout)."""
import importlib
import os

import numpy as np
import pytest


@pytest.fixture(scope="module")
def io():
    mesh = importlib.import_module("jax-cpfem_gb300.mesh")
    vtu = importlib.import_module("jax-cpfem_gb300.vtu")
    return mesh, vtu


def _write_gmsh22(path, mesh, grain):
    """A Neper-like file: 1-based node ids in shuffled order, a non-hex element first, hex
    elements (type 5) with 3 tags, physical tag = grain + 1."""
    rng = np.random.default_rng(0)
    perm = rng.permutation(mesh.points.shape[0])
    node_id = np.empty_like(perm)
    node_id[perm] = np.arange(1, perm.size + 1) * 3          # non-contiguous ids
    lines = ["$MeshFormat", "2.2 0 8", "$EndMeshFormat", "$Nodes", str(perm.size)]
    for k in perm:
        x, y, z = mesh.points[k]
        lines.append(f"{node_id[k]} {float(x)!r} {float(y)!r} {float(z)!r}")
    lines += ["$EndNodes", "$Elements", str(mesh.cells.shape[0] + 1), "1 15 2 1 1 3"]
    for e, c in enumerate(mesh.cells):
        lines.append(f"{e + 2} 5 3 {grain[e] + 1} {grain[e] + 1} 0 " + " ".join(str(node_id[v]) for v in c))
    lines += ["$EndElements", ""]
    path.write_text("\n".join(lines))


def test_gmsh22_reader_recovers_mesh_and_grains(io, tmp_path):
    mesh_mod, _ = io
    m = mesh_mod.box_mesh(3, 2, 2, 1.0, 2.0, 0.5)
    grain = np.arange(m.cells.shape[0]) % 5
    f = tmp_path / "domain.msh"
    _write_gmsh22(f, m, grain)
    got, g = mesh_mod.read_gmsh22(str(f))
    assert np.array_equal(g, grain)
    # same cells up to the node renumbering: compare coordinates cell by cell
    assert np.allclose(got.points[got.cells], m.points[m.cells])
    assert mesh_mod.structured_dims(m.points) == (4, 3, 3)


@pytest.mark.parametrize("compress", [True, False])
def test_vtu_round_trip(io, tmp_path, compress):
    mesh_mod, vtu = io
    m = mesh_mod.box_mesh(4, 3, 2)
    rng = np.random.default_rng(1)
    sol = rng.normal(size=(m.points.shape[0], 3))
    sig = rng.normal(size=(m.cells.shape[0],)).astype(np.float32)
    ori = np.arange(m.cells.shape[0], dtype=np.int64) % 7
    f = tmp_path / "u_000.vtu"
    vtu.write_vtu(str(f), m.points, m.cells, {"sol": sol}, {"sigma_zz": sig, "cell_ori_inds": ori},
                  compress=compress)
    r = vtu.read_vtu(str(f))
    assert np.array_equal(r["points"], m.points) and np.array_equal(r["cells"], m.cells)
    assert np.array_equal(r["point_data"]["sol"], sol)
    assert np.array_equal(r["cell_data"]["sigma_zz"], sig)
    assert np.array_equal(r["cell_data"]["cell_ori_inds"], ori)
    text = f.read_text()
    assert text.startswith('<?xml version="1.0"?>') and 'type="UnstructuredGrid"' in text
    assert ("vtkZLibDataCompressor" in text) == compress


# The reference's own Neper meshes, read where the reference checkout is available (set
# CPFEM_REFERENCE_ROOT to it; the golden fixtures were generated the same way).
_REF = os.environ.get("CPFEM_REFERENCE_ROOT")
NEPER_MESHES = [("calibration/data/neper/calibration_case4/UQ/n50-id0.msh", 20, 0.0295, 50),
                ("singlecrystal_tantalum/data/neper/singlecrystal_tantalum/mesh10.msh", 10, None, 1),
                ("polycrystal_DPsteel/data/neper/polycrystal_DPsteel/n1-id0-mesh16.msh", 16, None, 1),
                ("crystal_plasticity_OR_design/data/neper/sensitivity/mesh2.msh", 2, None, None)]


@pytest.mark.skipif(not (_REF and os.path.isdir(_REF)), reason="CPFEM_REFERENCE_ROOT is not set")
@pytest.mark.parametrize("rel,n,L,grains", NEPER_MESHES)
def test_gmsh22_reader_on_reference_neper_meshes(io, rel, n, L, grains):
    """Neper voxel meshes of the reference: a structured n^3 box numbered x fastest with
    gmsh-ordered HEX8 cells (what the multigrid levels and the golden fixtures assume), and
    the physical tag minus one as the grain (``calibration_case4_..._1D_GB.py:116``)."""
    mesh_mod, _ = io
    m, g = mesh_mod.read_gmsh22(os.path.join(_REF, rel))
    assert m.cells.shape == (n ** 3, 8)
    assert mesh_mod.structured_dims(m.points) == (n + 1, n + 1, n + 1)
    Lx = float(m.points[:, 0].max()) if L is None else L
    box = mesh_mod.box_mesh(n, n, n, Lx, Lx, Lx)
    assert np.abs(box.points - m.points).max() < 1e-9 * max(Lx, 1.0)
    assert np.array_equal(box.cells, m.cells)
    assert g.min() >= 0
    if grains is not None:
        assert g.max() + 1 == grains
    if rel.startswith("calibration"):
        gold = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))
        assert np.array_equal(g, gold["case4_grain"])
