"""VTU (VTK XML unstructured grid) output and input for HEX8 results.

The reference writes one VTU per load step through JAX-FEM's ``save_sol``
(``singlecrystal_copper/singlecrystal_copper.py:232-233``,
``polycrystal_304steel/polycrystal_304steel.py:265``), which uses meshio: inline base64
binary DataArrays, zlib-compressed (``vtkZLibDataCompressor``, UInt32 headers).  This module
writes the same layout -- the displacement ``sol`` as point data, any per-cell fields as
cell data -- so ParaView and meshio read it, and reads such files back (also the
reference's own golden outputs).
"""
from __future__ import annotations

import base64
import re
import zlib

import numpy as np

_VTK_HEXAHEDRON = 12
_TYPES = {np.dtype(np.float64): "Float64", np.dtype(np.float32): "Float32", np.dtype(np.int64): "Int64",
          np.dtype(np.int32): "Int32", np.dtype(np.uint8): "UInt8"}
_DTYPES = {v: k for k, v in _TYPES.items()}
_BLOCK = 32768


def _encode(arr, compress=True):
    raw = np.ascontiguousarray(arr).tobytes()
    if not compress:
        head = np.array([len(raw)], dtype=np.uint32).tobytes()
        return base64.b64encode(head + raw).decode()
    blocks = [raw[i:i + _BLOCK] for i in range(0, len(raw), _BLOCK)] or [b""]
    comp = [zlib.compress(b) for b in blocks]
    last = len(blocks[-1]) if blocks else 0
    head = np.array([len(blocks), _BLOCK, last] + [len(c) for c in comp], dtype=np.uint32)
    return base64.b64encode(head.tobytes()).decode() + base64.b64encode(b"".join(comp)).decode()


def _decode(text, dtype, compressed=True):
    text = "".join(text.split())
    if not compressed:
        raw = base64.b64decode(text)
        n = int(np.frombuffer(raw[:4], dtype=np.uint32)[0])
        return np.frombuffer(raw[4:4 + n], dtype=dtype)
    first = base64.b64decode(text[:16])
    nb = int(np.frombuffer(first[:4], dtype=np.uint32)[0])
    hlen = 4 * (3 + nb)
    hchars = 4 * ((hlen + 2) // 3)
    head = np.frombuffer(base64.b64decode(text[:hchars])[:hlen], dtype=np.uint32)
    data = base64.b64decode(text[hchars:])
    out, off = [], 0
    for c in head[3:3 + nb]:
        out.append(zlib.decompress(data[off:off + int(c)]))
        off += int(c)
    return np.frombuffer(b"".join(out), dtype=dtype)


def _array(name, arr, ncomp=1, compress=True):
    arr = np.asarray(arr)
    t = _TYPES[arr.dtype]
    nc = f' NumberOfComponents="{ncomp}"' if ncomp > 1 else ""
    return f'<DataArray type="{t}" Name="{name}"{nc} format="binary">\n{_encode(arr, compress)}\n</DataArray>\n'


def write_vtu(path, points, cells, point_data=None, cell_data=None, compress=True):
    """Write a HEX8 mesh with point data (e.g. ``sol``, (n,3)) and cell data (e.g. cell
    stresses, (E,) or (E,k)) as a VTU file."""
    points = np.asarray(points, dtype=np.float64)
    cells = np.asarray(cells, dtype=np.int64)
    E = cells.shape[0]
    comp = ' compressor="vtkZLibDataCompressor"' if compress else ""
    out = ['<?xml version="1.0"?>\n',
           f'<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian"{comp}>\n',
           '<UnstructuredGrid>\n', f'<Piece NumberOfPoints="{points.shape[0]}" NumberOfCells="{E}">\n',
           '<Points>\n', _array("Points", points, 3, compress), '</Points>\n', '<Cells>\n',
           _array("connectivity", cells.reshape(-1), 1, compress),
           _array("offsets", 8 * np.arange(1, E + 1, dtype=np.int64), 1, compress),
           _array("types", np.full(E, _VTK_HEXAHEDRON, dtype=np.uint8), 1, compress), '</Cells>\n']
    if point_data:
        out.append("<PointData>\n")
        for k, v in point_data.items():
            v = np.asarray(v)
            out.append(_array(k, v.reshape(points.shape[0], -1), v.reshape(points.shape[0], -1).shape[1], compress))
        out.append("</PointData>\n")
    if cell_data:
        out.append("<CellData>\n")
        for k, v in cell_data.items():
            v = np.asarray(v)
            out.append(_array(k, v.reshape(E, -1), v.reshape(E, -1).shape[1], compress))
        out.append("</CellData>\n")
    out += ["</Piece>\n", "</UnstructuredGrid>\n", "</VTKFile>\n"]
    with open(path, "w") as f:
        f.write("".join(out))


def read_vtu(path):
    """Read a VTU written by ``write_vtu`` or meshio (inline binary, optional zlib):
    returns dict(points, cells, point_data, cell_data)."""
    text = open(path).read()
    compressed = "vtkZLibDataCompressor" in text[:400]
    res = {"point_data": {}, "cell_data": {}}
    sections = {"PointData": "point_data", "CellData": "cell_data"}
    for sec, key in sections.items():
        m = re.search(f"<{sec}>(.*?)</{sec}>", text, re.S)
        if m:
            for a in re.finditer(r'<DataArray type="(\w+)" Name="([^"]+)"(?: NumberOfComponents="(\d+)")?[^>]*>'
                                 r'(.*?)</DataArray>', m.group(1), re.S):
                arr = _decode(a.group(4), _DTYPES[a.group(1)], compressed)
                nc = int(a.group(3) or 1)
                res[key][a.group(2)] = arr.reshape(-1, nc) if nc > 1 else arr
    m = re.search(r'<Points>.*?<DataArray type="(\w+)"[^>]*>(.*?)</DataArray>', text, re.S)
    res["points"] = _decode(m.group(2), _DTYPES[m.group(1)], compressed).reshape(-1, 3)
    m = re.search(r'<DataArray type="(\w+)" Name="connectivity"[^>]*>(.*?)</DataArray>', text, re.S)
    res["cells"] = _decode(m.group(2), _DTYPES[m.group(1)], compressed).reshape(-1, 8)
    return res


def save_sol(fe, sol, path, cell_infos=None):
    """JAX-FEM's ``save_sol(fe, sol, vtk_path, cell_infos=[(name, data), ...])`` signature."""
    cd = {}
    for name, data in (cell_infos or []):
        cd[name] = data.detach().cpu().numpy() if hasattr(data, "detach") else np.asarray(data)
    s = sol.detach().cpu().numpy() if hasattr(sol, "detach") else np.asarray(sol)
    write_vtu(path, fe.points, fe.cells_np, {"sol": s.reshape(-1, 3)}, cd)
