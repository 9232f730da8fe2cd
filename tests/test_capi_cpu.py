"""Host-side checks that need no GPU: the shared library loads and exports every
declared entry point, the host pattern builder reproduces scipy's COO->CSR, host logic."""
import os
import re
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            names |= set(re.findall(r"^\s*(?:int|size_t|const char\*)\s+(cpfem_\w+)\s*\(", src, re.M))
    return names


@pytest.fixture(scope="module")
def lib(pkg):
    from importlib import import_module
    capi = import_module("jax-cpfem_gb300._capi")
    if not os.path.exists(capi.LIB_PATH):
        import_module("jax-cpfem_gb300.build").build()
    return capi.load()


def test_library_exports_every_declared_symbol(lib):
    names = _declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
    from importlib import import_module
    capi = import_module("jax-cpfem_gb300._capi")
    assert names == set(capi.SIGNATURES), names ^ set(capi.SIGNATURES)
    assert lib.cpfem_abi_version() == 3


def test_struct_layouts_match_the_library(lib):
    import ctypes
    from importlib import import_module
    capi = import_module("jax-cpfem_gb300._capi")
    for which, st in enumerate(capi.STRUCTS):
        assert lib.cpfem_struct_size(which) == ctypes.sizeof(st), st.__name__
    assert lib.cpfem_struct_size(len(capi.STRUCTS)) == 0
    # field offsets the kernels depend on: the FP32 V-cycle arrays follow the FP64 ones
    mg = capi.MGHierarchy
    assert mg.precision.offset == mg.scratch_nodes.offset + 8
    assert mg.b32.offset + 8 * capi.MG_MAX_LEVELS == ctypes.sizeof(mg)


def _pattern(lib, cells, n_nodes):
    cells = np.ascontiguousarray(cells, dtype=np.int32)
    nb = np.zeros(1, np.int64)
    assert lib.cpfem_pattern_count(cells.shape[0], cells.ctypes.data, n_nodes, nb.ctypes.data) == 0
    nb = int(nb[0])
    rp = np.zeros(n_nodes + 1, np.int32)
    cols = np.zeros(nb, np.int32)
    epos = np.zeros(cells.shape[0] * 64, np.uint8)
    tpos = np.zeros(nb, np.int32)
    assert lib.cpfem_pattern_build(cells.shape[0], cells.ctypes.data, n_nodes, rp.ctypes.data, cols.ctypes.data,
                                   epos.ctypes.data, tpos.ctypes.data) == 0
    indptr = np.zeros(3 * n_nodes + 1, np.int32)
    indices = np.zeros(9 * nb, np.int32)
    assert lib.cpfem_pattern_expand_csr(n_nodes, rp.ctypes.data, cols.ctypes.data, indptr.ctypes.data,
                                        indices.ctypes.data) == 0
    return rp, cols, epos, tpos, indptr, indices


def _scipy_pattern(cells, n_nodes):
    E = cells.shape[0]
    dof = (3 * cells[:, :, None] + np.arange(3)).reshape(E, 24)
    I = np.repeat(dof[:, :, None], 24, axis=2).ravel()
    J = np.repeat(dof[:, None, :], 24, axis=1).ravel()
    V = np.arange(I.size, dtype=np.float64) + 1.0
    A = sp.csr_array((V, (I, J)), shape=(3 * n_nodes, 3 * n_nodes))
    A.sum_duplicates()
    A.sort_indices()
    return A, I, J, V


@pytest.mark.parametrize("shape", [(1, 1, 1), (3, 2, 2), (4, 4, 4)])
def test_pattern_matches_scipy_coo_to_csr(lib, pkg, shape):
    m = pkg.box_mesh(*shape)
    n = m.points.shape[0]
    rp, cols, epos, tpos, indptr, indices = _pattern(lib, m.cells, n)
    A, I, J, V = _scipy_pattern(m.cells, n)
    assert np.array_equal(indptr, A.indptr) and np.array_equal(indices, A.indices)
    # scattering the COO values through elem_pos gives scipy's summed CSR values
    vals = np.zeros(9 * cols.size)
    E = m.cells.shape[0]
    Ke = V.reshape(E, 8, 3, 8, 3)
    for e in range(E):
        for a in range(8):
            na = m.cells[e, a]
            deg = rp[na + 1] - rp[na]
            for b in range(8):
                pos = epos[64 * e + 8 * a + b]
                for i in range(3):
                    for k in range(3):
                        vals[9 * rp[na] + i * 3 * deg + 3 * pos + k] += Ke[e, a, i, b, k]
    assert np.array_equal(vals, A.data)
    # transpose positions
    for a in range(n):
        for j in range(rp[a], rp[a + 1]):
            b = cols[j]
            assert cols[rp[b] + tpos[j]] == a


def test_pattern_on_permuted_irregular_numbering(lib, pkg):
    m = pkg.box_mesh(3, 3, 2)
    n = m.points.shape[0]
    perm = np.random.default_rng(0).permutation(n)
    cells = perm[m.cells]
    rp, cols, epos, tpos, indptr, indices = _pattern(lib, cells, n)
    A, *_ = _scipy_pattern(cells, n)
    assert np.array_equal(indptr, A.indptr) and np.array_equal(indices, A.indices)


def test_pattern_rejects_bad_node_index(lib):
    cells = np.arange(8, dtype=np.int32).reshape(1, 8)
    nb = np.zeros(1, np.int64)
    assert lib.cpfem_pattern_count(1, cells.ctypes.data, 7, nb.ctypes.data) != 0
    assert b"out of range" in lib.cpfem_last_error()


def test_material_struct_and_specs(pkg):
    m = pkg.material.BENCH_TANTALUM.to_ctypes()
    assert m.num_slip == 24 and m.qmode == 1 and m.C11 == 267.0e3
    d = np.array([[m.slip_d[a][i] for i in range(3)] for a in range(24)])
    nrm = np.array([[m.slip_n[a][i] for i in range(3)] for a in range(24)])
    assert np.allclose(np.linalg.norm(d, axis=1), 1) and np.abs((d * nrm).sum(1)).max() < 1e-15
    assert pkg.material.CALIB_CASE1.to_ctypes().qmode == 0


def test_bc_lists_later_entry_wins(pkg):
    import torch
    from importlib import import_module
    prob_mod = import_module("jax-cpfem_gb300.problem")
    fe = prob_mod.FiniteElement.__new__(prob_mod.FiniteElement)
    fe.device = torch.device("cpu")
    fe.set_dirichlet_lists([np.array([0, 1]), np.array([1, 2])], [2, 2], [0.0, 5.0])
    assert fe.bc_dofs.tolist() == [2, 5, 8] and fe.bc_vals.tolist() == [0.0, 5.0, 5.0]


def test_orthonormal_check_rejects_unnormalised_quaternion(pkg):
    R = pkg.material.rot_mat(np.array([[2.0, 0, 0, 0]]))
    with pytest.raises(ValueError):
        pkg.material.check_orthonormal(R)


def test_product_code_never_imports_the_oracle():
    pkg_dir = os.path.join(ROOT, "jax-cpfem_gb300")
    for dirpath, _, files in os.walk(pkg_dir):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".cpp")):
                src = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in src.replace("oracle/_ref", ""), f


def _sell(lib, rp, cols, tpos, n):
    slots = np.zeros(1, np.int64)
    assert lib.cpfem_sell_count(n, rp.ctypes.data, slots.ctypes.data) == 0
    S = int(slots[0])
    ng = (n + 31) // 32
    goff = np.zeros(ng + 1, np.int64)
    gw = np.zeros(ng, np.int32)
    sc = np.zeros(S, np.int32)
    st = np.zeros(S, np.int32)
    ds = np.zeros(n, np.int32)
    assert lib.cpfem_sell_build(n, rp.ctypes.data, cols.ctypes.data, tpos.ctypes.data, goff.ctypes.data,
                                gw.ctypes.data, sc.ctypes.data, st.ctypes.data, ds.ctypes.data) == 0
    m = np.zeros(9 * cols.size, np.int64)
    assert lib.cpfem_sell_csr_map(n, rp.ctypes.data, goff.ctypes.data, m.ctypes.data) == 0
    return goff, gw, sc, st, ds, m


@pytest.mark.parametrize("shape", [(2, 2, 2), (5, 4, 3)])
def test_sell_layout_reproduces_csr_products(lib, pkg, shape):
    """The sliced-ELL indexing the kernels use, replayed in numpy: A x, A^T x, the
    diagonal blocks and a Dirichlet row all agree with scipy on the scalar CSR."""
    m = pkg.box_mesh(*shape)
    n = m.points.shape[0]
    rp, cols, epos, tpos, indptr, indices = _pattern(lib, m.cells, n)
    goff, gw, sc, st, ds, cmap = _sell(lib, rp, cols, tpos, n)
    rng = np.random.default_rng(1)
    data = rng.normal(size=indices.size)
    A = sp.csr_array((data, indices, indptr), shape=(3 * n, 3 * n))
    vals = np.zeros(9 * goff[-1])
    vals[cmap] = data
    assert np.unique(cmap).size == cmap.size
    x = rng.normal(size=3 * n)
    y, yt = np.zeros(3 * n), np.zeros(3 * n)
    for a in range(n):
        g, lane = a >> 5, a & 31
        for j in range(gw[g]):
            b = sc[goff[g] + 32 * j + lane]
            for i in range(3):
                for k in range(3):
                    y[3 * a + i] += vals[9 * goff[g] + 32 * (9 * j + 3 * i + k) + lane] * x[3 * b + k]
                    tp = st[goff[g] + 32 * j + lane]
                    yt[3 * a + i] += vals[9 * goff[b >> 5] + 32 * (9 * tp + 3 * k + i) + (b & 31)] * x[3 * b + k]
        for i in range(3):
            assert vals[9 * goff[g] + 32 * (9 * ds[a] + 4 * i) + lane] == A[3 * a + i, 3 * a + i]
    assert np.allclose(y, A @ x, rtol=1e-13, atol=1e-12)
    assert np.allclose(yt, A.T @ x, rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("shape", [(4, 3, 2), (6, 6, 6)])
def test_cell_colouring_is_conflict_free(lib, pkg, shape):
    m = pkg.box_mesh(*shape)
    cells = np.ascontiguousarray(m.cells, dtype=np.int32)
    color = np.zeros(cells.shape[0], np.int32)
    nc = np.zeros(1, np.int32)
    assert lib.cpfem_color_cells(cells.shape[0], cells.ctypes.data, m.points.shape[0], color.ctypes.data,
                                 nc.ctypes.data) == 0
    assert nc[0] == 8
    for c in range(nc[0]):
        nodes = cells[color == c].ravel()
        assert np.unique(nodes).size == nodes.size


def test_multiphase_spec_and_golden_dp_fixture(pkg):
    """The dual-phase spec mirrors models_DPsteel_inhomo.py (BCC24, coplanar 3-block q,
    10 internal variables), cubic C round-trips, and the DP golden fixture is coherent."""
    m = pkg.material
    spec = m.DP_STEEL
    assert spec.num_internal_vars == 10 and spec.num_slip == 24 and spec.to_ctypes().qmode == 1
    assert [p.gss_initial for p in spec.phases] == [170.0, 435.0]
    rows = np.stack([p.elastic_row() for p in spec.phases])
    np.testing.assert_array_equal(m.cubic_constants(m.cubic_tensor(rows)), rows)
    bad = m.cubic_tensor(rows)
    bad[0, 0, 1, 0, 2] = 1.0
    with pytest.raises(ValueError):
        m.cubic_constants(bad)
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "golden.npz"))
    assert np.bincount(g["dp_phase"]).tolist() == [600, 400]     # phase of the Kalidindi parameters
    assert (g["dp_stiff_phase"] == 1 - g["dp_phase"]).all()     # the stiffness the files were made with
    assert g["dp_ori"].max() >= g["dp_quat"].shape[0]          # clamped indices occur
    assert np.abs(np.linalg.norm(g["dp_quat"], axis=1) - 1).max() < 1e-12
    assert g["dp_sig"].shape == (50, 3, 1000)


def _fake_hierarchy(capi):
    """A two-level cpfem_mg_t whose pointers are non-null placeholders: enough for the
    argument checks, which run before any device access."""
    import ctypes
    mg = capi.MGHierarchy()
    mg.num_levels, mg.pre_sweeps, mg.post_sweeps, mg.coarse_sweeps, mg.omega = 2, 1, 1, 4, 0.45
    fake = 4096
    for l, d in enumerate((3, 2)):
        for k in range(3):
            mg.dims[l][k] = d
        s = mg.sell[l]
        s.num_nodes, s.num_groups = d ** 3, (d ** 3 + 31) // 32
        s.group_off = s.group_width = s.cols = s.tpos = s.diag_slot = fake
        mg.values[l] = mg.minv[l] = mg.slot[l] = mg.x[l] = mg.t[l] = mg.r[l] = mg.b[l] = fake
    mg.scratch[0] = mg.scratch[1] = fake
    mg.scratch_nodes = 1 << 20
    return mg


@pytest.mark.parametrize("field,value,message", [("precision", 7, "precision"), ("local_nodes", -1, "local_nodes"),
                                                 ("omega", 2.5, "omega")])
def test_multigrid_argument_checks(lib, field, value, message):
    import ctypes
    from importlib import import_module
    capi = import_module("jax-cpfem_gb300._capi")
    mg = _fake_hierarchy(capi)
    setattr(mg, field, value)
    rc = lib.cpfem_mg_setup(ctypes.byref(mg), ctypes.c_void_p(4096), None)
    assert rc == 1 and message in lib.cpfem_last_error().decode()


def test_fp32_multigrid_needs_its_arrays(lib):
    """precision = 1 without the FP32 copies is an argument error, not a device fault."""
    import ctypes
    from importlib import import_module
    capi = import_module("jax-cpfem_gb300._capi")
    mg = _fake_hierarchy(capi)
    mg.precision = 1
    rc = lib.cpfem_mg_setup(ctypes.byref(mg), ctypes.c_void_p(4096), None)
    assert rc == 1 and "arrays missing" in lib.cpfem_last_error().decode()
