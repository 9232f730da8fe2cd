"""Host logic that needs no GPU: the Newton loop's last-iterate prediction and the
autotuner's coordinate search (with a stand-in for the timed solve)."""
import importlib

import numpy as np
import pytest


@pytest.fixture(scope="module")
def solver_mod(pkg):
    return importlib.import_module("jax-cpfem_gb300.solver")


@pytest.fixture(scope="module")
def tuning(pkg):
    return importlib.import_module("jax-cpfem_gb300.tuning")


def test_last_iterate_prediction(solver_mod):
    f = solver_mod._expect_converged
    assert not f([1.0], 1e-6)                      # no rate yet
    assert not f([1.0, 2.0], 1e-6)                 # not contracting
    assert f([1.0, 1e-3], 1e-6)                    # predicted 1e-9, well below the limit
    assert not f([1.0, 1e-2], 1e-6)                # predicted 1e-6: not below a quarter of it
    assert f([5.0, 1e-1, 1e-4], 1e-6) and not f([5.0, 1e-1, 2e-2], 1e-6)


def test_tuner_coordinate_search_keeps_the_fastest_converging(tuning, monkeypatch):
    """Each setting is tried in turn from the best so far; a faster configuration that does
    not converge, or one the library rejects, is never chosen."""
    cost = {"precision": {"fp64": 10.0, "fp32": 6.0}, "omega": {0.35: 1.0, 0.4: 0.5, 0.45: 0.0},
            "coarse_sweeps": {4: 0.2, 8: 0.0, 12: 0.7}, "grid_blocks": {0: 0.0, 152: -0.5, 304: -2.0}}
    seen = []

    def fake_time(problem, A, b, x0, cfg, reps, tol=1e-10):
        seen.append(dict(cfg))
        if cfg["grid_blocks"] == 76:
            raise RuntimeError("rejected")
        ms = sum(cost[k][cfg[k]] for k in cost if cfg[k] in cost[k])
        converged = cfg["grid_blocks"] != 304            # the fastest one does not converge
        return ms, 20, converged

    class FakeProblem:
        def multigrid(self, **kw):
            self.kw = kw

    monkeypatch.setattr(tuning, "_time_solve", fake_time)
    prob = FakeProblem()
    search = (("precision", ("fp64", "fp32")), ("omega", (0.35, 0.4, 0.45)), ("coarse_sweeps", (4, 8, 12)),
              ("grid_blocks", (0, 76, 152, 304)))
    cfg, table = tuning.tune_linear_solver(prob, None, None, None, search=search)
    assert cfg["precision"] == "fp32" and cfg["omega"] == 0.45 and cfg["coarse_sweeps"] == 8
    assert cfg["grid_blocks"] == 152
    assert all(t[0]["grid_blocks"] != 76 for t in table)      # the rejected one is left out
    assert prob.kw == {k: cfg[k] for k in tuning.MG_KEYS}      # the hierarchy ends in the choice


def test_custom_solver_node_block_pattern(pkg):
    """The custom_solver binding recovers the node-block pattern of a HEX8 scalar CSR matrix
    (scipy's COO->CSR of the element triplets) and refuses other patterns."""
    import importlib
    import scipy.sparse as sp
    cs = importlib.import_module("jax-cpfem_gb300.custom_solver")
    mesh = pkg.box_mesh(3, 2, 2)
    E = mesh.cells.shape[0]
    dof = (3 * mesh.cells[:, :, None] + np.arange(3)).reshape(E, 24)
    I = np.repeat(dof[:, :, None], 24, axis=2).ravel()
    J = np.repeat(dof[:, None, :], 24, axis=1).ravel()
    A = sp.csr_array((np.ones(I.size), (I, J)))
    A.sum_duplicates()
    A.sort_indices()
    rowptr, cols, node_of = cs.node_block_pattern(A.indptr.astype(np.int64), A.indices.astype(np.int64))
    n = mesh.points.shape[0]
    B = sp.csr_array((np.ones(cols.size), cols, rowptr), shape=(n, n))
    assert (sp.kron(B, np.ones((3, 3))).tocsr() != A.astype(bool)).nnz == 0
    with pytest.raises(ValueError):
        R = sp.random(9, 9, density=0.5, format="csr", random_state=0) + sp.eye(9)
        cs.node_block_pattern(R.indptr.astype(np.int64), R.indices.astype(np.int64))
