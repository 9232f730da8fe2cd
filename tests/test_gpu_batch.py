"""Ragged batch of RVEs (one launch per Newton stage, per-instance Krylov scalars and
convergence) against the same RVEs solved one at a time."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_matches_serial(pkg, gpu):
    batch = importlib.import_module("jax-cpfem_gb300.batch")
    base = pkg.material.BENCH_STEEL
    inst = batch.sample_instances(4, base, seed=3, edges=(2, 3, 4), grains=(2, 5))
    b = batch.Batch(inst)
    disps = [1e-3, 2e-3, 3e-3]
    szz = np.stack([b.step(d, 0.1).cpu().numpy() for d in disps], axis=1)
    ref = batch.run_serial(inst, disps, 0.1)
    rel = np.abs(szz - ref) / np.abs(ref)
    assert rel.max() < 1e-8, rel
    # instances converge independently
    assert len(b.stats["newton_iters"]) == 3


def test_batch_against_oracle(pkg, gpu):
    """The batch with the benchmark path's settings (extrapolated Newton guess, FP32
    consistent tangent, Newton limit 1e-8) against the compiled oracle converged far below
    that limit, instance by instance: per-step mean sigma_zz and the final displacements
    to 1e-8 of their magnitudes.  Instances of different sizes, grain maps and Kalidindi
    parameters (each parameter scaled by U(0.8, 1.2))."""
    import os
    import types
    from oracle import coracle
    from tests.common import fast_oracle_problem, oracle_history
    batch = importlib.import_module("jax-cpfem_gb300.batch")
    W = importlib.import_module("jax-cpfem_gb300.workloads")
    inst = batch.sample_instances(3, pkg.material.BENCH_STEEL, seed=11, edges=(4, 6, 8), grains=(3, 8))
    b = batch.Batch(inst)
    b.predictor = "linear"
    b.problem.fp32_tangent = True
    steps = 3
    disps = [1e-3 * (i + 1) for i in range(steps)]
    szz = np.stack([b.step(d, 0.1, tol=1e-8, rel_tol=1e-8).cpu().numpy() for d in disps], axis=1)
    sol = b.sol.cpu().numpy()
    coracle.set_threads(os.cpu_count() or 1)
    for k, it in enumerate(inst):
        mesh, quat, ori = b.meshes[k]
        orc = fast_oracle_problem(it.material, mesh, quat, ori)
        w = types.SimpleNamespace(dt=0.1, strain_step=1e-3,
                                  bc_triples=lambda d, m=mesh: list(zip(*W.roller_lists(m, d))))
        sig_o, us_o, _, _ = oracle_history(orc, w, steps, {"tol": 1e-9, "rel_tol": 1e-12})
        err_s = np.abs(szz[k] - sig_o[:, 2, 2]).max() / np.abs(sig_o[:, 2, 2]).max()
        u = sol[3 * b.node_off_np[k]:3 * b.node_off_np[k + 1]]
        err_u = np.abs(u - us_o[-1]).max() / np.abs(us_o[-1]).max()
        assert err_s < 1e-8 and err_u < 1e-8, (k, it.edge, err_s, err_u)
