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
