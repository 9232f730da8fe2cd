"""BiCGSTAB breakdown semantics and the restart option, and the ragged batched solver with
multi-block teams, on the GPU through the C ABI."""
import ctypes
import importlib

import numpy as np
import pytest
import torch

from oracle import cpfem_oracle as O

pytestmark = pytest.mark.gpu


def _one_node_system(lib, capi, A):
    """A single node's 3x3 block as a sliced-ELL system (one group, one slot)."""
    rowptr = np.array([0, 1], dtype=np.int32)
    cols = np.array([0], dtype=np.int32)
    tpos = np.array([0], dtype=np.int32)
    slots = np.zeros(1, dtype=np.int64)
    capi.check(lib.cpfem_sell_count(1, rowptr.ctypes.data, slots.ctypes.data))
    goff = np.zeros(2, dtype=np.int64)
    gw = np.zeros(1, dtype=np.int32)
    scols = np.zeros(int(slots[0]), dtype=np.int32)
    stpos = np.zeros(int(slots[0]), dtype=np.int32)
    dslot = np.zeros(1, dtype=np.int32)
    capi.check(lib.cpfem_sell_build(1, rowptr.ctypes.data, cols.ctypes.data, tpos.ctypes.data, goff.ctypes.data,
                                    gw.ctypes.data, scols.ctypes.data, stpos.ctypes.data, dslot.ctypes.data))
    arrays = [torch.tensor(v, device="cuda") for v in (goff, gw, scols, stpos, dslot)]
    sell = capi.Sell(1, 1, *(a.data_ptr() for a in arrays))
    # value of (row 3*0+i, col 3*0+k) of slot 0 lives at 32*(3i+k) (lane 0)
    vals = np.zeros(9 * 32 * int(slots[0]))
    for i in range(3):
        for k in range(3):
            vals[32 * (3 * i + k)] = A[i, k]
    return sell, arrays, torch.tensor(vals, device="cuda")


def _solve(lib, capi, sell, vals, b, restarts):
    x = torch.zeros(3, dtype=torch.float64, device="cuda")
    bd = torch.tensor(b, device="cuda")
    ws = torch.zeros(int(lib.cpfem_bicgstab_workspace_bytes(1)) // 8 + 64, dtype=torch.float64, device="cuda")
    info = np.zeros(2, dtype=np.int32)
    opts = capi.KrylovOpts(0, 0, 100, restarts, 1e-10, 1e-10)
    capi.check(lib.cpfem_bicgstab_ex(ctypes.byref(sell), vals.data_ptr(), bd.data_ptr(), x.data_ptr(),
                                     ctypes.byref(opts), ws.data_ptr(), info.ctypes.data,
                                     torch.cuda.current_stream().cuda_stream))
    stats = np.zeros(7)
    capi.check(lib.cpfem_bicgstab_last_stats(stats.ctypes.data))
    return x.cpu().numpy(), info, stats


def test_breakdown_matches_jax_and_restart_converges(pkg, gpu):
    capi = importlib.import_module("jax-cpfem_gb300._capi")
    lib = capi.load()
    # a12 a21 + a13 a31 = 0 makes the first recursive residual orthogonal to rhat = b:
    # rho = 0 exactly at the second iteration (jax returns code -10 there)
    A = np.array([[2.0, 1.0, 1.0], [1.0, 3.0, 0.5], [-1.0, 0.25, 4.0]])
    b = np.array([1.0, 0.0, 0.0])
    x_o, k_o = O.bicgstab(A, b, np.zeros(3), lambda v: v)
    assert k_o == -10
    sell, keep, vals = _one_node_system(lib, capi, A)
    x, info, stats = _solve(lib, capi, sell, vals, b, restarts=0)
    assert info[0] == -10 and info[1] == 0
    np.testing.assert_allclose(x, x_o, rtol=1e-13, atol=1e-15)
    assert stats[0] == -10 and stats[3] == 0.0 and stats[6] == 0
    x, info, stats = _solve(lib, capi, sell, vals, b, restarts=5)
    assert info[1] == 1 and info[0] > 0 and stats[6] >= 1
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-9)


def test_ragged_batch_with_multi_block_teams(pkg, gpu):
    """Instances of 343..1331 nodes get teams of several blocks (team barriers and
    team-ordered reductions); results match the instances solved one at a time."""
    batch = importlib.import_module("jax-cpfem_gb300.batch")
    inst = batch.sample_instances(3, pkg.material.BENCH_STEEL, seed=5, edges=(6, 8, 10), grains=(3, 6))
    b = batch.Batch(inst)
    disps = [1e-3, 2e-3]
    szz = np.stack([b.step(d, 0.1).cpu().numpy() for d in disps], axis=1)
    ref = batch.run_serial(inst, disps, 0.1)
    assert np.abs(szz - ref).max() / np.abs(ref).max() < 1e-8
    assert max(int(k.max()) for k in b.stats["krylov_iters"]) > 10
