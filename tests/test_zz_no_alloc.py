"""The allocation-free BiCGSTAB entry point against the workspace one.

cpfem_bicgstab_noalloc exists for callers that cannot allocate device memory -- a host
code that owns every device byte through its own pool, or a loop that must not allocate --
and keeps its scratch in a fixed array inside the library.  This file is collected last
so that a failure here does not stop the rest of the suite; it must pass both alone in a
fresh process and after the other tests.
"""
import ctypes
import importlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precond", [1, 2])
def test_noalloc_bicgstab_matches_workspace_solver_twice(pkg, gpu, precond):
    """Jacobi (1) and 3x3 block-Jacobi (2): both carve their preconditioner out of the
    fixed scratch."""
    problem_mod, solver_mod = gpu
    capi = importlib.import_module("jax-cpfem_gb300._capi")
    lib = capi.load()
    spec = pkg.material.BENCH_STEEL
    mesh = pkg.box_mesh(6, 5, 4)
    ori, rng = pkg.mesh.voronoi_grains(mesh, 5, 2)
    quat = pkg.material.random_quaternions(rng, 5)
    prob = problem_mod.CrystalPlasticity(mesh, additional_info=(quat, ori), material=spec)
    p = mesh.points
    fn = pkg.mesh.face_nodes
    prob.fes[0].set_dirichlet_lists([fn(p, 0, 0.0), fn(p, 1, 0.0), fn(p, 2, 0.0), fn(p, 2, 1.0)], [0, 1, 2, 2],
                                    [0.0, 0.0, 0.0, 1e-3])
    prob.dt = 0.1
    u = torch.zeros(prob.num_total_dofs_all_vars, dtype=torch.float64, device="cuda")
    res, A = solver_mod.newton_update_helper(prob, u)
    b = torch.neg(res)
    x0 = solver_mod.initial_increment(prob, u).clone()
    x_ref, k_ref, ok_ref = solver_mod.bicgstab(prob, A, b, x0, precond=precond)
    assert ok_ref and k_ref > 0
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        x = x0.clone()
        info = np.zeros(2, dtype=np.int32)
        rc = lib.cpfem_bicgstab_noalloc(prob.sell, A.values.data_ptr(), b.data_ptr(), x.data_ptr(), precond, 0,
                                        1e-10, 1e-10, 10000, info.ctypes.data, stream)
        capi.check(rc)
        assert info[1] == 1 and info[0] == k_ref, (call, info, k_ref)
        rel = float((x - x_ref).abs().max() / x_ref.abs().max())
        assert rel < 1e-12, (call, rel)


def test_noalloc_rejects_sizes_beyond_its_scratch(pkg, gpu):
    capi = importlib.import_module("jax-cpfem_gb300._capi")
    lib = capi.load()
    big = capi.Sell(65537, (65537 + 31) // 32, 1, 1, 1, 1, 1)   # never dereferenced: rejected first
    info = np.zeros(2, dtype=np.int32)
    rc = lib.cpfem_bicgstab_noalloc(big, 1, 1, 1, 1, 0, 1e-10, 1e-10, 10, info.ctypes.data, None)
    assert rc == 3
    assert b"exceed the fixed scratch" in lib.cpfem_last_error()
