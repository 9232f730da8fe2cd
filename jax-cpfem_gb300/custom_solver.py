"""The GPU BiCGSTAB behind JAX-FEM's ``custom_solver`` hook.

JAX-FEM's ``linear_solver`` hands the Newton system to a user function when the solver
options carry one (``crystal_plasticity_OR_design/solver.py:106-109``)::

    sol_list = solver(problem, {"custom_solver": GpuBicgstab(), "initial_guess": sol_list})

``GpuBicgstab`` is that function for a driver that keeps the reference's own JAX-FEM
problem on the host: it takes the host CSR matrix JAX-FEM assembled (a PETSc AIJ matrix
read with ``getValuesCSR()`` as ``jax_solve`` reads it, ``solver.py:26-31``, or any scipy
CSR matrix), finds its 3x3 node-block pattern (HEX8, 3 dofs per node), lays the values
out for the library once per pattern, and runs ``cpfem_bicgstab`` on the device with the
reference's settings (Jacobi, tol = atol = 1e-10, maxiter 10000) and its
``||Ax - b|| < 0.1`` check (``solver.py:43-46``).  The pattern and the device buffers are
kept while the matrix pattern does not change, so a Newton iteration costs one host-to-
device copy of the values, b and x0, the solve, and the copy of x back.

With this package's own ``CrystalPlasticity`` the tangent never leaves the device and the
``jax_solver`` path is the faster one; the hook is for host codes that keep their own
assembly.
"""
from __future__ import annotations

import numpy as np
import torch

from . import _capi


def _host_csr(A):
    """(indptr, indices, data) of a PETSc AIJ matrix, a scipy sparse matrix, or any object
    with ``getValuesCSR()``."""
    if hasattr(A, "getValuesCSR"):
        indptr, indices, data = A.getValuesCSR()
    else:
        A = A.tocsr()
        indptr, indices, data = A.indptr, A.indices, A.data
    return (np.ascontiguousarray(indptr, dtype=np.int64), np.ascontiguousarray(indices, dtype=np.int64),
            np.ascontiguousarray(data, dtype=np.float64))


def node_block_pattern(indptr, indices):
    """Node-block pattern (rowptr, cols) of a scalar CSR pattern with 3 dofs per node,
    each node-row's three rows holding the same column blocks {3b, 3b+1, 3b+2}; raises
    ValueError for any other pattern."""
    n = indptr.size - 1
    if n % 3:
        raise ValueError("the matrix size is not a multiple of 3 (3 dofs per node)")
    nn = n // 3
    lens = np.diff(indptr)
    if np.any(lens % 3) or np.any(lens[0::3] != lens[1::3]) or np.any(lens[0::3] != lens[2::3]):
        raise ValueError("the rows of a node do not share one 3x3 block pattern")
    first = indptr[0:-1:3]
    nb = lens[0::3] // 3
    rowptr = np.concatenate([[0], np.cumsum(nb)]).astype(np.int64)
    # the block columns: every third entry of the node's first row
    sel = np.repeat(first, nb) + 3 * (np.arange(int(rowptr[-1])) - np.repeat(rowptr[:-1], nb))
    cols = indices[sel] // 3
    expand = (3 * cols[:, None] + np.arange(3)[None, :]).reshape(-1)
    node_of = np.repeat(np.arange(nn), nb)
    for i in range(3):
        row_cols = indices[(np.repeat(indptr[i:-1:3], 3 * nb) +
                            np.arange(3 * int(rowptr[-1])) - np.repeat(3 * rowptr[:-1], 3 * nb))]
        if not np.array_equal(row_cols, expand):
            raise ValueError("the rows of a node do not share one 3x3 block pattern")
    key = node_of * nn + cols
    if np.any(np.diff(key) <= 0):
        raise ValueError("column indices must be sorted and unique within each row")
    return rowptr.astype(np.int32), cols.astype(np.int32), node_of


class GpuBicgstab:
    """``custom_solver(A, b, x0, solver_options)`` running the library's persistent
    BiCGSTAB on the GPU.  Returns x as the type b came in (a torch tensor for torch input,
    else a numpy array)."""

    def __init__(self, precond=1, tol=1e-10, atol=1e-10, maxiter=10000, device="cuda"):
        self.lib = _capi.load()
        self.precond, self.tol, self.atol, self.maxiter = int(precond), float(tol), float(atol), int(maxiter)
        self.device = torch.device(device)
        self._key = None
        self.last_iterations = None

    def _layout(self, indptr, indices):
        if self._key is not None and np.array_equal(self._key[0], indptr) and np.array_equal(self._key[1], indices):
            return
        lib, dev = self.lib, self.device
        rowptr, cols, node_of = node_block_pattern(indptr, indices)
        nn = rowptr.size - 1
        # position of node a in the list of its neighbour b (the transposed product)
        keys = node_of.astype(np.int64) * nn + cols
        tpos = (np.searchsorted(keys, cols.astype(np.int64) * nn + node_of) - rowptr[cols]).astype(np.int32)
        slots = np.zeros(1, dtype=np.int64)
        _capi.check(lib.cpfem_sell_count(nn, rowptr.ctypes.data, slots.ctypes.data))
        ng = (nn + 31) // 32
        goff = np.zeros(ng + 1, dtype=np.int64)
        gw = np.zeros(ng, dtype=np.int32)
        scols = np.zeros(int(slots[0]), dtype=np.int32)
        stpos = np.zeros(int(slots[0]), dtype=np.int32)
        dslot = np.zeros(nn, dtype=np.int32)
        _capi.check(lib.cpfem_sell_build(nn, rowptr.ctypes.data, cols.ctypes.data, tpos.ctypes.data,
                                         goff.ctypes.data, gw.ctypes.data, scols.ctypes.data, stpos.ctypes.data,
                                         dslot.ctypes.data))
        cmap = np.zeros(9 * int(rowptr[-1]), dtype=np.int64)
        _capi.check(lib.cpfem_sell_csr_map(nn, rowptr.ctypes.data, goff.ctypes.data, cmap.ctypes.data))
        self._arrays = [torch.tensor(a, device=dev) for a in (goff, gw, scols, stpos, dslot)]
        self.sell = _capi.Sell(nn, ng, *(a.data_ptr() for a in self._arrays))
        self._map = torch.tensor(cmap, device=dev)
        self._values = torch.zeros(9 * int(slots[0]), dtype=torch.float64, device=dev)
        nbytes = int(lib.cpfem_bicgstab_workspace_bytes(nn))
        self._ws = torch.empty(nbytes // 8 + 64, dtype=torch.float64, device=dev)
        self._key = (indptr.copy(), indices.copy())

    def __call__(self, A, b, x0, solver_options=None):
        indptr, indices, data = _host_csr(A)
        self._layout(indptr, indices)
        dev = self.device
        as_torch = isinstance(b, torch.Tensor)
        self._values[self._map] = torch.as_tensor(data, device=dev)
        bd = torch.as_tensor(np.asarray(b) if not as_torch else b, dtype=torch.float64, device=dev).reshape(-1)
        bd = bd.contiguous()
        x = torch.as_tensor(np.asarray(x0) if not isinstance(x0, torch.Tensor) else x0, dtype=torch.float64,
                            device=dev).reshape(-1).clone()
        info = np.zeros(2, dtype=np.int32)
        stream = torch.cuda.current_stream(dev).cuda_stream
        _capi.check(self.lib.cpfem_bicgstab(self.sell, self._values.data_ptr(), bd.data_ptr(), x.data_ptr(),
                                            self.precond, 0, self.tol, self.atol, self.maxiter, self._ws.data_ptr(),
                                            info.ctypes.data, stream))
        self.last_iterations = int(info[0])
        r = torch.empty_like(x)
        _capi.check(self.lib.cpfem_spmv(self.sell, self._values.data_ptr(), x.data_ptr(), r.data_ptr(), 0, stream))
        err = float((r - bd).norm())
        if not err < 0.1:
            raise RuntimeError(f"linear solver failed to converge with err = {err} (iterations {info[0]})")
        return x if as_torch else x.cpu().numpy()


gpu_bicgstab = GpuBicgstab
