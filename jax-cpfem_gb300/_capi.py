"""ctypes binding of ``libcpfem_gb300.so`` (declared in ``include/cpfem_gb300.h``).

The library must exist: there is no CPU fallback.  ``load()`` raises ``ImportError`` with
the build command when the shared object is missing.
"""
from __future__ import annotations

import ctypes
import os

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libcpfem_gb300.so")

MAX_SLIP = 24

CPFEM_GP_MAXITER = 1
CPFEM_GP_NONFINITE = 2
CPFEM_GP_BOUNDS = 4


class CPFEMError(RuntimeError):
    """A C-ABI call returned a non-zero status."""


class Material(ctypes.Structure):
    _fields_ = [
        ("num_slip", ctypes.c_int32),
        ("qmode", ctypes.c_int32),
        ("max_sub_step", ctypes.c_int32),
        ("max_iter", ctypes.c_int32),
        ("local_tol", ctypes.c_double),
        ("ao", ctypes.c_double),
        ("C11", ctypes.c_double),
        ("C12", ctypes.c_double),
        ("C44", ctypes.c_double),
        ("slip_d", (ctypes.c_double * 3) * MAX_SLIP),
        ("slip_n", (ctypes.c_double * 3) * MAX_SLIP),
    ]


class GPArgs(ctypes.Structure):
    _fields_ = [
        ("num_gp", ctypes.c_int64),
        ("num_cells", ctypes.c_int32),
        ("weight_jxw", ctypes.c_int32),
        ("dt", ctypes.c_double),
        ("u", ctypes.c_void_p),
        ("cells", ctypes.c_void_p),
        ("shape_grads", ctypes.c_void_p),
        ("jxw", ctypes.c_void_p),
        ("u_grad", ctypes.c_void_p),
        ("fpi", ctypes.c_void_p),
        ("g", ctypes.c_void_p),
        ("slip", ctypes.c_void_p),
        ("rot_table", ctypes.c_void_p),
        ("rot_idx", ctypes.c_void_p),
        ("param_table", ctypes.c_void_p),
        ("param_idx", ctypes.c_void_p),
        ("elastic_table", ctypes.c_void_p),
        ("pk1", ctypes.c_void_p),
        ("tangent", ctypes.c_void_p),
        ("stress", ctypes.c_void_p),
        ("fpi_new", ctypes.c_void_p),
        ("g_new", ctypes.c_void_p),
        ("slip_new", ctypes.c_void_p),
        ("s_out", ctypes.c_void_p),
        ("iters", ctypes.c_void_p),
        ("status", ctypes.c_void_p),
        ("cell_list", ctypes.c_void_p),
        ("num_listed", ctypes.c_int32),
        ("local_flags", ctypes.c_int32),
        ("order", ctypes.c_void_p),
        ("s_warm", ctypes.c_void_p),
        ("s_dsdf", ctypes.c_void_p),
        ("s_f", ctypes.c_void_p),
        ("tangent32", ctypes.c_void_p),
    ]


class VjpArgs(ctypes.Structure):
    _fields_ = [
        ("num_gp", ctypes.c_int64),
        ("num_cells", ctypes.c_int32),
        ("mode", ctypes.c_int32),
        ("dt", ctypes.c_double),
        ("num_nodes", ctypes.c_int32),
        ("num_rot", ctypes.c_int32),
        ("num_param", ctypes.c_int32),
        ("pad", ctypes.c_int32),
    ] + [(name, ctypes.c_void_p) for name in (
        "u", "cells", "shape_grads", "jxw", "fpi", "g", "rot_table", "rot_idx", "param_table", "param_idx",
        "elastic_table", "cell_sig_bar", "fpi_bar", "g_bar", "mu", "f_bar", "fpi_bar_old", "g_bar_old", "theta_bar", "rot_bar",
        "status", "s_start")]


class Sell(ctypes.Structure):
    _fields_ = [
        ("num_nodes", ctypes.c_int32),
        ("num_groups", ctypes.c_int32),
        ("group_off", ctypes.c_void_p),
        ("group_width", ctypes.c_void_p),
        ("cols", ctypes.c_void_p),
        ("tpos", ctypes.c_void_p),
        ("diag_slot", ctypes.c_void_p),
    ]


MG_MAX_LEVELS = 8


class MGHierarchy(ctypes.Structure):
    """cpfem_mg_t."""
    _fields_ = [
        ("num_levels", ctypes.c_int32),
        ("pre_sweeps", ctypes.c_int32),
        ("post_sweeps", ctypes.c_int32),
        ("coarse_sweeps", ctypes.c_int32),
        ("omega", ctypes.c_double),
        ("dims", (ctypes.c_int32 * 3) * MG_MAX_LEVELS),
        ("sell", Sell * MG_MAX_LEVELS),
        ("values", ctypes.c_void_p * MG_MAX_LEVELS),
        ("minv", ctypes.c_void_p * MG_MAX_LEVELS),
        ("slot", ctypes.c_void_p * MG_MAX_LEVELS),
        ("x", ctypes.c_void_p * MG_MAX_LEVELS),
        ("t", ctypes.c_void_p * MG_MAX_LEVELS),
        ("r", ctypes.c_void_p * MG_MAX_LEVELS),
        ("b", ctypes.c_void_p * MG_MAX_LEVELS),
        ("free_dof", ctypes.c_void_p),
        ("scratch", ctypes.c_void_p * 2),
        ("scratch_nodes", ctypes.c_int64),
        ("precision", ctypes.c_int32),
        ("local_nodes", ctypes.c_int32),
        ("values32", ctypes.c_void_p * MG_MAX_LEVELS),
        ("minv32", ctypes.c_void_p * MG_MAX_LEVELS),
        ("x32", ctypes.c_void_p * MG_MAX_LEVELS),
        ("t32", ctypes.c_void_p * MG_MAX_LEVELS),
        ("r32", ctypes.c_void_p * MG_MAX_LEVELS),
        ("b32", ctypes.c_void_p * MG_MAX_LEVELS),
    ]


class SolveReport(ctypes.Structure):
    _fields_ = [
        ("k", ctypes.c_int32),
        ("error", ctypes.c_int32),
        ("rs", ctypes.c_double),
        ("atol2", ctypes.c_double),
        ("rho", ctypes.c_double),
        ("alpha", ctypes.c_double),
        ("omega", ctypes.c_double),
        ("restarts", ctypes.c_int32),
        ("pad", ctypes.c_int32),
        ("true_rs", ctypes.c_double),
        ("bb", ctypes.c_double),
    ]


class KrylovOpts(ctypes.Structure):
    _fields_ = [
        ("precond", ctypes.c_int32),
        ("transpose", ctypes.c_int32),
        ("maxiter", ctypes.c_int32),
        ("max_restarts", ctypes.c_int32),
        ("tol", ctypes.c_double),
        ("atol", ctypes.c_double),
        ("mg", ctypes.POINTER(MGHierarchy)),
        ("grid_blocks", ctypes.c_int32),
        ("flags", ctypes.c_int32),
        ("report", ctypes.c_void_p),
    ]


_P = ctypes.c_void_p
_I32 = ctypes.c_int32
_I64 = ctypes.c_int64
_D = ctypes.c_double

_SP = ctypes.POINTER(Sell)

# name -> (restype, argtypes); every symbol declared in include/cpfem_gb300.h
SIGNATURES = {
    "cpfem_abi_version": (ctypes.c_int, []),
    "cpfem_last_error": (ctypes.c_char_p, []),
    "cpfem_pattern_count": (ctypes.c_int, [_I32, _P, _I32, _P]),
    "cpfem_pattern_build": (ctypes.c_int, [_I32, _P, _I32, _P, _P, _P, _P]),
    "cpfem_pattern_expand_csr": (ctypes.c_int, [_I32, _P, _P, _P, _P]),
    "cpfem_sell_count": (ctypes.c_int, [_I32, _P, _P]),
    "cpfem_sell_build": (ctypes.c_int, [_I32, _P, _P, _P, _P, _P, _P, _P, _P]),
    "cpfem_sell_csr_map": (ctypes.c_int, [_I32, _P, _P, _P]),
    "cpfem_gp_eval": (ctypes.c_int, [ctypes.POINTER(Material), ctypes.POINTER(GPArgs), _P]),
    "cpfem_gp_vjp": (ctypes.c_int, [ctypes.POINTER(Material), ctypes.POINTER(VjpArgs), _P]),
    "cpfem_elem_assemble": (ctypes.c_int, [_I32, _P, _P, _SP, _P, _P, _I32, _P, _P, _P, _P, _P]),
    "cpfem_elem_assemble_ex": (ctypes.c_int, [_I32, _P, _P, _SP, _P, _P, _I32, _P, _P, _P, _P, _I32, _P]),
    "cpfem_color_cells": (ctypes.c_int, [_I32, _P, _I32, _P, _P]),
    "cpfem_apply_dirichlet": (ctypes.c_int, [_I32, _P, _P, _P, _P, _SP, _P, _P]),
    "cpfem_bc_initial_guess": (ctypes.c_int, [_I64, _I32, _P, _P, _P, _P, _P]),
    "cpfem_cell_average": (ctypes.c_int, [_I32, _P, _P, _P, _P]),
    "cpfem_axpy": (ctypes.c_int, [_I64, _D, _P, _P, _P]),
    "cpfem_segmented_dot": (ctypes.c_int, [_I32, _P, _P, _P, _P, _P]),
    "cpfem_dot_workspace_bytes": (ctypes.c_size_t, [_I64]),
    "cpfem_dot": (ctypes.c_int, [_I64, _P, _P, _P, _P, _P]),
    "cpfem_spmv": (ctypes.c_int, [_SP, _P, _P, _P, _I32, _P]),
    "cpfem_bicgstab_workspace_bytes": (ctypes.c_size_t, [_I32]),
    "cpfem_bicgstab": (ctypes.c_int, [_SP, _P, _P, _P, _I32, _I32, _D, _D, _I32, _P, _P, _P]),
    "cpfem_bicgstab_noalloc": (ctypes.c_int, [_SP, _P, _P, _P, _I32, _I32, _D, _D, _I32, _P, _P]),
    "cpfem_bicgstab_last_stats": (ctypes.c_int, [_P]),
    "cpfem_bicgstab_last_stats_ex": (ctypes.c_int, [_P, _I32]),
    "cpfem_mg_slot_table": (ctypes.c_int, [_I32, _P, _P, _P, _P]),
    "cpfem_struct_size": (ctypes.c_size_t, [_I32]),
    "cpfem_mg_setup": (ctypes.c_int, [ctypes.POINTER(MGHierarchy), _P, _P]),
    "cpfem_bicgstab_ex": (ctypes.c_int, [_SP, _P, _P, _P, ctypes.POINTER(KrylovOpts), _P, _P, _P]),
    "cpfem_bicgstab_batched_workspace_bytes": (ctypes.c_size_t, [_I32]),
    "cpfem_bicgstab_batched": (ctypes.c_int, [_SP, _P, _P, _P, _I32, _D, _D, _I32, _I32, _P, _I32, _P, _P, _P, _P, _P]),
    "cpfem_probe_dfma": (ctypes.c_int, [_I64, _I32, _P, _P, _P]),
}

# the order of cpfem_struct_size's argument
STRUCTS = (Material, GPArgs, VjpArgs, Sell, MGHierarchy, KrylovOpts, SolveReport)

_lib = None


def load():
    """Load the library once and declare every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with "
                          f"`python -c 'import __graft_entry__ as g; g.build()'`")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.cpfem_abi_version() != 3:
        raise ImportError("libcpfem_gb300.so ABI version mismatch")
    for which, st in enumerate(STRUCTS):
        if lib.cpfem_struct_size(which) != ctypes.sizeof(st):
            raise ImportError(f"libcpfem_gb300.so: {st.__name__} is {ctypes.sizeof(st)} bytes here but "
                              f"{lib.cpfem_struct_size(which)} in the library (stale build?)")
    _lib = lib
    return lib


def check(rc):
    if rc != 0:
        msg = load().cpfem_last_error().decode(errors="replace")
        raise CPFEMError(f"cpfem call failed (status {rc}): {msg}")


def ptr(t):
    """Device (or host) address of a tensor / array, or None."""
    if t is None:
        return None
    if hasattr(t, "data_ptr"):
        return t.data_ptr()
    return t.ctypes.data
