"""ctypes binding of the C-ABI in include/fastode_gb300.h.

The shared library is required: there is no host fallback. Loading raises
``RuntimeError`` with the build command when the library is missing.
"""
from __future__ import annotations

import ctypes as C
import threading

from .build import library_path

FO_OK = 0
FO_E_INVALID, FO_E_CUDA, FO_E_UNSUPPORTED, FO_E_WORKSPACE, FO_E_ALLOC = -1, -2, -3, -4, -5
STATUS_STRINGS = ("converged", "too many steps", "step too small", "nan or inf", "projection failed",
                  "accepted unconverged")
NUM_COUNTS = 13
ORDERINGS = {"auto": 0, "natural": 1, "min_degree": 2, "min_fill": 3, "refined": 4}
ORDERING_NAMES = {v: k for k, v in ORDERINGS.items()}


class MechanismDesc(C.Structure):
    _fields_ = [("n", C.c_int32), ("R", C.c_int32), ("P", C.c_int32),
                ("react", C.POINTER(C.c_int64)),
                ("s_indptr", C.POINTER(C.c_int32)), ("s_idx", C.POINTER(C.c_int32)),
                ("s_val", C.POINTER(C.c_double)),
                ("nnz", C.c_int32),
                ("pat_rows", C.POINTER(C.c_int64)), ("pat_cols", C.POINTER(C.c_int64)),
                ("j_indptr", C.POINTER(C.c_int32)), ("j_idx", C.POINTER(C.c_int32)),
                ("j_val", C.POINTER(C.c_double)),
                ("mass", C.POINTER(C.c_double))]


class PlanInfo(C.Structure):
    _fields_ = [("n", C.c_int32), ("R", C.c_int32), ("P", C.c_int32), ("nnz_jac", C.c_int32),
                ("ordering", C.c_int32), ("nnz_lu", C.c_int32), ("nnz_l", C.c_int32), ("nnz_u", C.c_int32),
                ("lu_fma", C.c_int64), ("solve_fma", C.c_int64), ("jac_terms", C.c_int32),
                ("stoich_nnz", C.c_int32), ("scratch_doubles_per_cell", C.c_int64),
                ("smem_doubles_per_cell", C.c_int32), ("compact_smem_doubles_per_cell", C.c_int32)]

    def as_dict(self):
        d = {name: getattr(self, name) for name, _ in self._fields_}
        d["ordering"] = ORDERING_NAMES.get(d["ordering"], d["ordering"])
        return d


class Options(C.Structure):
    _fields_ = [("tableau", C.c_int32), ("controller", C.c_int32), ("b", C.c_double),
                ("safety", C.c_double), ("fac_min", C.c_double), ("fac_max", C.c_double),
                ("carry", C.c_int32), ("quantize", C.c_int32), ("carry_memory", C.c_int32),
                ("max_steps", C.c_int32), ("variant", C.c_int32), ("loop", C.c_int32),
                ("step_change_rows", C.c_int32),
                ("max_iterations", C.c_int32), ("nreductions", C.c_int32),
                ("reductions", C.c_double * 8), ("small", C.c_double), ("lockstep", C.c_int32)]


VARIANTS = {"pipelined": 0, "plain": 1, "compact": 2, "generated": 3}
LOOPS = {"algorithm": 0, "restarting": 1, "backward-euler": 2}
SCORE_RULES = {"ts1": 0, "digits": 1}


class GenInfo(C.Structure):
    _fields_ = [("from_cache", C.c_int32), ("registers", C.c_int32), ("tile", C.c_int32),
                ("local_bytes", C.c_int32), ("seconds", C.c_double), ("ptx_bytes", C.c_int64),
                ("cubin_bytes", C.c_int64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}


class RateLaw(C.Structure):
    _fields_ = [("type", C.c_int32), ("column", C.c_int32), ("c", C.c_double * 8)]


RATE_ARRHENIUS, RATE_TROE, RATE_USER, RATE_SURFACE = 0, 1, 2, 3


class BatchDesc(C.Structure):
    _fields_ = [("plan", C.c_void_p), ("opt", Options), ("ngroups", C.c_int32),
                ("group_offsets", C.c_void_p), ("max_group_cells", C.c_int32),
                ("Y", C.c_void_p), ("y_cell_stride", C.c_int64), ("y_species_stride", C.c_int64),
                ("k", C.c_void_p), ("k_cell_stride", C.c_int64), ("k_reaction_stride", C.c_int64),
                ("atol", C.c_void_p), ("rtol", C.c_double), ("dt", C.c_double),
                ("memory", C.c_void_p), ("counts", C.c_void_p), ("status", C.c_void_p)]


_P = C.c_void_p
_I32 = C.c_int32
_I64 = C.c_int64
_D = C.c_double

# name -> (restype, argtypes); the declarations of include/fastode_gb300.h
SIGNATURES = {
    "fo_last_error": (C.c_char_p, []),
    "fo_analyze": (C.c_int, [C.POINTER(MechanismDesc), _I32, C.POINTER(PlanInfo), C.POINTER(C.c_int32)]),
    "fo_plan_create": (C.c_int, [C.POINTER(MechanismDesc), _I32, C.POINTER(_P)]),
    "fo_plan_info_get": (C.c_int, [_P, C.POINTER(PlanInfo)]),
    "fo_plan_destroy": (C.c_int, [_P]),
    "fo_plan_permutation": (C.c_int, [_P, C.POINTER(C.c_int32)]),
    "fo_workspace_bytes": (C.c_int, [_P, _I32, _I32, C.POINTER(C.c_size_t)]),
    "fo_plan_generate": (C.c_int, [_P, C.c_char_p, C.POINTER(GenInfo)]),
    "fo_plan_set_generation": (C.c_int, [_P, _I32, _I32]),
    "fo_generate_check": (C.c_int, [C.POINTER(MechanismDesc), _I32, _I32, C.POINTER(GenInfo)]),
    "fo_solve": (C.c_int, [_P, C.POINTER(Options), _I32, _P, _I32,
                           _P, _I64, _I64, _P, _I64, _I64, _P, _D, _D,
                           _P, _P, _P, _P, C.c_size_t, _I32, _P, _I32, _P, _P]),
    "fo_solve_static": (C.c_int, [_P, C.POINTER(Options), _I32, _P, _I32,
                                  _P, _I64, _I64, _P, _I64, _I64, _P, _D, _D, _P, _P, _P, _P]),
    "fo_eval_rhs": (C.c_int, [_P, _I32, _P, _I64, _I64, _P, _I64, _I64, _P, _P]),
    "fo_eval_jac": (C.c_int, [_P, _I32, _P, _I64, _I64, _P, _I64, _I64, _P, _P]),
    "fo_rate_constants": (C.c_int, [_I32, _I32, _P, _P, _P, _P, _P, _P, _I64, _I64, _P]),
    "fo_update_photolysis": (C.c_int, [_I32, _I32, _P, _P, _P, _D, _D, _P, _I64, _I64, _P]),
    "fo_photolysis_factor": (C.c_int, [_I32, _I32, _P, _P, _P, _P, _I64, _I64, _P]),
    "fo_rate_laws": (C.c_int, [_I32, _I32, _P, _P, _P, _P, _I64, _P, _P, _I64, _I64, _P]),
    "fo_fp64_fma_rate": (C.c_int, [C.POINTER(C.c_double)]),
    "fo_scale_photolysis": (C.c_int, [_I32, _I32, _P, _P, _P, _D, _P, _I64, _I64, _P]),
    "fo_score_accumulate": (C.c_int, [_I32, _I32, _P, _I64, _I64, _I32, _P, _P, _I64, _I64, _D, _I32,
                                      _P, _P, _P, _P]),
    "fo_multi_workspace_bytes": (C.c_int, [_I32, C.POINTER(BatchDesc), _I32, C.POINTER(C.c_size_t)]),
    "fo_multi_prepare": (C.c_int, [_I32, C.POINTER(BatchDesc), _P, C.c_size_t, _I32, C.POINTER(_P)]),
    "fo_multi_launch": (C.c_int, [_P, _P]),
    "fo_multi_destroy": (C.c_int, [_P]),
    "fo_update_photolysis_clock": (C.c_int, [_I32, _I32, _P, _P, _P, _D, _P, _P, _I64, _I64, _P]),
    "fo_advance_clock": (C.c_int, [_P, _D, _P]),
    "fo_adjoint_workspace_bytes": (C.c_int, [_P, _I32, _I32, _I32, C.POINTER(C.c_size_t)]),
    "fo_adjoint_interval": (C.c_int, [_P, C.POINTER(Options), _I32, _P, _I32,
                                      _P, _I64, _I64, _P, _I64, _I64, _P, _D,
                                      _P, _P, _I32, _P, _P, _I32,
                                      _P, _I64, _I64, _P, _I64, _I64, _P, _I64, _I64,
                                      _P, _P, C.c_size_t, _P]),
}

_lib = None
_lock = threading.Lock()


class FastodeError(RuntimeError):
    pass


def lib():
    """The loaded library; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            path = library_path()
            if not path.exists():
                raise RuntimeError(f"{path} is missing: build it with `python -m fastode_gb300.build` "
                                   "(the GPU integrator has no host fallback)")
            handle = C.CDLL(str(path))
            for name, (res, args) in SIGNATURES.items():
                f = getattr(handle, name)
                f.restype = res
                f.argtypes = args
            _lib = handle
    return _lib


def check(rc: int, what: str) -> None:
    if rc != FO_OK:
        msg = lib().fo_last_error().decode(errors="replace")
        raise FastodeError(f"{what} failed (code {rc}): {msg}")
