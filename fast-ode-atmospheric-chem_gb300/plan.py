"""Plans: a mechanism (and mass vector) analysed and uploaded to the GPU.

A plan is what the reference rebuilds on every factorization — the ordering
and fill of SuperLU (fastode/linalg.py:70-78) — plus the mechanism's compiled
tables (fastode/chem.py:19-79), computed once on the host by the library's
symbolic analysis and kept on the device.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np

from . import _abi
from .chem import mechanism_tables


def _ptr(a: np.ndarray, ctype):
    return a.ctypes.data_as(C.POINTER(ctype))


class _Desc:
    """A MechanismDesc with the numpy arrays it points into kept alive."""

    def __init__(self, mech, mass=None):
        t = mechanism_tables(mech)
        self.tables = t
        self.arrays = {k: np.ascontiguousarray(v) for k, v in t.items() if isinstance(v, np.ndarray)}
        a = self.arrays
        self.mass = None if mass is None else np.ascontiguousarray(np.asarray(mass, dtype=np.float64))
        self.desc = _abi.MechanismDesc(
            t["n"], t["R"], t["P"],
            _ptr(a["react"], C.c_int64),
            _ptr(a["s_indptr"], C.c_int32), _ptr(a["s_idx"], C.c_int32), _ptr(a["s_val"], C.c_double),
            len(a["rows"]),
            _ptr(a["rows"], C.c_int64), _ptr(a["cols"], C.c_int64),
            _ptr(a["j_indptr"], C.c_int32), _ptr(a["j_idx"], C.c_int32), _ptr(a["j_val"], C.c_double),
            _ptr(self.mass, C.c_double) if self.mass is not None else None,
        )


def analyze(mech, ordering: str = "auto", mass=None) -> dict:
    """Host-only symbolic analysis (no GPU): ordering, fill and flop counts;
    ``perm`` is the elimination order."""
    d = _Desc(mech, mass)
    info = _abi.PlanInfo()
    perm = np.zeros(int(mech.n), dtype=np.int32)
    _abi.check(_abi.lib().fo_analyze(C.byref(d.desc), _abi.ORDERINGS[ordering], C.byref(info),
                                     _ptr(perm, C.c_int32)), "fo_analyze")
    out = info.as_dict()
    out["perm"] = perm
    return out


class Plan:
    """A device plan for one mechanism and mass vector."""

    def __init__(self, mech, mass=None, ordering: str = "auto", tile: int = 6):
        import torch
        if not torch.cuda.is_available():
            raise RuntimeError("fastode_gb300 needs a CUDA GPU: there is no host integrator")
        self.mech = mech
        self._desc = _Desc(mech, mass)
        self.n = self._desc.tables["n"]
        self.R = self._desc.tables["R"]
        self.P = self._desc.tables["P"]
        self.nnz = len(self._desc.arrays["rows"])
        self.mass = np.ones(self.n) if mass is None else np.asarray(mass, dtype=np.float64)
        self.device = torch.cuda.current_device()
        handle = C.c_void_p()
        _abi.check(_abi.lib().fo_plan_create(C.byref(self._desc.desc), _abi.ORDERINGS[ordering],
                                             C.byref(handle)), "fo_plan_create")
        self.handle = handle
        self._finalizer = weakref.finalize(self, _abi.lib().fo_plan_destroy, handle)
        self.tile = int(tile)
        _abi.check(_abi.lib().fo_plan_set_generation(handle, self.tile, 8), "fo_plan_set_generation")
        info = _abi.PlanInfo()
        _abi.check(_abi.lib().fo_plan_info_get(handle, C.byref(info)), "fo_plan_info_get")
        self.info = info.as_dict()
        perm = np.zeros(self.n, dtype=np.int32)
        _abi.check(_abi.lib().fo_plan_permutation(handle, _ptr(perm, C.c_int32)), "fo_plan_permutation")
        self.perm = perm
        self._workspaces = {}
        self.gen_info = None

    def generate(self, cache_dir=None) -> dict:
        """Prepare the generated variant (fo_plan_generate): the mechanism's
        factorization and solves as straight-line code linked with the
        integrator, cached on disk; idempotent. Returns what it did."""
        if self.gen_info is None:
            info = _abi.GenInfo()
            arg = None if cache_dir is None else str(cache_dir).encode()
            _abi.check(_abi.lib().fo_plan_generate(self.handle, arg, C.byref(info)), "fo_plan_generate")
            self.gen_info = info.as_dict()
        return self.gen_info

    def options_for(self, algorithm, max_group_cells: int):
        """The fo_options of `algorithm` for groups of up to `max_group_cells`
        cells. The generated variant prepares this plan first; it runs groups
        of at most 32 cells, so larger groups take the compact variant."""
        o = algorithm.options()
        if algorithm.kernel == "generated":
            if max_group_cells <= 32:
                self.generate()
            else:
                o.variant = _abi.VARIANTS["compact"]
        return o

    @property
    def has_constraints(self) -> bool:
        return bool(np.any(self.mass == 0.0))

    def smem_items(self, kernel: str = "pipelined") -> int:
        """Shared-memory doubles per cell of a block running ``kernel``."""
        if kernel == "compact":
            return int(self.info["compact_smem_doubles_per_cell"])
        return int(self.info["smem_doubles_per_cell"])

    def workspace_bytes(self, slots: int, max_group_cells: int) -> int:
        out = C.c_size_t()
        _abi.check(_abi.lib().fo_workspace_bytes(self.handle, int(slots), int(max_group_cells), C.byref(out)),
                   "fo_workspace_bytes")
        return int(out.value)

    def workspace(self, slots: int, max_group_cells: int):
        """A cached device workspace big enough for (slots, max_group_cells)."""
        import torch
        need = self.workspace_bytes(slots, max_group_cells)
        ws = self._workspaces.get("ws")
        if ws is None or ws.numel() < need:
            ws = torch.empty(need, dtype=torch.uint8, device=f"cuda:{self.device}")
            self._workspaces["ws"] = ws
        return ws

    def flops_per_attempt(self, stages: int = 3, new_rhs: int = 1) -> dict:
        """FP64 operations of one attempt by part (multiply-adds count 2)."""
        i = self.info
        n = self.n
        lu = 2 * i["lu_fma"] + i["nnz_l"] + n            # updates, multipliers, reciprocals
        solve = 2 * i["solve_fma"] + n                     # per stage solve
        rates = self.R * self.P                            # products incl. k
        rhs = rates + 2 * i["stoich_nnz"]
        jac = self.R * self.P * max(self.P - 1, 1) + 2 * i["jac_terms"]
        return {"lu": lu, "solve": solve, "rhs": rhs, "jac": jac}


_cache: dict = {}


def plan_for(mech, mass=None, ordering: str = "auto", tile: int = 6) -> Plan:
    """The cached plan of a mechanism object (reference or this package's),
    mass vector and generated-code tile on the current device."""
    import torch
    m = np.ones(mech.n) if mass is None else np.asarray(mass, dtype=np.float64)
    key = (id(mech), m.tobytes(), ordering, int(tile), torch.cuda.current_device())
    hit = _cache.get(key)
    if hit is not None and hit.mech is mech:
        return hit
    p = Plan(mech, m, ordering, tile)
    _cache[key] = p
    return p
