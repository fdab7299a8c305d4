"""Autotuner: choose the kernel variant, the group size, the launch shape and
the generated code's register tiling per mechanism by measuring them on a
sample of the workload.

The dimensions:
  * kernel: the generated variant (the mechanism's own straight-line code) or
    a table-driven one (compact, pipelined, plain);
  * group size: cells per group (one thread per cell; the generated variant
    runs groups of up to 32 cells);
  * tile: the rows and columns of the generated factorization's register
    tiles (register tiling of the factorization: the larger the tile, the
    fewer loads per multiply-add and the more registers), measured against
    the occupancy it costs;
  * persistent: one block per group, or persistent blocks pulling a queue.
Threads per cell is one: on GB300 a double-precision warp instruction costs
the same issue slot whether one lane or 32 are active, and a second lane per
cell would wait on the first through every pivot of the elimination, so every
lane integrates a cell of its own.

Group size is a numerical choice as well as a speed one: the cells of a group
share one step sequence and one error norm (the reference's groups of 32,
fastode/ts1.py:196), so a larger group takes the steps its stiffest cell needs
and a smaller one wastes lanes of a warp (a warp of 32 lanes costs the same
FP64 issue slots however many lanes hold cells). The tuner therefore scores
candidates by cell-intervals per second on the sample, which counts both.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

SMEM_LIMIT = 232448


@dataclass(frozen=True)
class Config:
    kernel: str = "compact"       # FO_VARIANT_*
    group_size: int = 32
    persistent: bool = False      # one block per group, or persistent blocks pulling a queue
    tile: int = 6                 # the generated factorization's register tile


@dataclass
class TuneResult:
    best: Config
    table: list = field(default_factory=list)   # (config, cell-intervals/s or None when it does not fit)


def _items(smem_doubles_per_cell, kernel: str) -> int:
    """Shared-memory doubles per cell: one figure for every kernel, or a dict
    kernel -> figure (the compact kernel needs about half)."""
    if isinstance(smem_doubles_per_cell, dict):
        return smem_doubles_per_cell[kernel]
    return smem_doubles_per_cell


def fits(smem_doubles_per_cell, group_size: int, kernel: str = "pipelined") -> bool:
    if kernel == "generated" and group_size > 32:
        return False                      # the generated code runs groups of at most 32 cells
    lanes = ((group_size + 31) // 32) * 32
    return 8 * (32 + _items(smem_doubles_per_cell, kernel) * lanes) <= SMEM_LIMIT


def candidates(smem_doubles_per_cell: int, group_sizes=(16, 32, 64, 128),
               kernels=("compact", "pipelined", "plain"), persistent=(False, True), tiles=(6,)) -> list:
    out = []
    for k in kernels:
        for g in group_sizes:
            for p in persistent:
                for t in (tiles if k == "generated" else (6,)):
                    out.append(Config(k, g, p, t))
    return out


def autotune(measure, smem_doubles_per_cell: int, configs=None) -> TuneResult:
    """measure(config) -> cell-intervals/s; configs that do not fit in shared
    memory are skipped (scored None). Returns the fastest."""
    configs = configs if configs is not None else candidates(smem_doubles_per_cell)
    table = []
    best, best_v = None, -1.0
    for c in configs:
        if not fits(smem_doubles_per_cell, c.group_size, c.kernel):
            table.append((c, None))
            continue
        v = float(measure(c))
        table.append((c, v))
        if v > best_v:
            best, best_v = c, v
    if best is None:
        raise ValueError("no candidate configuration fits in shared memory")
    return TuneResult(best, table)


def measure_on_device(mech, Y0, k_of, dt, atol, rtol, warm: int = 1, timed: int = 2, mass=None):
    """A measure function for ``autotune``: integrates the sample cells Y0
    (C, n) with each configuration over `warm` untimed and `timed` timed
    intervals (k_of(i) -> (C, R) host rate constants) and returns
    cell-intervals per second of the timed intervals."""
    import torch

    from .batch import Batch
    from .multi import default_slots
    from .solvers import Algorithm

    ks = [torch.from_numpy(np.ascontiguousarray(k_of(i).T)).cuda() for i in range(warm + timed)]
    at = torch.from_numpy(np.ascontiguousarray(atol, dtype=np.float64)).cuda()

    def measure(c: Config) -> float:
        alg = Algorithm(kernel=c.kernel, tile=c.tile)
        b = Batch(mech, Y0, group_size=c.group_size, algorithm=alg, mass=mass)
        if c.persistent:
            lanes = ((c.group_size + 31) // 32) * 32
            if c.kernel == "generated":
                per_sm = 16                   # register-bound: 128 registers per thread
            else:
                per_sm = max(1, min(8, SMEM_LIMIT // (8 * (32 + b.plan.smem_items(c.kernel) * lanes))))
            b = Batch(mech, Y0, group_size=c.group_size, algorithm=alg, mass=mass,
                      slots=torch.cuda.get_device_properties(b.plan.device).multi_processor_count * per_sm)
        for i in range(warm):
            b.step(ks[i], dt, at, rtol)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(warm, warm + timed):
            b.step(ks[i], dt, at, rtol)
        torch.cuda.synchronize()
        return b.C * timed / (time.perf_counter() - t0)

    return measure
