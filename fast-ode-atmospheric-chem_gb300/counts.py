"""Operation counters of one integrator call on a group of cells.

Field names, order and meaning follow fastode/counts.py:10-30 of the reference:
every count is per call of the counted operation on a whole group, so counts per
group are counts per cell. The device writes the same thirteen fields as int64,
one row per group (``COUNT_FIELDS`` gives the column order of that row).
"""
from __future__ import annotations

from dataclasses import dataclass, fields

COUNT_FIELDS = ("steps", "accepted", "rejected", "rhs", "jac", "lu", "solves", "newton",
                "failures", "unconverged", "proj_passes", "proj_trials", "calls")


@dataclass
class Counts:
    steps: int = 0          # attempted steps (accepted + rejected)
    accepted: int = 0
    rejected: int = 0
    rhs: int = 0            # right-hand-side (forcing) evaluations
    jac: int = 0            # Jacobian evaluations
    lu: int = 0             # factorizations
    solves: int = 0         # triangular-solve pairs
    newton: int = 0         # Newton iterations (backward Euler)
    failures: int = 0       # Newton convergence failures (backward Euler)
    unconverged: int = 0    # unconverged iterates accepted (backward Euler)
    proj_passes: int = 0    # projection passes (consistent initialization)
    proj_trials: int = 0    # projection line-search trials
    calls: int = 0          # solver calls (intervals)

    def add(self, other: "Counts") -> None:
        for f in fields(self):
            setattr(self, f.name, getattr(self, f.name) + getattr(other, f.name))

    def add_row(self, row) -> None:
        """Accumulate one device counts row (13 integers in COUNT_FIELDS order)."""
        for name, v in zip(COUNT_FIELDS, row):
            setattr(self, name, getattr(self, name) + int(v))

    def as_dict(self) -> dict:
        return {f.name: getattr(self, f.name) for f in fields(self)}
