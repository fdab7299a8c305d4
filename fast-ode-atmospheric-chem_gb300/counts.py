"""Operation counters of one integrator call on a group of cells.

Field names, order and meaning follow fastode/counts.py:10-30 of the reference:
every count is per call of the counted operation on a whole group, so counts per
group are counts per cell. The device writes the same thirteen fields as int64,
one row per group (``COUNT_FIELDS`` gives the column order of that row).
"""
from __future__ import annotations

from dataclasses import dataclass

COUNT_FIELDS = ("steps", "accepted", "rejected", "rhs", "jac", "lu", "solves", "newton",
                "failures", "unconverged", "proj_passes", "proj_trials", "calls")


@dataclass
class Counts:
    """Thirteen integer counters, accumulated over calls. The three step
    counters split every try of a step size into taken and retried; the next
    four count the work each try costs (forcing evaluations, Jacobian
    evaluations, factorizations of the stage matrix, and forward/backward
    substitution pairs); the backward Euler loop alone moves the Newton
    counters; the projection of constrained systems moves the two projection
    counters; ``calls`` counts intervals."""

    steps: int = 0
    accepted: int = 0
    rejected: int = 0
    rhs: int = 0
    jac: int = 0
    lu: int = 0
    solves: int = 0
    newton: int = 0
    failures: int = 0
    unconverged: int = 0
    proj_passes: int = 0
    proj_trials: int = 0
    calls: int = 0

    def add(self, other: "Counts") -> None:
        """Accumulate another Counts field by field."""
        for name in COUNT_FIELDS:
            setattr(self, name, getattr(self, name) + getattr(other, name))

    def add_row(self, row) -> None:
        """Accumulate one device counts row (13 integers in COUNT_FIELDS order)."""
        for name, v in zip(COUNT_FIELDS, row):
            setattr(self, name, getattr(self, name) + int(v))

    def as_dict(self) -> dict:
        """The counters by name, in COUNT_FIELDS order."""
        return dict(zip(COUNT_FIELDS, (getattr(self, name) for name in COUNT_FIELDS)))
