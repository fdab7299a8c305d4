"""Loading the golden fixtures of tests/golden/ (made by make_golden.py from
the reference itself) into this package's objects."""
from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ("ros3_20x40", "ros3_210x500")
A_FLOOR = 1.0e-14      # the absolute scale a of atol = rtol * a


def load(name):
    return dict(np.load(GOLDEN / f"{name}.npz"))


def reactions_of(f):
    n = int(f["n"])
    species = [f"S{i:03d}" for i in range(n)]
    out = []
    for rt, pt, yt in zip(f["reactants"], f["products"], f["yields"]):
        reactants = ["M" if r == -2 else species[r] for r in rt if r != -1]
        products = [(species[p], float(y)) for p, y in zip(pt, yt) if p != -1]
        out.append((reactants, products))
    return species, out


def mechanism_of(f):
    from fastode_gb300.chem import Mechanism
    species, reactions = reactions_of(f)
    return Mechanism(species, reactions)


def rel_err(y, ref, floor=A_FLOOR):
    """|y - ref| / max(|ref|, a), elementwise."""
    return np.abs(y - ref) / np.maximum(np.abs(ref), floor)
