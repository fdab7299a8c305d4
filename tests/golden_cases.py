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


DAE_CASES = ("rodas3_robertson_qssa", "rodas3_chapman_qssa", "rodas3_tropospheric_qssa")


class _Pattern:
    def __init__(self, rows, cols):
        self.rows = np.asarray(rows, dtype=np.int64)
        self.cols = np.asarray(cols, dtype=np.int64)
        self.nnz = len(self.rows)


class TableMechanism:
    """A mechanism given by the reference's compiled tables (react, S,
    pattern, GT map) as stored in a fixture."""

    def __init__(self, f):
        self.n, self.R, self.P = int(f["m_n"]), int(f["m_R"]), int(f["m_P"])
        self.react = np.asarray(f["m_react"], dtype=np.int64)
        self.S = np.asarray(f["m_S"], dtype=np.float64)
        self.pattern = _Pattern(f["m_rows"], f["m_cols"])
        self._gt = (np.asarray(f["m_gt_indptr"], np.int32), np.asarray(f["m_gt_indices"], np.int32),
                    np.asarray(f["m_gt_data"], np.float64))
        self.species = [f"y{i}" for i in range(self.n)]

    def jac_csr(self):
        return tuple(a.copy() for a in self._gt)

    def dense_jacobian(self, vals):
        J = np.zeros((vals.shape[0], self.n, self.n))
        J[:, self.pattern.rows, self.pattern.cols] = vals
        return J


def table_mechanism(f):
    """TableMechanism from a fixture that stores S as COO (m_S_rows/cols/vals)."""
    if "m_S" not in f:
        S = np.zeros((int(f["m_n"]), int(f["m_R"])))
        S[f["m_S_rows"], f["m_S_cols"]] = f["m_S_vals"]
        f = dict(f, m_S=S)
    return TableMechanism(f)


def ts1_k(f, i):
    """Rate constants of interval i of the TS1 fixture, built as the
    reference's run_scenario builds them (fastode/ts1.py:204-214): the static
    k with every photolysis column set to (base * f(t)) * scaling."""
    k = np.array(f["k_static"], copy=True)
    k[:, f["photo"]] = (f["base"] * f["f"][i]) * f["scaling"][None, :]
    return k
