"""Rosenbrock tableaus in the transformed (KPP) form.

The stage equations are

    (M/(h*gamma) - J) K_r = F(Y + sum_s a[r,s] K_s) + (M/h) sum_s c[r,s] K_s
    Y_new = Y + sum_r m[r] K_r,        E = sum_r e[r] K_r

with the ROS3 and RODAS3 coefficients of Sandu et al. (1997) as KPP prints
them. The constants and the forcing-reuse rule follow fastode/tableaus.py:15-90
of the reference; they are published method data, kept digit for digit so that
the device integrator and the reference take identical steps.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass(frozen=True)
class Tableau:
    name: str
    gamma: float
    a: np.ndarray        # (S, S) strictly lower triangular
    c: np.ndarray        # (S, S) strictly lower triangular
    m: np.ndarray        # (S,)
    e: np.ndarray        # (S,)
    order: int
    embedded: int
    ident: int           # tableau id passed through the C-ABI

    @property
    def stages(self) -> int:
        return len(self.m)

    @property
    def k(self) -> float:
        """Order of the error estimate plus one; the controller exponent is 1/k
        (fastode/tableaus.py:30-33)."""
        return float(self.embedded + 1)

    @property
    def new_forcing(self) -> list:
        """Stage r evaluates F anew unless its predicted point equals stage
        r-1's (fastode/tableaus.py:35-42)."""
        out = [True]
        for r in range(1, self.stages):
            prev = list(self.a[r - 1, : r - 1]) + [0.0]
            same = all(float(x) == float(y) for x, y in zip(self.a[r, :r], prev))
            out.append(not same)
        return out

    def standard_form(self):
        """(A, Gamma, b, bhat) of the standard Rosenbrock form."""
        S = self.stages
        G = np.linalg.inv(np.eye(S) / self.gamma - self.c)
        A = self.a @ G
        b = G.T @ self.m
        return A, G, b, b - G.T @ self.e

    def packed(self) -> np.ndarray:
        """The 4x4-padded coefficient block handed to the device:
        [gamma, S, a(16), c(16), m(4), e(4), new_forcing(4)] as float64."""
        S = self.stages
        a = np.zeros((4, 4)); a[:S, :S] = self.a
        c = np.zeros((4, 4)); c[:S, :S] = self.c
        m = np.zeros(4); m[:S] = self.m
        e = np.zeros(4); e[:S] = self.e
        nf = np.zeros(4); nf[:S] = [1.0 if f else 0.0 for f in self.new_forcing]
        return np.concatenate([[self.gamma, float(S)], a.ravel(), c.ravel(), m, e, nf])


def _strict_lower(S, values):
    out = np.zeros((S, S))
    it = iter(values)
    for r in range(1, S):
        for s in range(r):
            out[r, s] = next(it)
    return out


ROS3 = Tableau(
    name="ros3",
    gamma=0.43586652150845899941601945119356,
    a=_strict_lower(3, [1.0, 1.0, 0.0]),
    c=_strict_lower(3, [-0.10156171083877702091975600115545e01,
                        0.40759956452537699824805835358067e01,
                        0.92076794298330791242156818474003e01]),
    m=np.array([1.0, 0.61697947043828245592553615689730e01,
                -0.42772256543218573326238373806514]),
    e=np.array([0.5, -0.29079558716805469821718236208017e01,
                0.22354069897811569627360909276199]),
    order=3, embedded=2, ident=0,
)

RODAS3 = Tableau(
    name="rodas3",
    gamma=0.5,
    a=_strict_lower(4, [0.0, 2.0, 0.0, 2.0, 0.0, 1.0]),
    c=_strict_lower(4, [4.0, 1.0, -1.0, 1.0, -1.0, -8.0 / 3.0]),
    m=np.array([2.0, 0.0, 1.0, 1.0]),
    e=np.array([0.0, 0.0, 0.0, 1.0]),
    order=3, embedded=2, ident=1,
)

TABLEAUS = {"ros3": ROS3, "rodas3": RODAS3}
