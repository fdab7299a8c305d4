"""Test infrastructure only (the oracle): a NumPy restatement of
fastode.ts1.TS1.rate_constants (fastode/ts1.py:66-103) that reads the
package's compiled rate-law records (fo_rate_law: type, parameter column,
constants) instead of the reaction dictionaries. Same expressions in the same
order as the reference, so on the same host it gives the reference's rate
constants bit for bit; tests use it to check the law table, never the device
path.
"""
from __future__ import annotations

import math

import numpy as np

BOLTZMANN = 1.380649e-23
AVOGADRO = 6.02214076e23
R_GAS = BOLTZMANN * AVOGADRO
ARRHENIUS, TROE, USER, SURFACE = 0, 1, 2, 3


def rate_constants(law_type, law_column, law_c, params, T, P, power):
    """(C, R) k from the law records; params (ncolumns, C)."""
    T = np.asarray(T, dtype=float)
    P = np.asarray(P, dtype=float)
    M = P / (R_GAS * T)                                              # fastode/ts1.py:71
    k = np.empty((len(T), len(law_type)))
    for j, (t, col, c) in enumerate(zip(law_type, law_column, law_c)):
        c = [float(x) for x in c]
        if t == ARRHENIUS:                                           # :75-78
            A, B, Cc, D, E = c[:5]
            k[:, j] = A * np.exp(Cc / T) * (T / D) ** B * (1.0 + E * P)
        elif t == TROE:                                              # :79-84
            k0 = c[0] * np.exp(c[2] / T) * (T / 300.0) ** c[1]
            kinf = c[3] * np.exp(c[5] / T) * (T / 300.0) ** c[4]
            Fc, N = c[6], c[7]
            ratio = k0 * M / kinf
            k[:, j] = k0 * M / (1.0 + ratio) * Fc ** (N / (N + np.log10(ratio) ** 2))
        elif t == USER:                                              # :85-86
            k[:, j] = params[col] * c[0]
        elif t == SURFACE:                                           # :87-96
            radius, number = params[col], params[col + 1]
            v = np.sqrt(c[0] * T)
            k[:, j] = 4.0 * number * math.pi * radius * radius / (radius / c[1] + 4.0 / (v * c[2]))
        else:
            raise ValueError(f"rate type {t}")
    power = np.asarray(power, dtype=float)
    if np.any(power):                                                # :99-102
        k *= M[:, None] ** power[None, :]
    return k
