"""Seeded synthetic mass-action mechanisms and cells.

The reference publishes no benchmark inputs for its integrator, so these
generators define the workloads: each reaction has 1-2 reactants drawn uniformly
from the species and 1-3 products with yields U(0.1, 1]; thermal rate constants
are k = A exp(-E/T) with A log-uniform on [1e-20, 1e-10] and E uniform on
[0, 2000] K; 15% of the reactions (rounded) are photolytic, with one reactant
and J log-uniform on [1e-8, 1e-2] s^-1. With ``third_body_fraction`` > 0 that
fraction of the thermal reactions carries a third body M whose density
[M] = p / (R T) (mol m^-3) is folded into k, as fastode/ts1.py:72,100-102 does.

Cells draw T, pressure, initial concentrations (log-uniform on [1e-15, 1e-3]
mol m^-3) and a solar phase; photolysis is J * f(t) with the diurnal cosine
f = max(0, cos(phase + 2 pi t / 86400)), updated at interval starts as
fastode/ts1.py:204-214 updates the scenario's photolysis columns.

Everything is a pure function of the seed, so the reference and the device
integrator consume bit-identical inputs.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .chem import Mechanism

BOLTZMANN = 1.380649e-23
AVOGADRO = 6.02214076e23
R_GAS = BOLTZMANN * AVOGADRO


@dataclass
class SyntheticMechanism:
    mech: Mechanism
    species: list
    reactions: list          # (reactants, products) as passed to Mechanism
    A: np.ndarray            # (R,) pre-exponential factors (0 for photolysis)
    E: np.ndarray            # (R,) activation temperatures [K]
    J: np.ndarray            # (R,) photolysis rates at f = 1 (0 for thermal)
    photolytic: np.ndarray   # (R,) bool

    @property
    def n(self):
        return self.mech.n

    @property
    def R(self):
        return self.mech.R


def synthetic_mechanism(n_species: int, n_reactions: int, seed: int,
                        photolytic_fraction: float = 0.15,
                        third_body_fraction: float = 0.0) -> SyntheticMechanism:
    rng = np.random.default_rng(seed)
    n, R = int(n_species), int(n_reactions)
    species = [f"S{i:03d}" for i in range(n)]
    n_photo = int(round(photolytic_fraction * R))
    photolytic = np.zeros(R, dtype=bool)
    photolytic[rng.choice(R, size=n_photo, replace=False)] = True
    reactions = []
    A = np.zeros(R)
    E = np.zeros(R)
    J = np.zeros(R)
    for j in range(R):
        n_react = 1 if photolytic[j] else int(rng.integers(1, 3))
        reactants = [species[int(i)] for i in rng.integers(0, n, size=n_react)]
        n_prod = int(rng.integers(1, 4))
        prod_idx = rng.integers(0, n, size=n_prod)
        yields = 0.1 + 0.9 * (1.0 - rng.random(n_prod))          # (0.1, 1]
        products = [(species[int(i)], float(y)) for i, y in zip(prod_idx, yields)]
        if photolytic[j]:
            J[j] = 10.0 ** rng.uniform(-8.0, -2.0)
        else:
            A[j] = 10.0 ** rng.uniform(-20.0, -10.0)
            E[j] = rng.uniform(0.0, 2000.0)
            if third_body_fraction > 0.0 and rng.random() < third_body_fraction:
                reactants = reactants + ["M"]
        reactions.append((reactants, products))
    mech = Mechanism(species, reactions)
    return SyntheticMechanism(mech, species, reactions, A, E, J, photolytic)


@dataclass
class SyntheticCells:
    T: np.ndarray            # (C,) temperature [K]
    p: np.ndarray            # (C,) pressure [Pa]
    phase: np.ndarray        # (C,) solar phase [rad]
    Y0: np.ndarray           # (C, n) initial concentrations [mol m^-3]

    @property
    def C(self):
        return len(self.T)


def synthetic_cells(sm: SyntheticMechanism, n_cells: int, seed: int,
                    T_range=(220.0, 300.0), p_range_hpa=(1013.25, 1013.25),
                    phase_range=(0.0, 0.0)) -> SyntheticCells:
    rng = np.random.default_rng(seed)
    C = int(n_cells)
    T = rng.uniform(T_range[0], T_range[1], size=C)
    p = 100.0 * rng.uniform(p_range_hpa[0], p_range_hpa[1], size=C)
    phase = rng.uniform(phase_range[0], phase_range[1], size=C)
    Y0 = 10.0 ** rng.uniform(-15.0, -3.0, size=(C, sm.n))
    return SyntheticCells(T, p, phase, Y0)


def diurnal_factor(cells: SyntheticCells, t: float) -> np.ndarray:
    """Photolysis factor max(0, cos(phase + 2 pi t / 86400)) per cell."""
    return np.maximum(0.0, np.cos(cells.phase + 2.0 * math.pi * t / 86400.0))


def rate_constants(sm: SyntheticMechanism, cells: SyntheticCells, t: float = 0.0) -> np.ndarray:
    """k of shape (C, R) at time t: Arrhenius (times [M]^power for third bodies)
    for thermal reactions, J * f(t) for photolytic ones."""
    T = cells.T[:, None]
    k = sm.A[None, :] * np.exp(-sm.E[None, :] / T)
    power = sm.mech.third_body_power
    if np.any(power):
        M = cells.p / (R_GAS * cells.T)
        k = k * M[:, None] ** power[None, :]
    f = diurnal_factor(cells, t)
    photo = sm.photolytic
    k[:, photo] = sm.J[None, photo] * f[:, None]
    return np.ascontiguousarray(k)


# -- the workloads -----------------------------------------------------------------

@dataclass
class Workload:
    name: str
    sm: SyntheticMechanism
    cells: SyntheticCells
    dt: float
    intervals: int
    rtol: float
    group_size: int
    update_photolysis: bool

    @property
    def atol(self) -> np.ndarray:
        """atol = rtol * 1e-14 for every species (a = 1e-14)."""
        return np.full(self.sm.n, self.rtol * 1.0e-14)

    def k_at(self, interval: int) -> np.ndarray:
        t = interval * self.dt if self.update_photolysis else 0.0
        return rate_constants(self.sm, self.cells, t)

    def subset(self, sl: slice) -> "Workload":
        """The same workload restricted to the cells of `sl`."""
        c = self.cells
        cells = SyntheticCells(c.T[sl].copy(), c.p[sl].copy(), c.phase[sl].copy(), c.Y0[sl].copy())
        return Workload(self.name, self.sm, cells, self.dt, self.intervals, self.rtol, self.group_size,
                        self.update_photolysis)


def plain_small(n_cells: int = 64, intervals: int = 20, seed: int = 1) -> Workload:
    """Plain ROS3, 20 species / 40 reactions, 64 cells in groups of 32,
    T U[220, 300] K, dt = 30 s x 20 intervals, rtol 1e-3, constant photolysis."""
    sm = synthetic_mechanism(20, 40, seed)
    cells = synthetic_cells(sm, n_cells, seed + 1000, T_range=(220.0, 300.0))
    return Workload("ros3-20x40", sm, cells, 30.0, intervals, 1.0e-3, 32, False)


def batched_uneven(n_cells: int = 1_048_576, intervals: int = 240, seed: int = 3,
                   sizes=((60, 40), (120, 260), (210, 500))) -> list:
    """Batched uneven workload: the cells split (in whole groups of 32) across
    three synthetic mechanisms, T U[200, 310] K, p U[10, 1000] hPa, a solar
    phase U(-pi, pi) so that half the cells are in darkness (J = 0), dt = 60 s,
    rtol 1e-3, photolysis updated at every interval start."""
    groups = n_cells // 32
    share = [groups // len(sizes) + (1 if i < groups % len(sizes) else 0) for i in range(len(sizes))]
    out = []
    for i, ((n, R), g) in enumerate(zip(sizes, share)):
        sm = synthetic_mechanism(n, R, seed + 10 * i, third_body_fraction=0.1)
        cells = synthetic_cells(sm, g * 32, seed + 10 * i + 1000, T_range=(200.0, 310.0),
                                p_range_hpa=(10.0, 1000.0), phase_range=(-math.pi, math.pi))
        out.append(Workload(f"ros3-{n}x{R}", sm, cells, 60.0, intervals, 1.0e-3, 32, True))
    return out


@dataclass
class DaeWorkload(Workload):
    mass: np.ndarray = None          # (n,) 1 differential, 0 algebraic


def dae_constrained(n_cells: int = 16384, intervals: int = 120, seed: int = 5, n_diff: int = 150,
                    n_alg: int = 10, n_reactions: int = 330) -> DaeWorkload:
    """RODAS3 constrained workload: a synthetic mechanism of n_diff + n_alg
    species in which the last n_alg species are held in quasi-steady state
    (mass = 0, fastode/chem.py:112-113). Each of them gets a fast first-order
    loss (k = A with A log-uniform on [1e2, 1e4] s^-1, no temperature
    dependence) into two differential species, so its constraint row has a
    nonzero diagonal: fast equilibrium with its producers. T U[200, 310] K,
    p U[10, 1000] hPa, daylight phases U(-1.2, 1.2), dt = 60 s, rtol 1e-4."""
    n = n_diff + n_alg
    base = synthetic_mechanism(n, n_reactions, seed, third_body_fraction=0.1)
    rng = np.random.default_rng(seed + 77)
    species = base.species
    reactions = list(base.reactions)
    A = list(base.A)
    E = list(base.E)
    J = list(base.J)
    photo = list(base.photolytic)
    for a in range(n_diff, n):
        prods = rng.integers(0, n_diff, size=2)
        reactions.append(([species[a]], [(species[int(p)], 1.0) for p in prods]))
        A.append(10.0 ** rng.uniform(2.0, 4.0))
        E.append(0.0)
        J.append(0.0)
        photo.append(False)
    mech = Mechanism(species, reactions)
    sm = SyntheticMechanism(mech, species, reactions, np.array(A), np.array(E), np.array(J),
                            np.array(photo, dtype=bool))
    cells = synthetic_cells(sm, n_cells, seed + 1000, T_range=(200.0, 310.0), p_range_hpa=(10.0, 1000.0),
                            phase_range=(-1.2, 1.2))
    mass = np.ones(n)
    mass[n_diff:] = 0.0
    return DaeWorkload("rodas3-dae-%dx%d" % (n, len(reactions)), sm, cells, 60.0, intervals, 1.0e-4, 32, True,
                       mass=mass)


def photolysis_factors(cells: SyntheticCells, dt: float, intervals: int) -> np.ndarray:
    """(intervals, C) diurnal factors f of every interval start t = i * dt, as
    ``rate_constants`` computes them; photolysis column j of interval i is
    then J[j] * f[i] (one IEEE product, reproduced exactly on the device)."""
    return np.stack([diurnal_factor(cells, i * dt) for i in range(intervals)])


# The seeded parity subset of the 210/500, 65,536-cell workload: eight whole
# groups of 32 cells spread over the 2,048 groups. The reference is run on
# these groups (tests/golden/ros3_210x500_subset.npz) and the measured run is
# checked against it on the same groups.
PLAIN_LARGE_PARITY_GROUPS = (0, 292, 585, 877, 1170, 1462, 1755, 2047)


def plain_large(n_cells: int = 65536, intervals: int = 120, seed: int = 2) -> Workload:
    """Plain ROS3, 210 species / 500 reactions, 65,536 cells in groups of 32,
    T U[200, 310] K, p U[10, 1000] hPa setting [M], dt = 30 s x 120 intervals,
    rtol 1e-3, photolysis updated at every interval start."""
    sm = synthetic_mechanism(210, 500, seed, third_body_fraction=0.1)
    cells = synthetic_cells(sm, n_cells, seed + 1000, T_range=(200.0, 310.0),
                            p_range_hpa=(10.0, 1000.0), phase_range=(-1.2, 1.2))
    return Workload("ros3-210x500", sm, cells, 30.0, intervals, 1.0e-3, 32, True)
