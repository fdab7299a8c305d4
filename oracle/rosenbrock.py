"""NumPy/SciPy restatement of the reference integrator (test infrastructure).

Each function names the reference code it restates. Where the device must
reproduce the reference bit for bit (the step rules, the controller) the
expressions are kept operation for operation; the linear algebra calls the
same SciPy routines the reference calls (LAPACK getrf/getrs per cell for
n <= 60, SuperLU on the block-diagonal group matrix otherwise), so the oracle's
timings and its roundoff are the reference's.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, fields

import numpy as np
import scipy.linalg as sla
import scipy.sparse as sp
import scipy.sparse.linalg as spla

ROUND_OFF = float(np.finfo(float).eps)
H_MIN_FRACTION = 1.0e-15
H_START_FRACTION = 1.0e-6
ERROR_MIN = 1.0e-10


# ---- counters, memory (fastode/counts.py:10-30, solvers.py:181-186) ----------------

@dataclass
class OCounts:
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

    def add(self, o):
        for f in fields(self):
            setattr(self, f.name, getattr(self, f.name) + getattr(o, f.name))

    def as_tuple(self):
        return tuple(getattr(self, f.name) for f in fields(self))


@dataclass
class OMemory:
    h_next: float = 0.0
    err_prev: float = 0.0
    h_prev: float = 0.0


# ---- tableaus (fastode/tableaus.py:15-90) --------------------------------------------

def _lower(S, flat):
    out = np.zeros((S, S))
    it = iter(flat)
    for r in range(1, S):
        for s in range(r):
            out[r, s] = next(it)
    return out


@dataclass(frozen=True)
class OTableau:
    name: str
    gamma: float
    a: np.ndarray
    c: np.ndarray
    m: np.ndarray
    e: np.ndarray
    embedded: int

    @property
    def stages(self):
        return len(self.m)

    @property
    def k(self):
        return float(self.embedded + 1)

    @property
    def new_forcing(self):
        flags = [True]
        for r in range(1, self.stages):
            prev = np.concatenate([self.a[r - 1, : r - 1], [0.0]])
            flags.append(not (np.array_equal(self.a[r, :r], prev) and self.a[r, r - 1] == 0.0))
        return flags


OROS3 = OTableau("ros3", 0.43586652150845899941601945119356,
                 _lower(3, [1.0, 1.0, 0.0]),
                 _lower(3, [-0.10156171083877702091975600115545e01, 0.40759956452537699824805835358067e01,
                            0.92076794298330791242156818474003e01]),
                 np.array([1.0, 0.61697947043828245592553615689730e01, -0.42772256543218573326238373806514]),
                 np.array([0.5, -0.29079558716805469821718236208017e01, 0.22354069897811569627360909276199]),
                 2)
ORODAS3 = OTableau("rodas3", 0.5, _lower(4, [0.0, 2.0, 0.0, 2.0, 0.0, 1.0]),
                   _lower(4, [4.0, 1.0, -1.0, 1.0, -1.0, -8.0 / 3.0]),
                   np.array([2.0, 0.0, 1.0, 1.0]), np.array([0.0, 0.0, 0.0, 1.0]), 2)
OTABLEAUS = {"ros3": OROS3, "rodas3": ORODAS3}


# ---- chemistry system (fastode/chem.py:81-134, linalg.py:15-81) ---------------------

class OChem:
    """A group's chemistry: the mechanism tables (react, S, pattern rows/cols
    with the diagonal first, GT map) with rate constants k (C or 1, R) and mass."""

    def __init__(self, mech, k, mass=None, dense=None):
        self.n = int(mech.n)
        self.react = np.asarray(mech.react)
        self.ST = np.ascontiguousarray(np.asarray(mech.S).T)
        self.P = int(mech.P)
        self.rows = np.asarray(mech.pattern.rows, dtype=np.int64)
        self.cols = np.asarray(mech.pattern.cols, dtype=np.int64)
        self.nnz = len(self.rows)
        if hasattr(mech, "GT"):
            self.GT = mech.GT
        else:
            ind, idx, val = mech.jac_csr()
            self.GT = sp.csr_matrix((val, idx, ind), shape=(self.nnz, int(mech.R) * self.P))
        where = {(int(r), int(c)): e for e, (r, c) in enumerate(zip(self.rows, self.cols))}
        self.diag = np.array([where[(i, i)] for i in range(self.n)], dtype=np.int64)
        self.order = np.lexsort((self.rows, self.cols))
        cnt = np.bincount(self.cols, minlength=self.n)
        self.block_indices = self.rows[self.order]
        self.block_indptr = np.concatenate([[0], np.cumsum(cnt)])
        k = np.atleast_2d(np.asarray(k))
        self.k = k if np.iscomplexobj(k) else k.astype(np.float64)     # complex: complex-step tangents
        self.mass = np.ones(self.n) if mass is None else np.asarray(mass, dtype=float)
        self.dense = (self.n <= 60) if dense is None else dense

    @property
    def has_constraints(self):
        return bool(np.any(self.mass == 0.0))

    def _gather(self, Y):
        Yp = np.concatenate([Y, np.ones((Y.shape[0], 1))], axis=1)
        return Yp[:, self.react]

    def rates(self, Y):                            # chem.py:86-87
        return self.k * self._gather(Y).prod(axis=2)

    def rhs(self, Y):                              # chem.py:89-90
        return self.rates(Y) @ self.ST

    def jac_values(self, Y):                       # chem.py:92-102
        X = self._gather(Y)
        C = X.shape[0]
        d = np.empty_like(X)
        for p in range(self.P):
            prod = self.k.copy() if self.k.ndim == 2 else np.broadcast_to(self.k, X.shape[:2]).copy()
            prod = np.broadcast_to(prod, X.shape[:2]).copy()
            for q in range(self.P):
                if q != p:
                    prod *= X[:, :, q]
            d[:, :, p] = prod
        return np.asarray((self.GT @ d.reshape(C, -1).T).T)

    def jac(self, Y):                              # chem.py:126-128
        vals = self.jac_values(Y)
        if not self.dense:
            return vals
        J = np.zeros((vals.shape[0], self.n, self.n), dtype=vals.dtype)
        J[:, self.rows, self.cols] = vals
        return J

    def factor(self, alpha, J, algebraic_rows_only=False):   # chem.py:130-134
        if self.dense:
            if algebraic_rows_only:
                J = J * (self.mass == 0.0)[None, :, None]
            A = -J.copy()
            idx = np.arange(J.shape[1])
            A[:, idx, idx] += alpha * self.mass
            return _DenseLU(A)
        vals = -J
        if algebraic_rows_only:
            vals = vals * (self.mass[self.rows] == 0.0)[None, :]
        else:
            vals = vals.copy()
        vals[:, self.diag] += alpha * self.mass[None, :]
        return _SparseLU(self, vals)


class _DenseLU:                                    # linalg.py:15-22
    def __init__(self, A):
        self.f = [sla.lu_factor(A[c], check_finite=False) for c in range(A.shape[0])]

    def solve(self, B):
        return np.stack([sla.lu_solve(f, B[c], check_finite=False) for c, f in enumerate(self.f)])


class _SparseLU:                                   # linalg.py:70-81
    def __init__(self, sysm: OChem, vals):
        C = vals.shape[0]
        n, nnz = sysm.n, sysm.nnz
        indices = np.concatenate([sysm.block_indices + c * n for c in range(C)])
        indptr = np.concatenate([sysm.block_indptr[:-1] + c * nnz for c in range(C)] + [[C * nnz]])
        data = vals[:, sysm.order].ravel()
        A = sp.csc_matrix((data, indices, indptr), shape=(n * C, n * C))
        self.lu = spla.splu(A, permc_spec="MMD_AT_PLUS_A")
        self.shape = (C, n)

    def solve(self, B):
        return self.lu.solve(np.ascontiguousarray(B).ravel()).reshape(self.shape)


# ---- the integrator (fastode/solvers.py:37-178, 270-415) -----------------------------

def error_norm(Y, Ynew, E, atol, rtol):           # solvers.py:37-43
    ymax = np.maximum(np.abs(Y), np.abs(Ynew))
    s = E / (atol[None, :] + rtol * ymax)
    value = math.sqrt(float(np.sum(s * s)) / s.size)
    return max(value, ERROR_MIN) if not math.isnan(value) else value


def quantize(h, interval):                         # solvers.py:46-51
    if h >= interval:
        return interval
    q = math.ceil(interval / h - 1.0e-9)
    return interval / max(q, 1)


def stages(system, tab, Y, F0, LU, H, counts):     # solvers.py:54-86
    dae = system.has_constraints
    K = []
    forcing = None
    for r in range(tab.stages):
        if r == 0:
            forcing = F0
        elif tab.new_forcing[r]:
            Yr = Y.copy()
            for s in range(r):
                if tab.a[r, s] != 0.0:
                    Yr += tab.a[r, s] * K[s]
            forcing = system.rhs(Yr)
            counts.rhs += 1
        rhs = forcing.copy()
        for s in range(r):
            coef = tab.c[r, s] / H
            if coef != 0.0:
                rhs += coef * (K[s] * system.mass[None, :] if dae else K[s])
        K.append(LU.solve(rhs))
        counts.solves += 1
    Ynew = Y.copy()
    E = np.zeros_like(Y)
    for r in range(tab.stages):
        if tab.m[r] != 0.0:
            Ynew += tab.m[r] * K[r]
        if tab.e[r] != 0.0:
            E += tab.e[r] * K[r]
    return Ynew, E


def clamp(system, Y):                              # solvers.py:89-97
    if system.has_constraints:
        diff = system.mass == 1.0
        Y[:, diff] = np.maximum(Y[:, diff], 0.0)
    else:
        np.maximum(Y, 0.0, out=Y)
    return Y


def project(system, Y, atol, rtol, counts, max_updates=10, tol=0.1, max_backtracks=24,
            backtrack_factor=0.5, sigma=1.0e-4):   # solvers.py:100-178
    alg = system.mass == 0.0
    if not np.any(alg):
        return Y, "converged"
    atol_a = atol[alg]

    def residual(Z):
        G = system.rhs(Z)
        counts.rhs += 1
        G[:, ~alg] = 0.0
        return G

    def finite(A):
        return bool(np.all(np.isfinite(A[:, alg])))

    def weighted(Z, D):
        z, d = Z[:, alg], D[:, alg]
        scale = atol_a[None, :] + rtol * np.maximum(np.abs(z), np.abs(z + d))
        with np.errstate(divide="ignore", invalid="ignore"):
            q = np.where(scale > 0.0, np.abs(d) / scale, np.where(d == 0.0, 0.0, np.inf))
        return float(q.max())

    original = None
    for update in range(max_updates + 1):
        G = residual(Y)
        if not finite(G):
            break
        counts.proj_passes += 1
        if float(np.abs(G[:, alg]).max()) == 0.0:
            return Y, "converged"
        J = system.jac(Y)
        counts.jac += 1
        LU = system.factor(1.0, J, algebraic_rows_only=True)
        counts.lu += 1
        delta = LU.solve(G)
        counts.solves += 1
        if not finite(delta):
            break
        q = weighted(Y, delta)
        if q <= tol:
            return Y, "converged"
        if update == max_updates:
            break
        if original is None:
            original = Y.copy()
        step = 1.0
        accepted = None
        for _ in range(max_backtracks + 1):
            candidate = Y.copy()
            candidate[:, alg] += step * delta[:, alg]
            step_used = step
            step *= backtrack_factor
            if not finite(candidate):
                continue
            Gc = residual(candidate)
            counts.proj_trials += 1
            if not finite(Gc):
                continue
            if float(np.abs(Gc[:, alg]).max()) == 0.0:
                accepted = candidate
                break
            trial = LU.solve(Gc)
            counts.solves += 1
            if not finite(trial):
                continue
            qt = weighted(candidate, trial)
            if qt <= tol or qt < (1.0 - sigma * step_used) * q:
                accepted = candidate
                break
        if accepted is None:
            break
        Y = accepted
    if original is not None:
        Y = original
    return Y, "projection failed"


@dataclass
class OAlgorithm:
    tableau: OTableau = OROS3
    controller: str = "h211b"
    b: float = 4.0
    safety: float = 0.9
    fac_min: float = 0.2
    fac_max: float = 6.0
    carry: bool = True
    quantize: bool = True
    max_steps: int = 1000
    carry_memory: bool = True
    trace: list = field(default=None)    # when a list: (t, H, err, outcome) per attempt

    def factor(self, err, H, mem):                 # solvers.py:297-303
        k = self.tableau.k
        fac = self.safety / err ** (1.0 / k)
        if self.controller == "h211b" and mem.err_prev > 0.0 and mem.h_prev > 0.0:
            fac = (self.safety * (err * mem.err_prev) ** (-1.0 / (self.b * k))
                   * (H / mem.h_prev) ** (-1.0 / self.b))
        return min(self.fac_max, max(self.fac_min, fac))

    def _rec(self, t, H, err, outcome):
        if self.trace is not None:
            self.trace.append((t, H, err, outcome))

    def solve(self, system, Y, dt, atol, rtol, counts, memory=None):   # solvers.py:305-415
        tab = self.tableau
        mem = memory if memory is not None else OMemory()
        if not (self.carry and self.carry_memory):
            mem.err_prev = mem.h_prev = 0.0
        counts.calls += 1
        h_min = H_MIN_FRACTION * dt
        h_max = dt
        H = mem.h_next if (self.carry and mem.h_next > 0.0) else H_START_FRACTION * dt
        H = min(max(h_min, H), h_max)
        if self.quantize:
            H = quantize(H, dt)
        proposed = H
        Y = Y.copy()
        if system.has_constraints:
            Y, status = project(system, Y, atol, rtol, counts)
            if status != "converged":
                return Y, status
        t = 0.0
        reject_last = reject_more = False
        nsteps = 0
        status = "running"
        while (t - dt + ROUND_OFF) <= 0.0 and status == "running":
            if nsteps >= self.max_steps:
                status = "too many steps"
                break
            if (t + 0.1 * H == t) or H < h_min:
                status = "step too small"
                break
            last = dt - t <= H * (1.0 + 1.0e-8)
            shortened = last and dt - t < H * (1.0 - 1.0e-8)
            H_ctrl = H
            if last:
                H = dt - t
            F0 = system.rhs(Y)
            counts.rhs += 1
            J = system.jac(Y)
            counts.jac += 1
            accepted = False
            while not accepted:
                if nsteps >= self.max_steps:
                    status = "too many steps"
                    break
                if H < h_min or t + 0.1 * H == t:
                    status = "step too small"
                    break
                LU = system.factor(1.0 / (H * tab.gamma), J)
                counts.lu += 1
                Ynew, E = stages(system, tab, Y, F0, LU, H, counts)
                err = error_norm(Y, Ynew, E, atol, rtol)
                nsteps += 1
                counts.steps += 1
                if math.isnan(err) or math.isinf(err):
                    self._rec(t, H, err, -1)
                    status = "nan or inf"
                    break
                if err < 1.0 and shortened:
                    self._rec(t, H, err, 1)
                    counts.accepted += 1
                    t = dt
                    Y = Ynew
                    proposed = H_ctrl
                    accepted = True
                elif err < 1.0:
                    self._rec(t, H, err, 1)
                    fac = self.factor(err, H, mem)
                    counts.accepted += 1
                    t = dt if last else t + H
                    Y = Ynew
                    mem.err_prev = err
                    mem.h_prev = H
                    Hnew = H * fac
                    if reject_last:
                        Hnew = min(Hnew, H)
                    Hnew = max(h_min, min(Hnew, h_max))
                    if self.quantize:
                        Hnew = quantize(Hnew, dt)
                    reject_last = reject_more = False
                    proposed = Hnew
                    H = Hnew
                    accepted = True
                else:
                    self._rec(t, H, err, 0)
                    Hnew = H * max(self.fac_min, self.safety / err ** (1.0 / tab.k))
                    if reject_more:
                        Hnew = H * 0.1
                    reject_more = reject_last
                    reject_last = True
                    if self.quantize:
                        Hnew = quantize(Hnew, dt)
                    H = Hnew
                    last = dt - t <= H * (1.0 + 1.0e-8)
                    shortened = last and dt - t < H * (1.0 - 1.0e-8)
                    H_ctrl = H
                    if last:
                        H = dt - t
                    counts.rejected += 1
        mem.h_next = proposed
        if status == "running":
            status = "converged"
        return clamp(system, Y), status


@dataclass
class OBackwardEuler:
    """fastode/solvers.py:418-491, statement by statement."""
    max_iterations: int = 11
    reductions: tuple = (0.5, 0.5, 0.5, 0.5, 0.1)
    small: float = 1.0e-40

    def new_memory(self):
        return None

    def converged(self, delta, Y, atol, rtol):     # solvers.py:432-437
        if not np.all(np.isfinite(delta)):
            return False
        bound = np.maximum(np.maximum(self.small, atol[None, :]), rtol * np.abs(Y))
        return bool(np.all(np.abs(delta) <= bound))

    def solve(self, system, Y, dt, atol, rtol, counts, memory=None):   # solvers.py:439-491
        counts.calls += 1
        H = dt
        t = 0.0
        n_success = n_fail = 0
        Yn = Y.copy()
        Yn1 = Y.copy()
        status = "converged"
        while t < dt:
            ok = False
            iterations = 0
            while True:
                counts.newton += 1
                F = system.rhs(Yn1)
                counts.rhs += 1
                J = system.jac(Yn1)
                counts.jac += 1
                LU = system.factor(1.0 / H, J)
                counts.lu += 1
                delta = LU.solve(F - (Yn1 - Yn) / H)
                counts.solves += 1
                Yn1 = np.maximum(Yn1 + delta, 0.0)
                iterations += 1
                if iterations > 1:
                    ok = self.converged(delta, Yn1, atol, rtol)
                if ok or iterations >= self.max_iterations:
                    break
            counts.steps += 1
            if not ok:
                counts.rejected += 1
                counts.failures += 1
                n_success = 0
                if n_fail >= len(self.reductions):
                    t += H
                    counts.unconverged += 1
                    status = "accepted unconverged"
                    if not np.all(np.isfinite(Yn1)):
                        status = "nan or inf"
                    break
                Yn1 = Yn.copy()
                H *= self.reductions[n_fail]
                n_fail += 1
            else:
                counts.accepted += 1
                t += H
                Yn = Yn1.copy()
                n_success += 1
                if n_success >= 2:
                    n_success = 0
                    H *= 2.0
            H = min(H, dt - t)
        return clamp(system, Yn1), status


def fixed_steps(system, tab, Y, t_end, n_steps, counts=None):   # solvers.py:494-504
    counts = counts or OCounts()
    H = t_end / n_steps
    for _ in range(n_steps):
        F0 = system.rhs(Y)
        J = system.jac(Y)
        LU = system.factor(1.0 / (H * tab.gamma), J)
        Y, _ = stages(system, tab, Y, F0, LU, H, counts)
    return Y


# ---- a scenario loop over groups and intervals (fastode/ts1.py:181-223 pattern) -------

def run_groups(mech, Y0, k_at, dt, intervals, atol, rtol, group_size=32, tableau=OROS3,
               mass=None, groups=None, trace=False, solver=None, **alg_kw):
    """Integrate the cells of Y0 (C, n) in groups over `intervals` intervals,
    each group with its own memory; k_at(i) gives the (C, R) rate constants of
    interval i. `solver`, when given, makes each group's solver (for example
    OBackwardEuler); the default is OAlgorithm(tableau, **alg_kw). Returns (Y,
    counts per group, statuses per group and interval, memory per group,
    traces per group)."""
    C = Y0.shape[0]
    starts = list(range(0, C, group_size))
    if groups is not None:
        starts = [starts[g] for g in groups]
    Y = Y0.copy()
    counts, statuses, memories, traces = [], [], [], []
    ks = [k_at(i) for i in range(intervals)]
    for g0 in starts:
        sl = slice(g0, min(g0 + group_size, C))
        alg = solver() if solver is not None else OAlgorithm(tableau=tableau, trace=[] if trace else None, **alg_kw)
        mem = alg.new_memory() if solver is not None else OMemory()
        c = OCounts()
        st = []
        Yg = Y[sl].copy()
        for i in range(intervals):
            system = OChem(mech, ks[i][sl], mass=mass)
            Yg, s = alg.solve(system, Yg, dt, atol, rtol, c, mem)
            st.append(s)
        Y[sl] = Yg
        counts.append(c)
        statuses.append(st)
        memories.append(mem)
        traces.append(getattr(alg, "trace", None))
    return Y, counts, statuses, memories, traces


# ---- the fixed-step map and its tangent (checks the device adjoint) ----------------

def replay_interval(system, tab, Y, steps):
    """The given step sizes in order with no error control (the accepted
    steps of a forward call, held fixed; fastode/solvers.py:494-504 with
    per-step sizes), then the clamp of fastode/solvers.py:89-97 written with a
    mask so that complex (complex-step) states pass through it."""
    for h in steps:
        F0 = system.rhs(Y)
        J = system.jac(Y)
        LU = system.factor(1.0 / (h * tab.gamma), J)
        Y, _ = stages(system, tab, Y, F0, LU, h, OCounts())
    keep = np.real(Y) > 0.0
    if system.has_constraints:
        keep = keep | (system.mass != 1.0)[None, :]
    return np.where(keep, Y, 0.0)


def replay_projection(system, Y, steps):
    """The projection's accepted Newton updates of one call with their
    line-search steps held fixed (solvers.py:110-160 without the decisions):
    Y_alg += step * (M - J)_alg^-1 G(Y), G the forcing on the algebraic rows."""
    alg = system.mass == 0.0
    for step in steps:
        G = system.rhs(Y)
        G[:, ~alg] = 0.0
        LU = system.factor(1.0, system.jac(Y), algebraic_rows_only=True)
        delta = LU.solve(G)
        Y = Y.copy()
        Y[:, alg] += step * delta[:, alg]
    return Y


def tangent_linear(mech, Y0, dY0, k_list, dlogk, steps_list, tab=None, mass=None, eps=1e-30, proj_list=None):
    """Directional derivative of the fixed-step map over all intervals in
    direction (dY0, dlogk) by the complex step: exact to roundoff, because the
    map is analytic in its inputs away from the clamp's kink. k_list[i] is
    (C, R); steps_list[i] is the list of step sizes of interval i; with
    constraints, proj_list[i] the line-search steps of the projection updates
    that start interval i."""
    tab = tab or OROS3
    Y = Y0.astype(np.complex128) + 1j * eps * dY0
    scale = np.exp(1j * eps * np.asarray(dlogk))[None, :]
    for i, (k, steps) in enumerate(zip(k_list, steps_list)):
        system = OChem(mech, k.astype(np.complex128) * scale, mass=mass, dense=True)
        if proj_list is not None:
            Y = replay_projection(system, Y, proj_list[i])
        Y = replay_interval(system, tab, Y, steps)
    return np.imag(Y) / eps, np.real(Y)
