"""Mass-action mechanisms and the chemistry system handed to the device integrator.

``Mechanism`` compiles a reaction list into the tables the reference builds in
fastode/chem.py:19-79 (same argument meaning, same table layout, same order of
Jacobian entries): the reactant index table ``react`` of shape (R, P) padded
with ``n`` (a column of ones), the stoichiometry ``S`` of shape (n, R), the
Jacobian pattern with the diagonal first, and the map from rate partials to
Jacobian values. The last is kept here as explicit term lists (entry, j, p,
coefficient) sorted as the reference's CSR map sums them.

``ChemSystem`` mirrors fastode/chem.py:111-134: a mechanism, rate constants k of
shape (C, R) and a mass vector (0 marks an algebraic, quasi-steady species).
Its ``rhs`` and ``jac`` run on the GPU through the C-ABI; there is no host
evaluation path.
"""
from __future__ import annotations

import numpy as np


class SparsePattern:
    """A fixed Jacobian sparsity pattern (rows, cols) that includes the diagonal
    (fastode/linalg.py:32-47)."""

    def __init__(self, n: int, rows, cols):
        self.n = n
        self.rows = np.asarray(rows, dtype=np.int64)
        self.cols = np.asarray(cols, dtype=np.int64)
        self.nnz = len(self.rows)
        where = {(int(r), int(c)): e for e, (r, c) in enumerate(zip(self.rows, self.cols))}
        self.diag = np.array([where[(i, i)] for i in range(n)], dtype=np.int64)


class Mechanism:
    def __init__(self, species, reactions, third_bodies=("M",)):
        """species: names of the state species; reactions: (reactants, products)
        pairs, reactants a list of names (repeats allowed, third bodies folded
        into k by the caller), products a list of (name, yield)."""
        self.species = list(species)
        n = self.n = len(self.species)
        index = {s: i for i, s in enumerate(self.species)}
        R = self.R = len(reactions)
        tb = set(third_bodies)
        self.third_body_power = np.zeros(R)
        lists = []
        for j, (reactants, _) in enumerate(reactions):
            kept = []
            for s in reactants:
                if s in tb:
                    self.third_body_power[j] += 1
                else:
                    kept.append(index[s])
            lists.append(kept)
        P = self.P = max(1, max((len(x) for x in lists), default=1))
        self.react = np.full((R, P), n, dtype=np.int64)
        for j, kept in enumerate(lists):
            self.react[j, : len(kept)] = kept
        S = np.zeros((n, R))
        for j, (_, products) in enumerate(reactions):
            for i in lists[j]:
                S[i, j] -= 1.0
            for s, y in products:
                if s not in tb:
                    S[index[s], j] += y
        self.S = S
        self.ST = np.ascontiguousarray(S.T)

        # Jacobian pattern: diagonal first, then entries in order of discovery
        # over reactions j, reactant slots p and species i with S[i, j] != 0.
        slot = {}
        rows, cols = [], []
        for i in range(n):
            slot[(i, i)] = i
            rows.append(i)
            cols.append(i)
        terms = []                                   # (entry, j*P+p, coefficient)
        for j in range(R):
            nz = np.nonzero(S[:, j])[0]
            for p in range(P):
                kk = int(self.react[j, p])
                if kk == n:
                    continue
                for i in nz:
                    key = (int(i), kk)
                    e = slot.get(key)
                    if e is None:
                        e = slot[key] = len(rows)
                        rows.append(int(i))
                        cols.append(kk)
                    terms.append((e, j * P + p, float(S[i, j])))
        self.pattern = SparsePattern(n, rows, cols)
        # the reference sums each Jacobian entry over its (j, p) columns in
        # ascending order (a CSR map); identical (entry, jp) pairs cannot occur
        terms.sort(key=lambda t: (t[0], t[1]))
        self.jac_terms = np.array([(t[0], t[1]) for t in terms], dtype=np.int64).reshape(-1, 2)
        self.jac_coef = np.array([t[2] for t in terms], dtype=np.float64)

    # -- tables for the C-ABI ------------------------------------------------
    def stoich_csr(self):
        """S by species rows: (indptr (n+1), reaction index, coefficient)."""
        indptr = [0]
        idx, val = [], []
        for i in range(self.n):
            nz = np.nonzero(self.S[i])[0]
            idx.extend(int(j) for j in nz)
            val.extend(float(self.S[i, j]) for j in nz)
            indptr.append(len(idx))
        return (np.array(indptr, dtype=np.int32), np.array(idx, dtype=np.int32),
                np.array(val, dtype=np.float64))

    def jac_csr(self):
        """Jacobian-value map by entry: (indptr (nnz+1), j*P+p, coefficient)."""
        e = self.jac_terms[:, 0] if len(self.jac_terms) else np.zeros(0, dtype=np.int64)
        counts = np.bincount(e, minlength=self.pattern.nnz)
        indptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.int32)
        jp = self.jac_terms[:, 1].astype(np.int32) if len(self.jac_terms) else np.zeros(0, np.int32)
        return indptr, jp, self.jac_coef.copy()

    def dense_jacobian(self, vals):
        vals = np.asarray(vals)
        J = np.zeros((vals.shape[0], self.n, self.n))
        J[:, self.pattern.rows, self.pattern.cols] = vals
        return J


def mechanism_tables(mech):
    """Duck-typed view of a mechanism: accepts this package's ``Mechanism`` or
    the reference's (fastode/chem.py:19-79), whose GT map is a scipy CSR matrix."""
    n, R, P = int(mech.n), int(mech.R), int(mech.P)
    react = np.ascontiguousarray(np.asarray(mech.react, dtype=np.int64))
    S = np.asarray(mech.S, dtype=np.float64)
    rows = np.asarray(mech.pattern.rows, dtype=np.int64)
    cols = np.asarray(mech.pattern.cols, dtype=np.int64)
    if hasattr(mech, "jac_csr"):
        j_indptr, j_idx, j_val = mech.jac_csr()
    else:
        GT = mech.GT.tocsr()
        GT.sort_indices()
        j_indptr = GT.indptr.astype(np.int32)
        j_idx = GT.indices.astype(np.int32)
        j_val = GT.data.astype(np.float64)
    s_indptr = [0]
    s_idx, s_val = [], []
    for i in range(n):
        nz = np.nonzero(S[i])[0]
        s_idx.extend(int(j) for j in nz)
        s_val.extend(float(S[i, j]) for j in nz)
        s_indptr.append(len(s_idx))
    return dict(n=n, R=R, P=P, react=react, rows=rows, cols=cols,
                s_indptr=np.array(s_indptr, np.int32), s_idx=np.array(s_idx, np.int32),
                s_val=np.array(s_val, np.float64),
                j_indptr=np.ascontiguousarray(j_indptr, dtype=np.int32),
                j_idx=np.ascontiguousarray(j_idx, dtype=np.int32),
                j_val=np.ascontiguousarray(j_val, dtype=np.float64))


class ChemSystem:
    """A mechanism with rate constants k (C, R) and mass (n,); mass[i] = 0 holds
    species i in quasi-steady state (fastode/chem.py:111-121)."""

    def __init__(self, mech, k, mass=None, dense=None):
        self.mech = mech
        self.k = np.atleast_2d(np.asarray(k, dtype=np.float64))
        self.n = mech.n
        self.names = list(getattr(mech, "species", [f"y{i}" for i in range(mech.n)]))
        self.mass = np.ones(self.n) if mass is None else np.asarray(mass, dtype=float)
        self.dense = (self.n <= 60) if dense is None else dense

    @property
    def has_constraints(self) -> bool:
        return bool(np.any(self.mass == 0.0))

    def rhs(self, Y):
        """Forcing F(Y) of shape (C, n), evaluated on the GPU."""
        from .solvers import device_rhs
        return device_rhs(self, Y)

    def jac(self, Y):
        """Jacobian values (C, nnz) on the pattern, or dense (C, n, n) when
        ``dense``; evaluated on the GPU."""
        from .solvers import device_jac
        vals = device_jac(self, Y)
        return self.mech.dense_jacobian(vals) if self.dense else vals
