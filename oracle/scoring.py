"""NumPy restatement of the reference's accuracy scores (test infrastructure).

``score`` restates fastode/ts1.py:226-264 (Sandu digits overall and per
species against a reference table, plus the sign/finiteness gate) and
``digits`` restates fastode/reference.py:41-59. ``read_csv_table`` restates
fastode/ts1.py:106-111. The accumulation order is the reference's, so the
oracle's digits are the reference's to the last bit.
"""
from __future__ import annotations

import csv
import math

import numpy as np


def read_csv_table(path):                                      # ts1.py:106-111
    with open(path, newline="") as f:
        reader = csv.reader(f)
        header = next(reader)
        rows = [[float(v) for v in row] for row in reader if row]
    return header, np.array(rows)


def _digits_of(values):
    if not values:
        return float("nan")
    ms = float(np.mean(values))
    return 16.0 if ms <= 0.0 else min(16.0, -math.log10(math.sqrt(ms)))


def score_table(result, cells_index, species, header, rows, threshold=1e-14):   # ts1.py:226-264
    """score() on an already-read table (header, rows)."""
    keyed = header[:2] == ["step", "cell"]
    start = 4 if keyed else 2
    ref_species = header[start:]
    col = {s: start + i for i, s in enumerate(ref_species)}
    sp_index = {s: i for i, s in enumerate(species)}
    want = list(cells_index)
    pos = {c: i for i, c in enumerate(want)}
    sq_by_species = {s: [] for s in ref_species}
    gate = True
    for step, Y in result.items():
        if not np.all(np.isfinite(Y)) or np.any(Y < -1e-20):
            gate = False
        if keyed:
            sel = rows[(rows[:, 0] == step) & np.isin(rows[:, 1], want)]
            pairs = [(Y[pos[int(row[1])]], row) for row in sel]
        else:
            pairs = [(Y[i], rows[c]) for i, c in enumerate(want)]
        for y_cell, row in pairs:
            for s in ref_species:
                ref = row[col[s]]
                if ref < threshold or s not in sp_index:
                    continue
                y = y_cell[sp_index[s]]
                sq_by_species[s].append(((y - ref) / ref) ** 2)
    all_sq = [v for vs in sq_by_species.values() for v in vs]
    per = {s: _digits_of(v) for s, v in sq_by_species.items() if v}
    return _digits_of(all_sq), per, gate


def score(result, cells_index, species, reference_path, threshold=1e-14):
    header, rows = read_csv_table(reference_path)
    return score_table(result, cells_index, species, header, rows, threshold)


def digits(result, reference, threshold, columns=None):           # reference.py:41-59
    R = np.asarray(reference)
    X = np.asarray(result)
    cols = range(R.shape[1]) if columns is None else columns
    per = {}
    all_sq = []
    for j in cols:
        mask = R[:, j] >= threshold
        if not np.any(mask):
            continue
        sq = ((X[mask, j] - R[mask, j]) / R[mask, j]) ** 2
        all_sq.extend(sq.tolist())
        ms = float(np.mean(sq))
        per[j] = 16.0 if ms <= 0.0 else min(16.0, -math.log10(math.sqrt(ms)))
    ms = float(np.mean(all_sq)) if all_sq else float("nan")
    overall = 16.0 if ms <= 0.0 else min(16.0, -math.log10(math.sqrt(ms)))
    return overall, per


def levels(overall, per, gate):                      # experiments/ts1_experiments.py:103-105
    """(worst species, its digits, level 2, level 3) of an archived run row."""
    worst = sorted(per.items(), key=lambda kv: kv[1])
    ws, wd = worst[0] if worst else ("", float("nan"))
    level = lambda L: bool(gate and overall >= L and wd >= L - 1)  # noqa: E731
    return ws, wd, level(2), level(3)
