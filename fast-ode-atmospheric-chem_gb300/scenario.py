"""The reference's scenario driver and accuracy scores, device-resident.

``run_scenario`` has the signature and results of fastode.ts1.run_scenario
(fastode/ts1.py:181-223): it takes the reference's own ``Scenario``, ``Cells``
and ``TS1`` objects (or anything with the same attributes) and returns
(snapshots, counts, statuses). Where the reference integrates one group after
the other, here every group of the scenario advances in one ``fo_solve``
launch per interval; groups never exchange data, so the results per group are
the same. The rate constants of the first interval are evaluated on the
device from the mechanism's rate laws (``rate_law_table``, ``fo_rate_laws``:
Arrhenius, Troe, user-defined and surface rows and the third-body fold of
fastode/ts1.py:66-103; a mechanism object without reaction records uses its
own ``rate_constants``), the per-interval photolysis columns are patched on
the device (``fo_scale_photolysis``), and snapshots are copies of the device
state.

``score`` and ``digits`` are fastode.ts1.score (fastode/ts1.py:226-264) and
fastode.reference.digits (fastode/reference.py:41-59): the reference table is
read on the host, and the squared relative errors and the gate are reduced on
the device (``fo_score_accumulate``).
"""
from __future__ import annotations

import csv
import ctypes as C
import math

import numpy as np

from . import _abi
from .batch import Batch


def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("fastode_gb300 needs a CUDA GPU: there is no host integrator")
    return torch


def read_csv_table(path):
    """(header, rows) of a numeric CSV table (fastode/ts1.py:106-111)."""
    with open(path, newline="") as f:
        reader = csv.reader(f)
        header = next(reader)
        rows = [[float(v) for v in row] for row in reader if row]
    return header, np.array(rows)


class _Photolysis:
    """The photolysis columns of a scenario's cells on the device: for each
    reaction j of ts1.photolysis_reactions, k[:, j] = (base * f) * scaling
    when its parameter is scaled by the scenario factor (names starting with
    "j", fastode/ts1.py:194, 204-206), base * scaling otherwise."""

    def __init__(self, ts1, cells, photolysis, dev):
        torch = _torch()
        groups = {True: [], False: []}
        for j in ts1.photolysis_reactions:
            r = ts1.reactions[j]
            name = r["MUSICA name"]
            groups[name in photolysis].append((j, np.asarray(cells.params[name], dtype=np.float64),
                                               float(r.get("scaling factor", 1.0))))
        self.parts = {}
        for scaled, entries in groups.items():
            if not entries:
                continue
            rxn = torch.tensor([e[0] for e in entries], dtype=torch.int32, device=dev)
            base = torch.from_numpy(np.ascontiguousarray(np.stack([e[1] for e in entries]))).to(dev)
            scaling = torch.tensor([e[2] for e in entries], dtype=torch.float64, device=dev)
            self.parts[scaled] = (rxn, base, scaling)

    def patch(self, k, C_cells: int, factor: float, stream) -> None:
        for scaled, (rxn, base, scaling) in self.parts.items():
            rc = _abi.lib().fo_scale_photolysis(C_cells, rxn.numel(), rxn.data_ptr(), base.data_ptr(),
                                                scaling.data_ptr(), float(factor) if scaled else 1.0,
                                                k.data_ptr(), 1, C_cells, C.c_void_p(stream.cuda_stream))
            _abi.check(rc, "fo_scale_photolysis")


RATE_DTYPE = np.dtype([("type", np.int32), ("column", np.int32), ("c", np.float64, (8,))])
BOLTZMANN = 1.380649e-23
AVOGADRO = 6.02214076e23
R_GAS = BOLTZMANN * AVOGADRO


def rate_law_table(ts1):
    """The rate laws of a TS1-style mechanism as fo_rate_law records, compiled
    from its reaction records (the keys and defaults fastode/ts1.py:72-98
    reads), and the names of the per-cell parameters they read, in column
    order. None when a reaction has a type the device does not evaluate."""
    laws = np.zeros(len(ts1.reactions), dtype=RATE_DTYPE)
    columns = []

    def column(name):
        if name not in columns:
            columns.append(name)
        return columns.index(name)

    for j, r in enumerate(ts1.reactions):
        t = r.get("type")
        c = np.zeros(8)
        col = -1
        if t == "ARRHENIUS":
            code = _abi.RATE_ARRHENIUS
            c[:5] = [r.get("A", 1.0), r.get("B", 0.0), r.get("C", 0.0), r.get("D", 300.0), r.get("E", 0.0)]
        elif t == "TROE":
            code = _abi.RATE_TROE
            c[:] = [r.get("k0_A", 1.0), r.get("k0_B", 0.0), r.get("k0_C", 0.0), r.get("kinf_A", 1.0),
                    r.get("kinf_B", 0.0), r.get("kinf_C", 0.0), r.get("Fc", 0.6), r.get("N", 1.0)]
        elif t == "USER_DEFINED":
            code = _abi.RATE_USER
            col = column(r["MUSICA name"])
            c[0] = r.get("scaling factor", 1.0)
        elif t == "SURFACE":
            code = _abi.RATE_SURFACE
            label = r["MUSICA name"]
            col = column(label + ".effective radius [m]")
            nxt = label + ".particle number concentration [# m-3]"
            if nxt in columns or col != len(columns) - 1:
                return None
            columns.append(nxt)
            sp = ts1.props[r["gas-phase reactant"]]
            c[0] = 8.0 * R_GAS / (math.pi * sp["molecular weight [kg mol-1]"])
            c[1] = sp["diffusion coefficient [m2 s-1]"]
            c[2] = r.get("reaction probability", 1.0)
        else:
            return None
        laws[j] = (code, col, c)
    return laws, columns


def device_rate_constants(ts1, T, P, params, dev, stream, table=None):
    """(R, C) rate constants, cells fastest, evaluated on the device by
    fo_rate_laws: fastode.ts1.TS1.rate_constants(T, P, params)
    (fastode/ts1.py:66-103) without the host loop."""
    torch = _torch()
    laws, columns = table if table is not None else rate_law_table(ts1)
    T = np.ascontiguousarray(T, dtype=np.float64)
    C_cells, R = len(T), len(laws)
    d_laws = torch.from_numpy(np.frombuffer(laws.tobytes(), dtype=np.uint8).copy()).to(dev)
    d_T = torch.from_numpy(T).to(dev)
    d_P = torch.from_numpy(np.ascontiguousarray(P, dtype=np.float64)).to(dev)
    mat = np.stack([np.asarray(params[nm], dtype=np.float64) for nm in columns]) if columns else np.zeros((1, C_cells))
    d_par = torch.from_numpy(np.ascontiguousarray(mat)).to(dev)
    power = np.asarray(ts1.mech.third_body_power, dtype=np.float64)
    d_pow = torch.from_numpy(power).to(dev) if np.any(power) else None
    k = torch.empty((R, C_cells), dtype=torch.float64, device=dev)
    _abi.check(_abi.lib().fo_rate_laws(C_cells, R, d_laws.data_ptr(), d_T.data_ptr(), d_P.data_ptr(),
                                       d_par.data_ptr(), C_cells, d_pow.data_ptr() if d_pow is not None else None,
                                       k.data_ptr(), 1, C_cells, C.c_void_p(stream.cuda_stream)), "fo_rate_laws")
    stream.synchronize()     # the uploads above are freed on return
    return k


def run_scenario(scenario, solver, cells, ts1, rtol, atol, group_size=32, constrained=(), warmup_steps=0,
                 steps=None, on_step=None, snapshots_on_device=False):
    """Run a solver on a scenario's cells in groups that share a step
    (fastode/ts1.py:181-223). Returns (snapshots: step -> (C, n), counts,
    statuses), statuses being (first cell of the group, step, status) for
    every call that did not converge, in the reference's order.
    ``solver`` is this package's Algorithm, RestartingLoop or BackwardEuler.
    With ``snapshots_on_device`` the snapshots are CUDA tensors (C, n)
    (transposed views of the device layout) that ``score`` reads in place."""
    torch = _torch()
    n = ts1.mech.n
    atol_v = np.full(n, atol) if np.isscalar(atol) else np.asarray(atol, dtype=np.float64)
    mass = np.ones(n)
    for s in constrained:
        mass[ts1.index[s]] = 0.0
    nsteps = scenario.steps if steps is None else steps
    snap_steps = [s for s in scenario.snapshot_steps() if s <= nsteps] if steps is None else [nsteps]
    photolysis = [k for k in cells.params if k.startswith("j")]
    f_first = scenario.factor(max(-warmup_steps, 0) * scenario.dt)
    params = dict(cells.params)
    for name in photolysis:
        params[name] = np.asarray(cells.params[name]) * f_first
    batch = Batch(ts1.mech, cells.Y, group_size=group_size, algorithm=solver,
                  mass=None if np.all(mass == 1.0) else mass)
    dev, Cc = batch.dev, batch.C
    stream = batch._stream()
    table = rate_law_table(ts1) if hasattr(ts1, "reactions") and hasattr(ts1, "props") else None
    if table is not None:
        # the rate constants of the first interval, on the device
        k = device_rate_constants(ts1, cells.T, cells.P, params, dev, stream, table)
    else:
        # a mechanism object without reaction records: its own rate_constants
        k_static = np.asarray(ts1.rate_constants(cells.T, cells.P, params), dtype=np.float64)
        k = torch.from_numpy(np.ascontiguousarray(k_static.T)).to(dev)   # (R, C), cells fastest
    atol_d = torch.from_numpy(np.ascontiguousarray(atol_v)).to(dev)
    photo = _Photolysis(ts1, cells, photolysis, dev)
    step_list = list(range(-warmup_steps, nsteps))
    status_hist = torch.zeros((len(step_list), batch.ngroups), dtype=torch.int32, device=dev)
    snaps = {}
    for idx, step in enumerate(step_list):
        if idx > 0:
            photo.patch(k, Cc, scenario.factor(max(step, 0) * scenario.dt), stream)
        batch.step(k, scenario.dt, atol_d, rtol)
        status_hist[idx].copy_(batch.status)
        if on_step is not None:
            Yh = batch.state()
            for g0 in batch.offsets_host[:-1]:
                on_step(int(g0), step, Yh[g0:g0 + group_size])
        if step + 1 in snap_steps:
            snaps[step + 1] = batch.Y.clone()
    stream.synchronize()
    hist = status_hist.cpu().numpy()
    statuses = [(int(g0), step, _abi.STATUS_STRINGS[int(hist[idx, g])])
                for g, g0 in enumerate(batch.offsets_host[:-1])
                for idx, step in enumerate(step_list) if hist[idx, g] != 0]
    counts = batch.total_counts()
    if snapshots_on_device:
        snapshots = {s: Y.t() for s, Y in snaps.items()}
    else:
        snapshots = {s: Y.t().contiguous().cpu().numpy() for s, Y in snaps.items()}
    return snapshots, counts, statuses


def _digits_of(ms: float) -> float:
    return 16.0 if ms <= 0.0 else min(16.0, -math.log10(math.sqrt(ms)))


class _Accumulator:
    """Device sums and counts of squared relative errors per reference column."""

    def __init__(self, m, dev):
        torch = _torch()
        self.torch = torch
        self.dev = dev
        self.sums = torch.zeros(m, dtype=torch.float64, device=dev)
        self.counts = torch.zeros(m, dtype=torch.int64, device=dev)
        self.gate = torch.ones(1, dtype=torch.int32, device=dev)
        self.stream = torch.cuda.current_stream(dev)

    def add(self, Y, species, ref, threshold, rule, gate: bool):
        """Y: CUDA tensor (C, n) of any strides; ref: CUDA tensor (m, C)."""
        Cc, n = Y.shape
        m = 0 if species is None else species.numel()
        rc = _abi.lib().fo_score_accumulate(
            Cc, n, Y.data_ptr(), Y.stride(0), Y.stride(1), m,
            species.data_ptr() if m else None, ref.data_ptr() if m else None, 1, Cc if m else 0,
            float(threshold), rule, self.sums.data_ptr(), self.counts.data_ptr(),
            self.gate.data_ptr() if gate else None, C.c_void_p(self.stream.cuda_stream))
        _abi.check(rc, "fo_score_accumulate")

    def result(self):
        self.stream.synchronize()
        return self.sums.cpu().numpy(), self.counts.cpu().numpy(), bool(self.gate.item())


def _on_device(Y, dev):
    torch = _torch()
    if isinstance(Y, torch.Tensor):
        return Y.to(dev, dtype=torch.float64)
    return torch.from_numpy(np.ascontiguousarray(np.asarray(Y, dtype=np.float64))).to(dev)


def score(result: dict, cells_index, species, reference_path, threshold=1e-14, steps=None):
    """Digits overall and per species (Sandu et al.) and the gate over the
    snapshots in `result` (step -> (C, n) array or CUDA tensor, rows in the
    order of cells_index) against a reference table (fastode/ts1.py:226-264).
    Returns (overall, per-species dict, gate)."""
    torch = _torch()
    header, rows = read_csv_table(reference_path)
    dev = torch.device("cuda", torch.cuda.current_device())
    keyed = header[:2] == ["step", "cell"]
    start = 4 if keyed else 2
    ref_species = header[start:]
    sp_index = {s: i for i, s in enumerate(species)}
    want = list(cells_index)
    pos = {c: i for i, c in enumerate(want)}
    smap = torch.tensor([sp_index.get(s, -1) for s in ref_species], dtype=torch.int32, device=dev)
    acc = _Accumulator(len(ref_species), dev)
    for step, Y in result.items():
        Yd = _on_device(Y, dev)
        acc.add(Yd, None, None, threshold, _abi.SCORE_RULES["ts1"], gate=True)
        if keyed:
            sel = rows[(rows[:, 0] == step) & np.isin(rows[:, 1], want)]
            idx = torch.tensor([pos[int(r[1])] for r in sel], dtype=torch.int64, device=dev)
            Ysel = Yd.index_select(0, idx)
        else:
            sel = rows[want]
            Ysel = Yd[:len(want)]
        if len(sel) == 0:
            continue
        ref = torch.from_numpy(np.ascontiguousarray(sel[:, start:].T)).to(dev)     # (m, C)
        acc.add(Ysel, smap, ref, threshold, _abi.SCORE_RULES["ts1"], gate=False)
    sums, counts, gate = acc.result()
    per = {s: _digits_of(sums[j] / counts[j]) for j, s in enumerate(ref_species) if counts[j] > 0}
    total = int(counts.sum())
    overall = float("nan") if total == 0 else _digits_of(float(sums.sum()) / total)
    return overall, per, gate


def digits(result, reference, threshold, columns=None):
    """Sandu digits overall and per variable over all samples (rows) whose
    reference value is at least the threshold; capped at 16
    (fastode/reference.py:41-59). Returns (overall, {column: digits})."""
    torch = _torch()
    dev = torch.device("cuda", torch.cuda.current_device())
    R = np.asarray(reference, dtype=np.float64)
    cols = list(range(R.shape[1]) if columns is None else columns)
    X = _on_device(result, dev)
    acc = _Accumulator(len(cols), dev)
    smap = torch.tensor(cols, dtype=torch.int32, device=dev)
    ref = torch.from_numpy(np.ascontiguousarray(R[:, cols].T)).to(dev)
    acc.add(X, smap, ref, threshold, _abi.SCORE_RULES["digits"], gate=False)
    sums, counts, _ = acc.result()
    per = {j: _digits_of(sums[i] / counts[i]) for i, j in enumerate(cols) if counts[i] > 0}
    total = int(counts.sum())
    # no samples: the reference's mean is NaN, and min(16.0, NaN) is 16.0
    overall = _digits_of(float("nan") if total == 0 else float(sums.sum()) / total)
    return overall, per
