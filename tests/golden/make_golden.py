"""Generate the golden fixtures by running the reference package itself.

    python tests/golden/make_golden.py [--reference /root/reference]

Imports fastode from the reference checkout (it runs unmodified on NumPy and
SciPy), integrates the seeded synthetic workloads with
``fastode.Algorithm(ROS3)`` in a ``run_scenario``-style loop (a fresh Memory per
group of 32 cells, fastode/ts1.py:196-222), and stores the inputs together with
the reference's outputs, so that the fixtures are self-contained: tests rebuild
the mechanism from the stored reaction tables rather than from the generator.

Outputs per case (``<case>.npz``): reactant/product tables, A, E, J, cell
parameters, Y0, per-interval rate constants, final states, Counts per group,
status codes per group and interval, final Memory per group, and the
(t, H, err, outcome) trace of every attempt, recorded by wrapping
``fastode.solvers.error_norm`` the way experiments/ts1_rejections.py:26-47 does.
"""
from __future__ import annotations

import argparse
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
STATUS = {"converged": 0, "too many steps": 1, "step too small": 2, "nan or inf": 3, "projection failed": 4}


def reaction_tables(sm):
    """(reactants, products, yields) as int/float arrays; -1 pads, -2 is M."""
    R = len(sm.reactions)
    index = {s: i for i, s in enumerate(sm.species)}
    rt = np.full((R, 3), -1, dtype=np.int32)
    pt = np.full((R, 3), -1, dtype=np.int32)
    yt = np.zeros((R, 3))
    for j, (reactants, products) in enumerate(sm.reactions):
        for a, s in enumerate(reactants):
            rt[j, a] = -2 if s == "M" else index[s]
        for a, (s, y) in enumerate(products):
            pt[j, a] = index[s]
            yt[j, a] = y
    return rt, pt, yt


def run_reference(fastode_mod, wl, n_groups, intervals):
    from fastode import Algorithm, Counts, ROS3
    from fastode.chem import ChemSystem, Mechanism
    import fastode.solvers as S

    rm = Mechanism(wl.sm.species, wl.sm.reactions)
    C = n_groups * wl.group_size
    Y0 = wl.cells.Y0[:C]
    ks = np.stack([wl.k_at(i)[:C] for i in range(intervals)])
    Y = Y0.copy()
    counts = np.zeros((n_groups, 13), dtype=np.int64)
    status = np.zeros((n_groups, intervals), dtype=np.int32)
    memory = np.zeros((n_groups, 3))
    traces = []
    original = S.error_norm
    original_stages = S.stages
    for g in range(n_groups):
        sl = slice(g * wl.group_size, (g + 1) * wl.group_size)
        alg = Algorithm(ROS3)
        mem = alg.new_memory()
        c = Counts()
        rec = []
        hrec = []

        def traced(Yv, Ynew, E, atol, rtol, _rec=rec):
            err = original(Yv, Ynew, E, atol, rtol)
            _rec.append(err)
            return err

        def traced_stages(system, tab, Yv, F0, LU, H, cnt, _h=hrec):
            _h.append(H)
            return original_stages(system, tab, Yv, F0, LU, H, cnt)

        S.error_norm = traced
        S.stages = traced_stages
        try:
            Yg = Y[sl].copy()
            for i in range(intervals):
                Yg, st = alg.solve(ChemSystem(rm, ks[i][sl]), Yg, wl.dt, wl.atol, wl.rtol, c, mem)
                status[g, i] = STATUS[st]
        finally:
            S.error_norm = original
            S.stages = original_stages
        Y[sl] = Yg
        counts[g] = list(c.as_dict().values())
        memory[g] = (mem.h_next, mem.err_prev, mem.h_prev)
        traces.append((np.array(hrec), np.array(rec)))
    L = max(len(t[1]) for t in traces)
    errs = np.full((n_groups, L), np.nan)
    hs = np.full((n_groups, L), np.nan)
    for g, (h, e) in enumerate(traces):
        errs[g, : len(e)] = e
        hs[g, : len(h)] = h
    return dict(Y0=Y0, k=ks, Y=Y, counts=counts, status=status, memory=memory, errs=errs, hs=hs,
                n_attempts=np.array([len(t[1]) for t in traces]))


def mechanism_arrays(mech):
    """The reference Mechanism's compiled tables (fastode/chem.py:19-79)."""
    GT = mech.GT.tocsr()
    return dict(m_n=mech.n, m_R=mech.R, m_P=mech.P, m_react=mech.react, m_S=mech.S,
                m_rows=mech.pattern.rows, m_cols=mech.pattern.cols,
                m_gt_indptr=GT.indptr, m_gt_indices=GT.indices, m_gt_data=GT.data)


def dae_cases():
    """RODAS3 with quasi-steady species (mass = 0), the reference's own small
    mechanisms of fastode/problems.py run through Algorithm.solve, which then
    starts every call with the consistent-initialization projection
    (fastode/solvers.py:100-178, 322-325)."""
    from fastode import Algorithm, Counts, RODAS3
    from fastode import problems as P
    from fastode.chem import ChemSystem
    out = {}
    specs = {
        # name: (system, Y0, dt, atol, rtol, intervals); tropospheric gets four
        # cells that differ in photolysis (j = 1, 0.5, 0.1, 0.02)
        "rodas3_robertson_qssa": (P.robertson(qssa=True), 1.0, 1e-10, 1e-4, 6),
        "rodas3_chapman_qssa": (P.chapman(qssa=True), 3600.0, 1e-6, 1e-4, 24),
        "rodas3_tropospheric_qssa": (None, 600.0, 600.0, 1e-3, 24),
    }
    for name, (made, dt, atol, rtol, intervals) in specs.items():
        if made is None:
            cells = [P.tropospheric(j=j, qssa=True) for j in (1.0, 0.5, 0.1, 0.02)]
            mech = cells[0][0].mech
            mass = cells[0][0].mass
            k = np.concatenate([c[0].k for c in cells])
            Y0 = np.concatenate([c[1] for c in cells])
        else:
            system, Y0 = made
            mech, mass, k = system.mech, system.mass, system.k
        alg = Algorithm(RODAS3)
        mem = alg.new_memory()
        c = Counts()
        Y = Y0.copy()
        atolv = np.full(mech.n, atol)
        status = []
        zero_residual_calls = 0
        for _ in range(intervals):
            system = ChemSystem(mech, k, mass=mass)
            # a call whose projection residual is exactly 0.0 at entry stops before
            # the Newton update; that test is a bit-level tie (the value depends on
            # the BLAS GEMM's summation order), recorded so tests can allow it
            G = system.rhs(Y)
            if float(np.abs(G[:, mass == 0.0]).max()) == 0.0:
                zero_residual_calls += 1
            Y, st = alg.solve(system, Y, dt, atolv, rtol, c, mem)
            status.append(STATUS[st])
        out[name] = dict(mechanism_arrays(mech), mass=mass, k=k, Y0=Y0, dt=dt, atol=atolv, rtol=rtol,
                         intervals=intervals, Y=Y, counts=np.array(list(c.as_dict().values())),
                         status=np.array(status), memory=np.array([mem.h_next, mem.err_prev, mem.h_prev]),
                         zero_residual_calls=zero_residual_calls)
    return out


def ts1_case(reference):
    """TS1 (209 species, 547 reactions, P = 3) on the tier1-30s scenario, 64
    cells x 101 intervals, Algorithm(ROS3) at rtol 1e-3, atol 1e-17, through
    the reference's own run_scenario (fastode/ts1.py:181-223). Stores what the
    device needs to rebuild every interval's rate constants exactly as
    run_scenario does (the static k, the photolysis columns' base values,
    scaling factors and the scenario factor of every interval) and checks the
    Counts against the archived record reference-results/ts1/runs.csv."""
    import csv
    from fastode import Algorithm, ROS3
    from fastode.ts1 import TS1, Cells, Scenario, run_scenario

    ts1 = TS1()
    sc = Scenario(Path(reference) / "data/scenarios/tier1-30s/scenario.txt")
    cells = Cells(ts1, sc.cells)
    snaps, counts, statuses = run_scenario(sc, Algorithm(ROS3), cells, ts1, 1e-3, 1e-17)
    with open(Path(reference) / "reference-results/ts1/runs.csv") as fh:
        row = next(r for r in csv.DictReader(fh)
                   if r["config"] == "alg" and r["scenario"] == "tier1-30s" and float(r["rtol"]) == 1e-3)
    for field in ("steps", "accepted", "rejected", "rhs", "jac", "lu", "solves"):
        assert int(row[field]) == getattr(counts, field), (field, row[field], getattr(counts, field))
    photo = ts1.photolysis_reactions
    names = [ts1.reactions[j]["MUSICA name"] for j in photo]
    scaling = np.array([ts1.reactions[j].get("scaling factor", 1.0) for j in photo])
    base = np.stack([cells.params[nm] for nm in names], axis=1)            # (C, nphoto)
    f = np.array([sc.factor(i * sc.dt) for i in range(sc.steps)])
    params0 = {k: (v * f[0] if k.startswith("j") else v) for k, v in cells.params.items()}
    k_static = ts1.rate_constants(cells.T, cells.P, params0)
    m = ts1.mech
    Sr, Sc = np.nonzero(m.S)
    GT = m.GT.tocsr()
    # the controller variants and the restarting loop on the same scenario,
    # each checked against its archived row (experiments/ts1_experiments.py:49-70)
    from fastode import RestartingLoop
    variants = {
        "alg-elementary": (Algorithm(ROS3, controller="elementary"), 5e-4, 5e-18),
        "alg-noquant": (Algorithm(ROS3, quantize=False), 5e-4, 5e-18),
        "alg-nomemory": (Algorithm(ROS3, carry_memory=False), 5e-4, 5e-18),
        "alg-reset": (Algorithm(ROS3, carry=False, quantize=False), 1e-2, 1e-16),
        "restart": (RestartingLoop(ROS3), 1e-3, 1e-15),
    }
    extra = {}
    for name, (solver, rtol, atol) in variants.items():
        s_snaps, s_counts, _ = run_scenario(sc, solver, cells, ts1, rtol, atol)
        with open(Path(reference) / "reference-results/ts1/runs.csv") as fh:
            row = next(r for r in csv.DictReader(fh)
                       if r["config"] == name and r["scenario"] == "tier1-30s" and float(r["rtol"]) == rtol)
        for field in ("steps", "accepted", "rejected", "rhs", "jac", "lu", "solves"):
            assert int(row[field]) == getattr(s_counts, field), (name, field)
        key = name.replace("-", "_")
        extra[f"{key}_Y"] = s_snaps[sc.steps]
        extra[f"{key}_counts"] = np.array(list(s_counts.as_dict().values()))
        extra[f"{key}_tol"] = np.array([rtol, atol])
    return dict(m_n=m.n, m_R=m.R, m_P=m.P, m_react=m.react, m_S_rows=Sr, m_S_cols=Sc, m_S_vals=m.S[Sr, Sc], **extra,
                m_rows=m.pattern.rows, m_cols=m.pattern.cols, m_gt_indptr=GT.indptr, m_gt_indices=GT.indices,
                m_gt_data=GT.data, Y0=cells.Y, k_static=k_static, photo=np.array(photo), base=base,
                scaling=scaling, f=f, dt=sc.dt, intervals=sc.steps, rtol=1e-3, atol=np.full(m.n, 1e-17),
                group_size=32, Y=snaps[sc.steps], counts=np.array(list(counts.as_dict().values())),
                n_failed=len(statuses))


# BackwardEuler on TS1 tier1-30s: the three archived configurations
# (experiments/ts1_experiments.py:60-61; Counts checked against
# reference-results/ts1/runs.csv) and two that make the Newton iteration fail,
# so that step cuts, doubling after two successes and accepted unconverged
# iterates all occur. name: (constructor arguments, rtol, atol, archived).
BE_CONFIGS = {
    "be": ({}, 1e-6, 1e-3, True),
    "be_tight_3": ({}, 1e-3, 1e-15, True),
    "be_tight_6": ({}, 1e-6, 1e-15, True),
    "be_it2": ({"max_iterations": 2}, 1e-6, 1e-15, False),
    "be_it3": ({"max_iterations": 3, "reductions": (0.5, 0.25)}, 1e-8, 1e-18, False),
}
BE_STATUS = {"converged": 0, "nan or inf": 3, "accepted unconverged": 5}


def backward_euler_ts1(reference):
    """Final states, Counts and per-interval statuses of the reference's
    BackwardEuler through run_scenario on TS1 tier1-30s (the inputs are those
    of ts1_tier1_30s.npz)."""
    import csv
    from fastode import BackwardEuler
    from fastode.ts1 import TS1, Cells, Scenario, run_scenario

    ts1 = TS1()
    sc = Scenario(Path(reference) / "data/scenarios/tier1-30s/scenario.txt")
    cells = Cells(ts1, sc.cells)
    out = {}
    for name, (kw, rtol, atol, archived) in BE_CONFIGS.items():
        snaps, counts, failed = run_scenario(sc, BackwardEuler(**kw), cells, ts1, rtol, atol)
        if archived:
            config = "be" if name == "be" else "be-tight"
            with open(Path(reference) / "reference-results/ts1/runs.csv") as fh:
                row = next(r for r in csv.DictReader(fh) if r["config"] == config and r["scenario"] == "tier1-30s"
                           and float(r["rtol"]) == rtol and float(r["atol"]) == atol)
            for field in ("steps", "accepted", "rejected", "rhs", "jac", "lu", "solves", "newton", "failures",
                          "unconverged"):
                assert int(row[field]) == getattr(counts, field), (name, field)
        ngroups = (cells.C + 31) // 32
        status = np.zeros((ngroups, sc.steps), dtype=np.int32)
        for g0, i, st in failed:          # (first cell of the group, interval, status)
            status[g0 // 32, i] = BE_STATUS[st]
        out[f"{name}_Y"] = snaps[sc.steps]
        out[f"{name}_counts"] = np.array(list(counts.as_dict().values()))
        out[f"{name}_tol"] = np.array([rtol, atol])
        out[f"{name}_max_iterations"] = np.array(kw.get("max_iterations", 11))
        out[f"{name}_reductions"] = np.array(kw.get("reductions", (0.5, 0.5, 0.5, 0.5, 0.1)))
        out[f"{name}_status"] = status
        print(name, list(counts.as_dict().values()), len(failed), "non-converged group-intervals")
    return out


def ts1_rate_laws(reference):
    """TS1's rate constants on the tier1-30s cells as the reference computes
    them for the first interval of run_scenario (fastode/ts1.py:194-210: the
    photolysis parameters scaled by the first scenario factor), with the
    inputs the device evaluates them from: this package's law table compiled
    from the reference's reaction records, the per-cell parameter columns,
    T, P and the third-body powers."""
    from fastode.ts1 import TS1, Cells, Scenario
    from fastode_gb300.scenario import rate_law_table
    ts1 = TS1()
    sc = Scenario(Path(reference) / "data/scenarios/tier1-30s/scenario.txt")
    cells = Cells(ts1, sc.cells)
    f0 = sc.factor(0.0)
    params = {k: (np.asarray(v) * f0 if k.startswith("j") else np.asarray(v)) for k, v in cells.params.items()}
    k = ts1.rate_constants(cells.T, cells.P, params)
    laws, columns = rate_law_table(ts1)
    return dict(law_type=laws["type"], law_column=laws["column"], law_c=laws["c"],
                params=np.stack([np.asarray(params[c], dtype=np.float64) for c in columns]),
                columns=np.array(columns), T=np.asarray(cells.T, dtype=np.float64),
                P=np.asarray(cells.P, dtype=np.float64),
                power=np.asarray(ts1.mech.third_body_power, dtype=np.float64), k=k)


SUBSET_INTERVALS = 30
SUBSET_SNAPSHOTS = (10, 20, 30)


def _subset_group(args):
    """One group of the 210/500 parity subset through the reference: cumulative
    Counts and status after every interval, the (H, err) of every attempt with
    the interval it belongs to, the state at the snapshot intervals and the
    final Memory."""
    reference, root, Y0, k0, photo, J, f, dt, atol, rtol, intervals = args
    sys.path.insert(0, reference)
    sys.path.insert(0, root)
    from fastode import Algorithm, Counts, ROS3
    from fastode.chem import ChemSystem, Mechanism
    import fastode.solvers as S
    from fastode_gb300 import synthetic as syn
    wl = syn.plain_large(n_cells=32, intervals=1)
    rm = Mechanism(wl.sm.species, wl.sm.reactions)
    hs, errs, where = [], [], []
    cur = [0]
    original, original_stages = S.error_norm, S.stages

    def traced(Yv, Ynew, E, at, rt):
        e = original(Yv, Ynew, E, at, rt)
        errs.append(e)
        where.append(cur[0])
        return e

    def traced_stages(system, tab, Yv, F0, LU, H, cnt):
        hs.append(H)
        return original_stages(system, tab, Yv, F0, LU, H, cnt)

    S.error_norm, S.stages = traced, traced_stages
    alg = Algorithm(ROS3)
    mem = alg.new_memory()
    c = Counts()
    Y = Y0.copy()
    counts, status, snaps = [], [], {}
    for i in range(intervals):
        cur[0] = i
        k = k0.copy()
        k[:, photo] = J[None, :] * f[i][:, None]
        Y, st = alg.solve(ChemSystem(rm, k), Y, dt, atol, rtol, c, mem)
        counts.append(list(c.as_dict().values()))
        status.append(STATUS[st])
        if i + 1 in SUBSET_SNAPSHOTS:
            snaps[i + 1] = Y.copy()
    return (np.array(counts), np.array(status), np.array(hs), np.array(errs), np.array(where),
            np.stack([snaps[s] for s in SUBSET_SNAPSHOTS]), np.array([mem.h_next, mem.err_prev, mem.h_prev]))


TIGHT_INTERVALS = 20


def _tight_group(args):
    """One group of the parity subset through the reference at rtol = 1e-10,
    atol = 1e-10 * a: the FP64 accuracy oracle, at intervals 10 and 20."""
    reference, root, Y0, k0, photo, J, f, dt, n, intervals = args
    sys.path.insert(0, reference)
    sys.path.insert(0, root)
    from fastode import Algorithm, Counts, ROS3
    from fastode.chem import ChemSystem, Mechanism
    from fastode_gb300 import synthetic as syn
    wl = syn.plain_large(n_cells=32, intervals=1)
    rm = Mechanism(wl.sm.species, wl.sm.reactions)
    alg = Algorithm(ROS3, max_steps=1000000)
    mem = alg.new_memory()
    c = Counts()
    Y = Y0.copy()
    atol = np.full(n, 1e-10 * 1e-14)
    snaps = []
    for i in range(intervals):
        k = k0.copy()
        k[:, photo] = J[None, :] * f[i][:, None]
        Y, st = alg.solve(ChemSystem(rm, k), Y, dt, atol, 1e-10, c, mem)
        assert st == "converged", st
        if i + 1 in (10, 20):
            snaps.append(Y.copy())
    return np.stack(snaps), c.steps


def c2_subset_tight(reference, subset):
    """The reference's tight solve of the parity subset's cells (the accuracy
    oracle of the measured run), one group per process."""
    import multiprocessing as mp
    gs = int(subset["group_size"])
    G = len(subset["groups"])
    jobs = [(reference, str(ROOT), subset["Y0"][j * gs:(j + 1) * gs], subset["k0"][j * gs:(j + 1) * gs],
             subset["photo"], subset["J"], subset["f"][:, j * gs:(j + 1) * gs], float(subset["dt"]),
             int(subset["n"]), TIGHT_INTERVALS) for j in range(G)]
    os.environ["OMP_NUM_THREADS"] = os.environ["OPENBLAS_NUM_THREADS"] = "1"
    with mp.get_context("spawn").Pool(min(G, os.cpu_count() or 1)) as pool:
        res = pool.map(_tight_group, jobs)
    return dict(tight_snapshots=np.array([10, 20]),
                Y_tight=np.stack([r[0] for r in res], axis=1).reshape(2, -1, int(subset["n"])),
                tight_steps=np.array([r[1] for r in res]))


def c2_subset(reference):
    """The reference on the seeded parity subset of the 210/500, 65,536-cell
    workload (synthetic.PLAIN_LARGE_PARITY_GROUPS, eight whole groups) over
    the first 30 intervals, one group per process. Stores the inputs of those
    cells (Y0, k at t = 0, the photolysis columns and every interval's diurnal
    factors), so that the device can consume exactly the reference's inputs."""
    import multiprocessing as mp
    from fastode_gb300 import synthetic as syn
    wl = syn.plain_large()
    groups = syn.PLAIN_LARGE_PARITY_GROUPS
    gs = wl.group_size
    cells = np.concatenate([np.arange(g * gs, (g + 1) * gs) for g in groups])
    sub = wl.subset(cells)
    k0 = sub.k_at(0)
    photo = np.nonzero(wl.sm.photolytic)[0].astype(np.int32)
    J = wl.sm.J[photo]
    f = syn.photolysis_factors(sub.cells, wl.dt, SUBSET_INTERVALS)
    for i in range(SUBSET_INTERVALS):          # the stored inputs rebuild k_at exactly
        k = k0.copy()
        k[:, photo] = J[None, :] * f[i][:, None]
        assert np.array_equal(k, sub.k_at(i))
    jobs = [(reference, str(ROOT), sub.cells.Y0[j * gs:(j + 1) * gs], k0[j * gs:(j + 1) * gs], photo, J,
             f[:, j * gs:(j + 1) * gs], wl.dt, wl.atol, wl.rtol, SUBSET_INTERVALS) for j in range(len(groups))]
    env = {k: os.environ.get(k) for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS")}
    os.environ["OMP_NUM_THREADS"] = os.environ["OPENBLAS_NUM_THREADS"] = "1"
    try:
        with mp.get_context("spawn").Pool(min(len(jobs), os.cpu_count() or 1)) as pool:
            res = pool.map(_subset_group, jobs)
    finally:
        for k, v in env.items():
            if v is None:
                os.environ.pop(k, None)
            else:
                os.environ[k] = v
    L = max(len(r[2]) for r in res)
    pad = lambda a, fill: np.concatenate([a, np.full(L - len(a), fill, dtype=np.asarray(a).dtype)])
    rt, pt, yt = reaction_tables(wl.sm)
    return dict(n=wl.sm.n, reactants=rt, products=pt, yields=yt, groups=np.array(groups), cells=cells,
                group_size=gs, Y0=sub.cells.Y0, k0=k0, photo=photo, J=J, f=f, dt=wl.dt,
                intervals=SUBSET_INTERVALS, rtol=wl.rtol, atol=wl.atol,
                counts=np.stack([r[0] for r in res]), status=np.stack([r[1] for r in res]),
                hs=np.stack([pad(r[2], np.nan) for r in res]), errs=np.stack([pad(r[3], np.nan) for r in res]),
                interval_of=np.stack([pad(r[4], -1) for r in res]),
                n_attempts=np.array([len(r[2]) for r in res]), snapshots=np.array(SUBSET_SNAPSHOTS),
                Y_snap=np.stack([r[5] for r in res], axis=1).reshape(len(SUBSET_SNAPSHOTS), -1, wl.sm.n),
                memory=np.stack([r[6] for r in res]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default="/root/reference")
    ap.add_argument("--only", choices=["backward-euler", "c2-subset", "c2-subset-tight", "ts1-rate-laws"],
                    default=None,
                    help="regenerate one fixture instead of all")
    a = ap.parse_args()
    sys.path.insert(0, a.reference)
    sys.path.insert(0, str(ROOT))
    import fastode
    from fastode_gb300 import synthetic as syn

    if a.only == "backward-euler":
        np.savez_compressed(HERE / "ts1_tier1_30s_backward_euler.npz", **backward_euler_ts1(a.reference))
        return
    if a.only == "ts1-rate-laws":
        np.savez_compressed(HERE / "ts1_rate_laws.npz", **ts1_rate_laws(a.reference))
        return
    if a.only == "c2-subset-tight":
        sub = dict(np.load(HERE / "ros3_210x500_subset.npz"))
        sub.update(c2_subset_tight(a.reference, sub))
        np.savez_compressed(HERE / "ros3_210x500_subset.npz", **sub)
        print("tight steps per group", sub["tight_steps"].tolist())
        return
    if a.only == "c2-subset":
        out = c2_subset(a.reference)
        out.update(c2_subset_tight(a.reference, out))
        np.savez_compressed(HERE / "ros3_210x500_subset.npz", **out)
        print("ros3_210x500_subset counts", out["counts"][:, -1].sum(axis=0).tolist(), "attempts",
              out["n_attempts"].tolist())
        return
    out = c2_subset(a.reference)
    out.update(c2_subset_tight(a.reference, out))
    np.savez_compressed(HERE / "ros3_210x500_subset.npz", **out)
    np.savez_compressed(HERE / "ts1_rate_laws.npz", **ts1_rate_laws(a.reference))
    np.savez_compressed(HERE / "ts1_tier1_30s_backward_euler.npz", **backward_euler_ts1(a.reference))

    ts1 = ts1_case(a.reference)
    np.savez_compressed(HERE / "ts1_tier1_30s.npz", **ts1)
    print("ts1_tier1_30s counts", ts1["counts"].tolist())

    # the constrained synthetic workload: one group of 32 cells, RODAS3 with the
    # projection at every call
    wl = syn.dae_constrained(n_cells=32, intervals=4)
    from fastode import Algorithm, Counts, RODAS3
    from fastode.chem import ChemSystem, Mechanism
    rm = Mechanism(wl.sm.species, wl.sm.reactions)
    alg = Algorithm(RODAS3)
    mem = alg.new_memory()
    c = Counts()
    Y = wl.cells.Y0.copy()
    ks = np.stack([wl.k_at(i) for i in range(wl.intervals)])
    status = []
    for i in range(wl.intervals):
        Y, st = alg.solve(ChemSystem(rm, ks[i], mass=wl.mass), Y, wl.dt, wl.atol, wl.rtol, c, mem)
        status.append(STATUS[st])
    rt, pt, yt = reaction_tables(wl.sm)
    np.savez_compressed(HERE / "rodas3_dae_160x340.npz", n=wl.sm.n, reactants=rt, products=pt, yields=yt,
                        mass=wl.mass, Y0=wl.cells.Y0, k=ks, dt=wl.dt, intervals=wl.intervals, rtol=wl.rtol,
                        atol=wl.atol, Y=Y, counts=np.array(list(c.as_dict().values())), status=np.array(status),
                        memory=np.array([mem.h_next, mem.err_prev, mem.h_prev]))
    print("rodas3_dae_160x340 counts", list(c.as_dict().values()), "status", status)

    for name, arrays in dae_cases().items():
        np.savez_compressed(HERE / f"{name}.npz", **arrays)
        print(name, "counts", arrays["counts"].tolist(), "status", arrays["status"].tolist())

    cases = {
        # name: (workload, groups, intervals)
        "ros3_20x40": (syn.plain_small(), 2, 20),
        "ros3_210x500": (syn.plain_large(n_cells=64, intervals=4), 2, 4),
    }
    for name, (wl, groups, intervals) in cases.items():
        out = run_reference(fastode, wl, groups, intervals)
        rt, pt, yt = reaction_tables(wl.sm)
        np.savez_compressed(
            HERE / f"{name}.npz",
            n=wl.sm.n, reactants=rt, products=pt, yields=yt, A=wl.sm.A, E=wl.sm.E, J=wl.sm.J,
            photolytic=wl.sm.photolytic, T=wl.cells.T[: groups * wl.group_size],
            p=wl.cells.p[: groups * wl.group_size], phase=wl.cells.phase[: groups * wl.group_size],
            dt=wl.dt, intervals=intervals, rtol=wl.rtol, atol=wl.atol, group_size=wl.group_size, **out)
        print(name, "counts", out["counts"].sum(axis=0).tolist())


if __name__ == "__main__":
    main()
