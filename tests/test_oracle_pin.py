"""Pin the oracle to the reference: the golden fixtures hold the reference's own
outputs (tests/golden/make_golden.py), and the controller cases restate the
known answers of the reference's unit tests (tests/test_fastode.py:89-208) on
one-species mechanisms. CPU only."""
import math

import numpy as np
import pytest

from golden_cases import CASES, load, mechanism_of
from oracle import rosenbrock as O

STATUS = ("converged", "too many steps", "step too small", "nan or inf", "projection failed")


@pytest.mark.parametrize("case", CASES)
def test_oracle_reproduces_reference_fixture(case):
    f = load(case)
    mech = mechanism_of(f)
    G = f["counts"].shape[0]
    gs = int(f["group_size"])
    intervals = int(f["intervals"])
    ks = f["k"]
    Y, counts, statuses, mems, traces = O.run_groups(
        mech, f["Y0"], lambda i: ks[i], float(f["dt"]), intervals, f["atol"], float(f["rtol"]),
        group_size=gs, trace=True)
    # the same NumPy/SciPy operations on the same inputs: bit-identical
    np.testing.assert_array_equal(Y, f["Y"])
    for g in range(G):
        assert counts[g].as_tuple() == tuple(f["counts"][g])
        assert [STATUS.index(s) for s in statuses[g]] == list(f["status"][g])
        assert (mems[g].h_next, mems[g].err_prev, mems[g].h_prev) == tuple(f["memory"][g])
        na = int(f["n_attempts"][g])
        assert [t[2] for t in traces[g]] == list(f["errs"][g, :na])
        assert [t[1] for t in traces[g]] == list(f["hs"][g, :na])


def one_species(lam):
    """y' = -lam*y as the mechanism A -> (nothing) with k = lam."""
    from fastode_gb300.chem import Mechanism
    return Mechanism(["A"], [(["A"], [])]), np.array([[lam]])


def test_oracle_quantize():
    # tests/test_fastode.py:89-93
    for h in (1.0, 7.3, 33.0, 600.0, 900.0):
        q = O.quantize(h, 600.0)
        n = round(600.0 / q)
        assert abs(n * q - 600.0) < 1e-9 and h / 2 < q <= h or h >= 600.0


def test_oracle_carried_step_takes_one_step():
    # tests/test_fastode.py:96-110
    mech, k = one_species(1e-6)
    alg = O.OAlgorithm(O.OROS3)
    mem = O.OMemory()
    Y = np.array([[1.0]])
    c = O.OCounts()
    for _ in range(5):
        Y, _ = alg.solve(O.OChem(mech, k), Y, 600.0, np.array([1e-10]), 1e-3, c, mem)
    c3 = O.OCounts()
    alg.solve(O.OChem(mech, k), Y, 600.0, np.array([1e-10]), 1e-3, c3, mem)
    assert c3.accepted == 1


def test_oracle_quantized_steps_land_on_interval_end():
    # tests/test_fastode.py:113-125
    mech, k = one_species(1e-9)
    alg = O.OAlgorithm(O.OROS3, fac_max=1.0)
    mem = O.OMemory(h_next=600.0 / 7)
    Y = np.array([[1.0]])
    for _ in range(3):
        c = O.OCounts()
        Y, st = alg.solve(O.OChem(mech, k), Y, 600.0, np.array([1e-10]), 1e-3, c, mem)
        assert st == "converged" and c.steps == 7
        assert abs(mem.h_next - 600.0 / 7) < 1e-9


def test_oracle_rejection_shrinks_step():
    # tests/test_fastode.py:128-136
    mech, k = one_species(1.0)
    alg = O.OAlgorithm(O.OROS3)
    mem = O.OMemory(1.0, 1e-8, 1.0)
    c = O.OCounts()
    alg.solve(O.OChem(mech, k), np.array([[1.0]]), 1.0, np.array([1e-12]), 4e-3, c, mem)
    assert c.rejected == 1


def test_oracle_no_forced_acceptance_below_minimum_step():
    # tests/test_fastode.py:152-169
    mech, k = one_species(1e15)
    alg = O.OAlgorithm(O.OROS3, max_steps=10)
    mem = O.OMemory(h_next=1e-15)
    c = O.OCounts()
    y0 = np.array([[1.0]])
    y, st = alg.solve(O.OChem(mech, k), y0, 1.0, np.array([1e-30]), 1e-12, c, mem)
    assert st == "step too small"
    assert c.steps == c.rejected == 1 and c.accepted == 0
    np.testing.assert_array_equal(y, y0)


@pytest.mark.parametrize("budget", [0, 1, 2])
def test_oracle_budget_includes_rejected(budget):
    # tests/test_fastode.py:172-187
    mech, k = one_species(1.0)
    alg = O.OAlgorithm(O.OROS3, max_steps=budget)
    mem = O.OMemory(h_next=1.0)
    c = O.OCounts()
    y0 = np.array([[1.0]])
    y, st = alg.solve(O.OChem(mech, k), y0, 1.0, np.array([1e-30]), 1e-13, c, mem)
    assert st == "too many steps"
    assert c.steps == c.rejected == budget and c.accepted == 0
    np.testing.assert_array_equal(y, y0)


@pytest.mark.parametrize("budget, expected", [(2, "too many steps"), (10, "converged")])
def test_oracle_budget_includes_accepted(budget, expected):
    # tests/test_fastode.py:190-208
    mech, k = one_species(1e-6)
    alg = O.OAlgorithm(O.OROS3, max_steps=budget, fac_max=1.0)
    mem = O.OMemory(h_next=0.1)
    c = O.OCounts()
    _, st = alg.solve(O.OChem(mech, k), np.array([[1.0]]), 1.0, np.array([1e-10]), 1e-3, c, mem)
    assert st == expected
    assert c.steps == c.accepted == budget and c.rejected == 0


def test_oracle_linear_invariant():
    # tests/test_fastode.py:68-72: Robertson conserves A + B + C under fixed steps
    from fastode_gb300.chem import Mechanism
    mech = Mechanism(["A", "B", "C"], [(["A"], [("B", 1.0)]), (["B", "B"], [("B", 1.0), ("C", 1.0)]),
                                       (["B", "C"], [("A", 1.0), ("C", 1.0)])])
    k = np.array([[0.04, 3.0e7, 1.0e4]])
    for tab in (O.OROS3, O.ORODAS3):
        Y = O.fixed_steps(O.OChem(mech, k), tab, np.array([[1.0, 0.0, 0.0]]), 1.0e-2, 50)
        assert abs(Y.sum() - 1.0) < 1e-14


def test_oracle_order_three():
    # tests/test_fastode.py:44-51 restated on a mass-action mechanism:
    # A + A + A -> 2A gives y' = -y^3 with k = 1
    from fastode_gb300.chem import Mechanism
    mech = Mechanism(["A"], [(["A", "A", "A"], [("A", 2.0)])])
    exact = 1.0 / math.sqrt(3.0)
    for tab in (O.OROS3, O.ORODAS3):
        errs = [abs(O.fixed_steps(O.OChem(mech, np.array([[1.0]])), tab, np.array([[1.0]]), 1.0, n)[0, 0] - exact)
                for n in (20, 40, 80)]
        orders = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
        assert min(orders) > 2.8


@pytest.mark.parametrize("case", ["rodas3_robertson_qssa", "rodas3_chapman_qssa", "rodas3_tropospheric_qssa"])
def test_oracle_reproduces_reference_dae_fixture(case):
    """RODAS3 with the consistent-initialization projection: the oracle gives
    the reference's Counts, statuses, memory and states bit for bit."""
    from golden_cases import TableMechanism
    f = load(case)
    mech = TableMechanism(f)
    alg = O.OAlgorithm(O.ORODAS3)
    mem, c = O.OMemory(), O.OCounts()
    Y = f["Y0"].copy()
    status = []
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        for _ in range(int(f["intervals"])):
            Y, st = alg.solve(O.OChem(mech, f["k"], mass=f["mass"]), Y, float(f["dt"]), f["atol"], float(f["rtol"]), c, mem)
            status.append(STATUS.index(st))
    assert c.as_tuple() == tuple(f["counts"])
    assert status == list(f["status"])
    assert (mem.h_next, mem.err_prev, mem.h_prev) == tuple(f["memory"])
    np.testing.assert_array_equal(Y, f["Y"])


def test_oracle_tangent_linear_matches_central_differences():
    """The host FP64 tangent-linear of the fixed-step map (complex step
    through the oracle's own steps) agrees with central differences, h = 1e-6."""
    f = load("ros3_20x40")
    mech = mechanism_of(f)
    Y0 = f["Y0"][:32]
    ks = [f["k"][i][:32] for i in range(3)]
    steps = [[30.0], [15.0, 15.0], [30.0]]
    rng = np.random.default_rng(0)
    dY = Y0 * rng.standard_normal(Y0.shape)
    dth = rng.standard_normal(mech.R)
    tl, _ = O.tangent_linear(mech, Y0, dY, ks, dth, steps)

    def run(Y, th):
        for k, s in zip(ks, steps):
            Y = O.replay_interval(O.OChem(mech, k * np.exp(th)[None, :], dense=True), O.OROS3, Y, s)
        return Y

    h = 1e-6
    fd = (run(Y0 + h * dY, h * dth) - run(Y0 - h * dY, -h * dth)) / (2 * h)
    assert np.max(np.abs(tl - fd)) <= 1e-8 * np.max(np.abs(tl))


def test_oracle_reproduces_ts1_tier1_archive():
    """TS1 on tier1-30s through the oracle (SuperLU path, as the reference's
    run_scenario uses): the archived Counts (334 / 330 / 4) and the reference's
    final states bit for bit."""
    from golden_cases import table_mechanism, ts1_k
    f = load("ts1_tier1_30s")
    mech = table_mechanism(f)
    Y, counts, statuses, _, _ = O.run_groups(mech, f["Y0"], lambda i: ts1_k(f, i), float(f["dt"]),
                                             int(f["intervals"]), f["atol"], float(f["rtol"]), group_size=32)
    total = np.sum([c.as_tuple() for c in counts], axis=0)
    np.testing.assert_array_equal(total, f["counts"])
    np.testing.assert_array_equal(Y, f["Y"])


@pytest.mark.parametrize("config", ["be_tight_6", "be_it3"])
def test_oracle_backward_euler_reproduces_ts1_reference(config):
    """BackwardEuler (fastode/solvers.py:418-491) on TS1 tier1-30s through the
    oracle: the reference's final states bit for bit, its Counts (for
    be_tight_6 the archived row of reference-results/ts1/runs.csv: 616 Newton
    iterations over 202 steps) and its per-interval statuses. be_it3 makes
    the Newton iteration fail, so step cuts and accepted unconverged iterates
    occur."""
    from golden_cases import table_mechanism, ts1_k
    f = load("ts1_tier1_30s")
    b = load("ts1_tier1_30s_backward_euler")
    mech = table_mechanism(f)
    rtol, atol = b[f"{config}_tol"]
    make = lambda: O.OBackwardEuler(max_iterations=int(b[f"{config}_max_iterations"]),  # noqa: E731
                                    reductions=tuple(b[f"{config}_reductions"]))
    Y, counts, statuses, _, _ = O.run_groups(mech, f["Y0"], lambda i: ts1_k(f, i), float(f["dt"]),
                                             int(f["intervals"]), np.full(mech.n, atol), float(rtol),
                                             group_size=32, solver=make)
    total = np.sum([c.as_tuple() for c in counts], axis=0)
    np.testing.assert_array_equal(total, b[f"{config}_counts"])
    codes = {"converged": 0, "nan or inf": 3, "accepted unconverged": 5}
    np.testing.assert_array_equal(np.array([[codes[s] for s in st] for st in statuses]), b[f"{config}_status"])
    np.testing.assert_array_equal(Y, b[f"{config}_Y"])


REFERENCE = __import__("pathlib").Path("/root/reference")
# fixture state -> the archived row of reference-results/ts1/runs.csv it was made with
SCORED = {
    ("ts1_tier1_30s", "Y"): ("alg", 1e-3),
    ("ts1_tier1_30s", "restart_Y"): ("restart", 1e-3),
    ("ts1_tier1_30s", "alg_elementary_Y"): ("alg-elementary", 5e-4),
    ("ts1_tier1_30s", "alg_noquant_Y"): ("alg-noquant", 5e-4),
    ("ts1_tier1_30s_backward_euler", "be_Y"): ("be", 1e-6),
    ("ts1_tier1_30s_backward_euler", "be_tight_3_Y"): ("be-tight", 1e-3),
}


@pytest.mark.skipif(not REFERENCE.exists(), reason="reference checkout not present")
@pytest.mark.parametrize("state", sorted(SCORED))
def test_oracle_score_reproduces_archived_digits(state):
    """The oracle's score (fastode/ts1.py:226-264) of the reference's final
    states on tier1-30s against the scenario's MICM reference table gives the
    archived digits, worst species, worst digits, gate and levels of
    reference-results/ts1/runs.csv (experiments/ts1_experiments.py:101-111)."""
    import csv
    import sys
    from oracle import scoring as OS
    sys.path.insert(0, str(REFERENCE))
    from fastode.ts1 import TS1
    species = TS1().species
    fixture, key = state
    config, rtol = SCORED[state]
    Y = load(fixture)[key]
    table = REFERENCE / "data/scenarios/tier1-30s/reference_final.csv"
    D, per, gate = OS.score({101: Y}, range(64), species, table)
    ws, wd, l2, l3 = OS.levels(D, per, gate)
    with open(REFERENCE / "reference-results/ts1/runs.csv") as fh:
        row = next(r for r in csv.DictReader(fh)
                   if r["config"] == config and r["scenario"] == "tier1-30s" and float(r["rtol"]) == rtol)
    assert round(D, 4) == float(row["digits"])
    assert ws == row["worst_species"] and round(wd, 4) == float(row["worst_digits"])
    assert (str(gate), str(l2), str(l3)) == (row["gate"], row["level2"], row["level3"])


def test_oracle_reproduces_the_measured_workload_subset():
    """The oracle on the measured 210-species / 500-reaction workload's parity
    subset (tests/golden/ros3_210x500_subset.npz, the reference run on eight
    seeded groups of the 65,536 cells): the first two intervals from the
    initial state, every group. Counts, statuses, every attempted step size
    and error norm bit for bit: the same NumPy and SciPy operations on the
    same inputs, with BLAS on one thread as the fixture was made (more
    threads block the forcing's matrix product differently, which moves the
    norms by up to 5e-9 relative)."""
    threadpoolctl = pytest.importorskip("threadpoolctl")
    f = load("ros3_210x500_subset")
    mech = mechanism_of(f)
    gs = int(f["group_size"])
    intervals = 2

    def k_of(i):
        k = np.array(f["k0"], copy=True)
        k[:, f["photo"]] = f["J"][None, :] * f["f"][i][:, None]
        return k

    with threadpoolctl.threadpool_limits(1):
        Y, counts, statuses, mems, traces = O.run_groups(
            mech, f["Y0"], k_of, float(f["dt"]), intervals, f["atol"], float(f["rtol"]), group_size=gs, trace=True)
    for g in range(len(f["groups"])):
        assert counts[g].as_tuple() == tuple(f["counts"][g, intervals - 1])
        assert [STATUS.index(s) for s in statuses[g]] == list(f["status"][g, :intervals])
        na = int((f["interval_of"][g, : int(f["n_attempts"][g])] < intervals).sum())
        assert len(traces[g]) == na
        assert [t[1] for t in traces[g]] == list(f["hs"][g, :na])
        assert [t[2] for t in traces[g]] == list(f["errs"][g, :na])
