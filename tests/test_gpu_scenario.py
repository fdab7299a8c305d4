"""The scenario driver and the accuracy scores on the device.

run_scenario (fastode/ts1.py:181-223) on TS1 tier1-30s, driven by stand-ins
for the reference's TS1, Cells and Scenario objects built from the fixture
(the rate constants the reference computed, the photolysis base values,
scaling factors and the scenario factor of every interval): the archived
Counts, the reference's final states, and the statuses of a backward Euler
configuration whose Newton iteration fails. score (fastode/ts1.py:226-264)
and digits (fastode/reference.py:41-59) on the device against the oracle's
restatement, which reproduces the archived digits of
reference-results/ts1/runs.csv."""
import numpy as np
import pytest

from golden_cases import load, rel_err, table_mechanism

pytestmark = pytest.mark.gpu


class FixtureTS1:
    """The attributes of fastode.ts1.TS1 that run_scenario reads."""

    def __init__(self, f):
        self.mech = table_mechanism(f)
        self.photolysis_reactions = [int(j) for j in f["photo"]]
        self.reactions = [{} for _ in range(self.mech.R)]
        for p, j in enumerate(self.photolysis_reactions):
            self.reactions[j] = {"MUSICA name": f"j_{p}", "scaling factor": float(f["scaling"][p])}
        self._k = np.asarray(f["k_static"])
        self._f0 = float(f["f"][0])
        self.index = {}

    def rate_constants(self, T, P, params):
        # the fixture's rate constants were computed with the photolysis
        # parameters scaled by the first interval's factor
        for p, j in enumerate(self.photolysis_reactions):
            assert np.array_equal(params[f"j_{p}"], self._base[:, p] * self._f0)
        return self._k.copy()


class FixtureCells:
    def __init__(self, f, ts1):
        self.C = f["Y0"].shape[0]
        self.Y = np.array(f["Y0"])
        self.T = np.full(self.C, 298.0)
        self.P = np.full(self.C, 101325.0)
        self.params = {f"j_{p}": np.array(f["base"][:, p]) for p in range(f["base"].shape[1])}
        ts1._base = np.asarray(f["base"])


class FixtureScenario:
    def __init__(self, f):
        self.steps = int(f["intervals"])
        self.dt = float(f["dt"])
        self._f = np.asarray(f["f"])

    def factor(self, t):
        return float(self._f[int(round(t / self.dt))])

    def snapshot_steps(self):
        return [50, self.steps]


def _standins():
    f = load("ts1_tier1_30s")
    ts1 = FixtureTS1(f)
    cells = FixtureCells(f, ts1)
    return f, ts1, cells, FixtureScenario(f)


def test_run_scenario_reproduces_the_archived_run(cuda):
    from fastode_gb300 import Algorithm
    from fastode_gb300.scenario import run_scenario
    f, ts1, cells, sc = _standins()
    snaps, counts, statuses = run_scenario(sc, Algorithm(), cells, ts1, 1e-3, 1e-17)
    assert statuses == []
    assert sorted(snaps) == [50, 101]
    np.testing.assert_array_equal(np.array(list(counts.as_dict().values())), f["counts"])
    assert rel_err(snaps[101], f["Y"]).max() <= 1e-8


def test_run_scenario_reports_statuses_in_reference_order(cuda):
    from fastode_gb300 import BackwardEuler
    from fastode_gb300.scenario import run_scenario
    f, ts1, cells, sc = _standins()
    b = load("ts1_tier1_30s_backward_euler")
    rtol, atol = b["be_it3_tol"]
    solver = BackwardEuler(max_iterations=3, reductions=(0.5, 0.25))
    snaps, counts, statuses = run_scenario(sc, solver, cells, ts1, float(rtol), float(atol),
                                           snapshots_on_device=True)
    names = {0: "converged", 3: "nan or inf", 5: "accepted unconverged"}
    want = [(g * 32, i, names[int(s)]) for g in range(2) for i, s in enumerate(b["be_it3_status"][g]) if s != 0]
    assert statuses == want
    np.testing.assert_array_equal(np.array(list(counts.as_dict().values())), b["be_it3_counts"])
    assert rel_err(snaps[101].cpu().numpy(), b["be_it3_Y"]).max() <= 1e-8


def _table(path, header, rows):
    with open(path, "w") as fh:
        fh.write(",".join(header) + "\n")
        for r in rows:
            fh.write(",".join(repr(float(v)) for v in r) + "\n")


@pytest.mark.parametrize("keyed", [False, True])
def test_score_matches_the_oracle(cuda, tmp_path, keyed):
    """Device score against the oracle on TS1 states: the backward Euler run
    scored against the Rosenbrock run at rtol 1e-3 as the reference table,
    over two snapshots, with unkeyed and (step, cell)-keyed tables, a cell
    subset, a species the result lacks and one the table lacks."""
    from fastode_gb300.scenario import score
    from oracle import scoring as OS
    f = load("ts1_tier1_30s")
    b = load("ts1_tier1_30s_backward_euler")
    n = f["Y"].shape[1]
    species = [f"s{i}" for i in range(n)]
    table_species = species[:-3] + ["not_in_result"]
    want = list(range(5, 61))
    ref = np.asarray(f["Y"])
    res = {50: np.asarray(b["be_Y"])[want], 101: np.asarray(b["be_tight_6_Y"])[want]}
    if keyed:
        header = ["step", "cell", "a", "b"] + table_species
        rows = [[s, c, 0.0, 0.0] + list(ref[c, :n - 3]) + [1.0] for s in (50, 101) for c in range(64)]
    else:
        header = ["cell", "a"] + table_species
        rows = [[c, 0.0] + list(ref[c, :n - 3]) + [1.0] for c in range(64)]
    path = tmp_path / "reference.csv"
    _table(path, header, rows)
    D, per, gate = score(res, want, species, path)
    Do, pero, gateo = OS.score(res, want, species, path)
    assert gate == gateo is True
    assert abs(D - Do) <= 1e-12 and set(per) == set(pero)
    assert max(abs(per[s] - pero[s]) for s in per) <= 1e-12
    # reproducible bit for bit
    assert score(res, want, species, path) == (D, per, gate)
    # the gate: a negative value below -1e-20 anywhere in a snapshot
    bad = {50: res[50].copy(), 101: res[101]}
    bad[50][3, 7] = -1e-18
    assert score(bad, want, species, path)[2] is False and OS.score(bad, want, species, path)[2] is False


def test_digits_matches_the_oracle(cuda):
    from fastode_gb300.scenario import digits
    from oracle import scoring as OS
    rng = np.random.default_rng(7)
    R = 10.0 ** rng.uniform(-20, -2, size=(300, 12))
    R[rng.random(R.shape) < 0.05] = np.nan                  # not a sample under reference >= threshold
    R[:, 4] = 1e-30                                         # a column with no samples
    X = R * (1.0 + 1e-6 * rng.standard_normal(R.shape))
    for cols in (None, [0, 2, 4, 11]):
        D, per = digits(X, R, 1e-14, cols)
        Do, pero = OS.digits(X, R, 1e-14, cols)
        assert abs(D - Do) <= 1e-12 and set(per) == set(pero)
        assert max(abs(per[j] - pero[j]) for j in per) <= 1e-12
    assert digits(X, R, 1.0)[0] == OS.digits(X, R, 1.0)[0] == 16.0     # no samples at all
