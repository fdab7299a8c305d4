"""The host-array entry points: ``solve_host`` (one interval per call, the
reference's calling pattern) against the oracle, and ``solve_host_intervals``
(copies overlapped with the integration) against repeated ``solve_host``
calls, bit for bit."""
import numpy as np
import pytest

from golden_cases import rel_err

pytestmark = pytest.mark.gpu


def _workload():
    from fastode_gb300 import synthetic as syn
    return syn.plain_small(n_cells=96, intervals=5)


def test_solve_host_matches_the_oracle(cuda):
    from oracle import rosenbrock as O
    from fastode_gb300.batch import solve_host
    wl = _workload()
    ks = [wl.k_at(i) for i in range(wl.intervals)]
    Y, state = wl.cells.Y0.copy(), None
    for i in range(wl.intervals):
        Yt, state, _ = solve_host(wl.sm.mech, Y, ks[i], wl.dt, wl.atol, wl.rtol, state=state)
        Y = Yt.numpy().copy()
    Yo, co, so, _, _ = O.run_groups(wl.sm.mech, wl.cells.Y0, lambda i: ks[i], wl.dt, wl.intervals, wl.atol, wl.rtol)
    counts = state.counts.cpu().numpy()
    for g in range(state.ngroups):
        assert tuple(counts[g]) == co[g].as_tuple()
    assert rel_err(Y, Yo).max() <= 1e-10


def test_overlapped_intervals_match_one_call_per_interval(cuda):
    import torch
    from fastode_gb300.batch import solve_host, solve_host_intervals
    wl = _workload()
    ks = [torch.from_numpy(wl.k_at(i)).pin_memory() for i in range(wl.intervals)]
    Y, s1, per_call = wl.cells.Y0.copy(), None, []
    for i in range(wl.intervals):
        Yt, s1, _ = solve_host(wl.sm.mech, Y, ks[i], wl.dt, wl.atol, wl.rtol, state=s1)
        Y = Yt.numpy().copy()
        per_call.append((Y.copy(), s1.status_out.numpy().copy()))
    got = {}

    def keep(i, Yh, st):
        got[i] = (Yh.numpy().copy(), st.numpy().copy())

    Ylast, s2, (h2d, d2h) = solve_host_intervals(wl.sm.mech, wl.cells.Y0, ks, wl.dt, wl.atol, wl.rtol,
                                                 on_result=keep)
    assert sorted(got) == list(range(wl.intervals))
    for i in range(wl.intervals):
        np.testing.assert_array_equal(got[i][0], per_call[i][0])
        np.testing.assert_array_equal(got[i][1], per_call[i][1])
    np.testing.assert_array_equal(Ylast.numpy(), per_call[-1][0])
    np.testing.assert_array_equal(s1.counts.cpu().numpy(), s2.counts.cpu().numpy())
    C, n = wl.cells.Y0.shape
    R = ks[0].shape[1]
    assert h2d == C * n * 8 + n * 8 + wl.intervals * C * R * 8
    assert d2h == wl.intervals * (C * n * 8 + s2.ngroups * 4)
