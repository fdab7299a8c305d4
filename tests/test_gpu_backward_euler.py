"""BackwardEuler (fastode/solvers.py:418-491) on the device.

TS1 tier1-30s, 64 cells in groups of 32 over 101 intervals of 30 s, in the
five configurations of tests/golden/ts1_tier1_30s_backward_euler.npz (made by
running the reference's BackwardEuler through its run_scenario): the three
archived ones of reference-results/ts1/runs.csv (be at rtol 1e-6, atol 1e-3;
be-tight at rtol 1e-3 and 1e-6, atol 1e-15) and two whose Newton iteration is
cut short (max_iterations 2 or 3), so that failed steps, step cuts, doubling
after two successes and accepted unconverged iterates all occur. Counts and
per-interval statuses must equal the reference's; states agree to roundoff of
the two LU factorizations (pivot-free here, SuperLU there)."""
import ctypes as C

import numpy as np
import pytest

from golden_cases import load, mechanism_of, rel_err, table_mechanism, ts1_k

pytestmark = pytest.mark.gpu

CONFIGS = ["be", "be_tight_3", "be_tight_6", "be_it2", "be_it3"]
Y_TOL = 1e-8   # relative, floor 1e-14: roundoff of the LU, carried over 101 intervals


def _solver(b, config, kernel="pipelined"):
    from fastode_gb300 import BackwardEuler
    return BackwardEuler(max_iterations=int(b[f"{config}_max_iterations"]),
                         reductions=tuple(float(r) for r in b[f"{config}_reductions"]), kernel=kernel)


def _run(torch, f, b, config, kernel="pipelined"):
    from fastode_gb300.batch import Batch
    mech = table_mechanism(f)
    rtol, atol_v = b[f"{config}_tol"]
    batch = Batch(mech, f["Y0"], group_size=32, algorithm=_solver(b, config, kernel))
    atol = torch.full((mech.n,), float(atol_v), dtype=torch.float64, device="cuda")
    codes = {s: i for i, s in enumerate(("converged", "too many steps", "step too small", "nan or inf",
                                         "projection failed", "accepted unconverged"))}
    status = []
    for i in range(int(f["intervals"])):
        batch.step(torch.from_numpy(np.ascontiguousarray(ts1_k(f, i).T)).cuda(), float(f["dt"]), atol, float(rtol))
        status.append([codes[s] for s in batch.statuses()])
    return batch, np.array(status).T


@pytest.mark.parametrize("config", CONFIGS)
def test_backward_euler_ts1_matches_reference(cuda, config):
    torch = cuda
    f = load("ts1_tier1_30s")
    b = load("ts1_tier1_30s_backward_euler")
    batch, status = _run(torch, f, b, config)
    total = batch.counts.cpu().numpy().sum(axis=0)
    np.testing.assert_array_equal(total, b[f"{config}_counts"])
    np.testing.assert_array_equal(status, b[f"{config}_status"])
    err = rel_err(batch.state(), b[f"{config}_Y"])
    print(f"BackwardEuler {config}: largest state difference {err.max():.3e}")
    assert err.max() <= Y_TOL, err.max()


@pytest.mark.parametrize("kernel", ["plain", "compact", "generated"])
def test_backward_euler_other_kernels(cuda, kernel):
    """The plain LU loops, the compact kernel and the generated code give the
    same Counts on the configuration with failed steps."""
    torch = cuda
    f = load("ts1_tier1_30s")
    b = load("ts1_tier1_30s_backward_euler")
    batch, status = _run(torch, f, b, "be_it3", kernel=kernel)
    np.testing.assert_array_equal(batch.counts.cpu().numpy().sum(axis=0), b["be_it3_counts"])
    np.testing.assert_array_equal(status, b["be_it3_status"])
    worst = rel_err(batch.state(), b["be_it3_Y"]).max()
    print(f"BackwardEuler be_it3 {kernel}: largest state difference {worst:.3e}")
    assert worst <= Y_TOL


def test_backward_euler_drop_in_solve_matches_oracle(cuda):
    """BackwardEuler.solve with the reference's signature (host arrays, one
    group per call, memory None) against the oracle on the 20-species
    synthetic mechanism."""
    from fastode_gb300 import BackwardEuler, ChemSystem, Counts
    from oracle import rosenbrock as O
    f = load("ros3_20x40")
    mech = mechanism_of(f)
    solver = BackwardEuler()
    assert solver.new_memory() is None
    Y = f["Y0"][:32].copy()
    Yo = Y.copy()
    c, co = Counts(), O.OCounts()
    oracle = O.OBackwardEuler()
    for i in range(6):
        k = f["k"][i][:32]
        Y, st = solver.solve(ChemSystem(mech, k), Y, float(f["dt"]), f["atol"], 1e-6, c)
        Yo, sto = oracle.solve(O.OChem(mech, k), Yo, float(f["dt"]), f["atol"], 1e-6, co)
        assert st == sto
    assert tuple(c.as_dict().values()) == co.as_tuple()
    assert rel_err(Y, Yo).max() <= 1e-10


def test_backward_euler_rejects_bad_reductions_through_the_abi(cuda):
    """A non-positive reduction would never let the step loop end: the C-ABI
    refuses it with FO_E_INVALID before launching anything."""
    from fastode_gb300 import _abi
    from fastode_gb300.plan import plan_for
    torch = cuda
    f = load("ros3_20x40")
    mech = mechanism_of(f)
    plan = plan_for(mech)
    o = _abi.Options()
    o.loop = _abi.LOOPS["backward-euler"]
    o.max_iterations = 11
    o.max_steps = 1000
    o.nreductions = 2
    o.reductions[0] = 0.5
    o.reductions[1] = 0.0
    Yd = torch.from_numpy(np.ascontiguousarray(f["Y0"][:32].T)).cuda()
    kd = torch.from_numpy(np.ascontiguousarray(f["k"][0][:32].T)).cuda()
    atol = torch.from_numpy(f["atol"]).cuda()
    mem = torch.zeros(3, dtype=torch.float64, device="cuda")
    cnt = torch.zeros(13, dtype=torch.int64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    offs = torch.tensor([0, 32], dtype=torch.int32, device="cuda")
    ws = plan.workspace(1, 32)
    rc = _abi.lib().fo_solve(plan.handle, C.byref(o), 1, offs.data_ptr(), 32, Yd.data_ptr(), 1, 32,
                             kd.data_ptr(), 1, 32, atol.data_ptr(), 1e-3, 30.0, mem.data_ptr(), cnt.data_ptr(),
                             st.data_ptr(), ws.data_ptr(), ws.numel(), 0, None, 0, None, None)
    assert rc == _abi.FO_E_INVALID
    assert b"reductions" in _abi.lib().fo_last_error()
