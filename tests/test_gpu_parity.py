"""Parity of the device integrator with the reference (golden fixtures made by
the reference itself) and with the oracle, through the C-ABI.

The bar (the reference's own outputs on the same inputs):
  * Counts per group and status per group and interval: identical;
  * the attempted step sizes: identical (they are quantized divisors of dt);
  * the error norm per attempt: within 1e-8 relative plus 1e-7 absolute, in
    units of the acceptance threshold err < 1 (the device LU is pivot-free in
    its own order, SuperLU pivots, so roundoff differs; an error norm near
    1e-10 is itself roundoff and may differ in its leading digits);
  * final states: within 1e-10 relative, floored at a = 1e-14.
"""
import numpy as np
import pytest

from golden_cases import CASES, load, mechanism_of, rel_err

pytestmark = pytest.mark.gpu

STATE_RTOL = 1e-10
ERR_RTOL = 1e-8
ERR_ATOL = 1e-7


def run_batch(cuda, f, trace_cap=64, slots=0, group_size=None, kernel="pipelined"):
    from fastode_gb300 import Algorithm
    from fastode_gb300.batch import Batch
    torch = cuda
    mech = mechanism_of(f)
    gs = int(f["group_size"]) if group_size is None else group_size
    b = Batch(mech, f["Y0"], group_size=gs, trace_cap=trace_cap, slots=slots, algorithm=Algorithm(kernel=kernel))
    atol = torch.from_numpy(f["atol"]).cuda()
    traces = [[] for _ in range(b.ngroups)]
    statuses = []
    for i in range(int(f["intervals"])):
        k = torch.from_numpy(np.ascontiguousarray(f["k"][i].T)).cuda()
        b.step(k, float(f["dt"]), atol, float(f["rtol"]))
        torch.cuda.synchronize()
        statuses.append(b.status.cpu().numpy().copy())
        if trace_cap:
            tl = b.trace_len.cpu().numpy()
            tr = b.trace.cpu().numpy()
            for g in range(b.ngroups):
                assert tl[g] <= trace_cap
                traces[g].extend(tr[g, : tl[g]].tolist())
    return b, np.array(statuses).T, traces


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kernel", ["pipelined", "plain", "compact", "generated"])
def test_device_matches_reference_fixture(cuda, case, kernel):
    f = load(case)
    b, statuses, traces = run_batch(cuda, f, kernel=kernel)
    counts = b.counts.cpu().numpy()
    np.testing.assert_array_equal(counts, f["counts"])
    np.testing.assert_array_equal(statuses, f["status"])
    mem = b.memory.cpu().numpy()
    np.testing.assert_array_equal(mem[:, 0], f["memory"][:, 0])      # h_next: quantized
    np.testing.assert_array_equal(mem[:, 2], f["memory"][:, 2])      # h_prev
    np.testing.assert_allclose(mem[:, 1], f["memory"][:, 1], rtol=ERR_RTOL, atol=ERR_ATOL)
    for g in range(b.ngroups):
        na = int(f["n_attempts"][g])
        tr = np.array(traces[g])
        assert len(tr) == na
        np.testing.assert_array_equal(tr[:, 1], f["hs"][g, :na])
        np.testing.assert_allclose(tr[:, 2], f["errs"][g, :na], rtol=ERR_RTOL, atol=ERR_ATOL)
        np.testing.assert_array_equal(tr[:, 3], (f["errs"][g, :na] < 1.0).astype(float))
    Y = b.state()
    assert rel_err(Y, f["Y"]).max() <= STATE_RTOL


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kernel", ["pipelined", "compact"])
def test_persistent_queue_gives_the_same_bits(cuda, case, kernel):
    """A persistent launch that pulls groups from the device queue computes
    exactly what one block per group computes."""
    f = load(case)
    b0, s0, _ = run_batch(cuda, f, trace_cap=0, kernel=kernel)
    b1, s1, _ = run_batch(cuda, f, trace_cap=0, slots=1, kernel=kernel)
    np.testing.assert_array_equal(b0.state(), b1.state())
    np.testing.assert_array_equal(b0.counts.cpu().numpy(), b1.counts.cpu().numpy())
    np.testing.assert_array_equal(s0, s1)


def test_dropin_solve_matches_fixture(cuda):
    """The reference-signature drop-in, group by group and interval by
    interval, gives the fixture's Counts and states."""
    from fastode_gb300 import Algorithm, ChemSystem, Counts, ROS3
    f = load("ros3_20x40")
    mech = mechanism_of(f)
    alg = Algorithm(ROS3)
    gs = int(f["group_size"])
    Y = f["Y0"].copy()
    for g in range(f["counts"].shape[0]):
        sl = slice(g * gs, (g + 1) * gs)
        mem = alg.new_memory()
        c = Counts()
        Yg = Y[sl]
        for i in range(int(f["intervals"])):
            Yg, st = alg.solve(ChemSystem(mech, f["k"][i][sl]), Yg, float(f["dt"]), f["atol"], float(f["rtol"]), c, mem)
            assert st == "converged"
        Y[sl] = Yg
        assert tuple(c.as_dict().values()) == tuple(f["counts"][g])
        assert mem.h_next == f["memory"][g, 0]
    assert rel_err(Y, f["Y"]).max() <= STATE_RTOL


@pytest.mark.parametrize("case", CASES)
def test_rhs_and_jacobian_match_oracle(cuda, case):
    from fastode_gb300 import ChemSystem
    from oracle.rosenbrock import OChem
    f = load(case)
    mech = mechanism_of(f)
    Y = f["Y0"]
    k = f["k"][0]
    ours = ChemSystem(mech, k, dense=False)
    ref = OChem(mech, k, dense=False)
    # Jacobian values: the same products summed in the reference's CSR order;
    # SciPy's compiled matvec may contract into FMA, so allow a few ulps of the
    # absolute sum of the terms
    J, Jr = ours.jac(Y), ref.jac_values(Y)
    absref = OChem(mech, np.abs(k), dense=False)
    absref.GT = abs(ref.GT)
    jscale = absref.jac_values(np.abs(Y))
    assert np.all(np.abs(J - Jr) <= 4e-16 * 8 * jscale + 1e-300)
    # forcing: the reference sums with a BLAS GEMM, the device in CSR order
    F, Fr = ours.rhs(Y), ref.rhs(Y)
    scale = np.abs(ref.rates(Y)) @ np.abs(ref.ST)
    assert np.all(np.abs(F - Fr) <= 1e-14 * scale + 1e-300)


@pytest.mark.parametrize("kernel", ["pipelined", "compact"])
def test_ragged_groups_and_idle_lanes(cuda, kernel):
    """Groups of 20 and 12 cells (idle lanes in the warp) give the oracle's
    Counts and states for those groups."""
    from oracle import rosenbrock as O
    from fastode_gb300 import Algorithm
    f = load("ros3_20x40")
    mech = mechanism_of(f)
    torch = cuda
    from fastode_gb300.batch import Batch
    offs = np.array([0, 20, 32, 64], dtype=np.int32)
    b = Batch(mech, f["Y0"], offsets=offs, algorithm=Algorithm(kernel=kernel))
    atol = torch.from_numpy(f["atol"]).cuda()
    n_int = 5
    for i in range(n_int):
        b.step(torch.from_numpy(np.ascontiguousarray(f["k"][i].T)).cuda(), float(f["dt"]), atol, float(f["rtol"]))
    Y = b.state()
    counts = b.counts.cpu().numpy()
    for g in range(3):
        sl = slice(offs[g], offs[g + 1])
        alg = O.OAlgorithm(O.OROS3)
        mem, c = O.OMemory(), O.OCounts()
        Yg = f["Y0"][sl].copy()
        for i in range(n_int):
            Yg, _ = alg.solve(O.OChem(mech, f["k"][i][sl]), Yg, float(f["dt"]), f["atol"], float(f["rtol"]), c, mem)
        assert tuple(counts[g]) == c.as_tuple()
        assert rel_err(Y[sl], Yg).max() <= STATE_RTOL
