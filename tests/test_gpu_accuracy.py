"""Accuracy against a tight solve: on the same inputs the device's error
against an FP64 rtol = 1e-10 solution equals the reference's error, and the
device's own tight solve agrees with that solution.

The tight solution is the reference's algorithm (the oracle) at rtol = 1e-10,
atol = 1e-10 * a (a = 1e-14), on the 20-species synthetic case (64 cells, 20
intervals of 30 s); errors are Sandu digits over all species with reference
values above a (fastode/reference.py:41-59)."""
import numpy as np
import pytest

from golden_cases import A_FLOOR, load, mechanism_of, rel_err

pytestmark = pytest.mark.gpu


def _device(torch, f, mech, rtol, atol, max_steps=1000):
    from fastode_gb300 import Algorithm
    from fastode_gb300.batch import Batch
    b = Batch(mech, f["Y0"], group_size=32, algorithm=Algorithm(max_steps=max_steps))
    at = torch.from_numpy(np.ascontiguousarray(atol)).cuda()
    for i in range(int(f["intervals"])):
        b.step(torch.from_numpy(np.ascontiguousarray(f["k"][i].T)).cuda(), float(f["dt"]), at, rtol)
    assert all(s == "converged" for s in b.statuses())
    return b.state()


def test_error_against_a_tight_solve_equals_the_references(cuda):
    from oracle import rosenbrock as O
    from oracle.scoring import digits
    torch = cuda
    f = load("ros3_20x40")
    mech = mechanism_of(f)
    tight_atol = np.full(mech.n, 1e-10 * A_FLOOR)
    Y_tight, counts, statuses, _, _ = O.run_groups(
        mech, f["Y0"], lambda i: f["k"][i], float(f["dt"]), int(f["intervals"]), tight_atol, 1e-10,
        group_size=32, max_steps=100000)
    assert all(s == "converged" for st in statuses for s in st)
    # the device at the fixture's tolerance, against the reference's own result
    Y_gpu = _device(torch, f, mech, float(f["rtol"]), f["atol"])
    d_gpu, _ = digits(Y_gpu, Y_tight, A_FLOOR)
    d_ref, _ = digits(f["Y"], Y_tight, A_FLOOR)
    assert abs(d_gpu - d_ref) <= 1e-5, (d_gpu, d_ref)
    assert d_ref > 5.0
    # the device's own tight solve
    Y_gpu_tight = _device(torch, f, mech, 1e-10, tight_atol, max_steps=100000)
    assert rel_err(Y_gpu_tight, Y_tight).max() <= 1e-8
