"""The reference's controller and step-rule tests (tests/test_fastode.py:96-208),
run through the drop-in ``Algorithm.solve`` on the GPU. The reference writes
them with DenseSystem lambdas for y' = -lam*y; here the same equation is the
mass-action mechanism A -> (nothing) with k = lam, which the device runs."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def decay(lam):
    from fastode_gb300 import ChemSystem, Mechanism
    return ChemSystem(Mechanism(["A"], [(["A"], [])]), np.array([[lam]]))


def test_carried_step_takes_one_step(cuda):
    # tests/test_fastode.py:96-110
    from fastode_gb300 import ROS3, Algorithm, Counts
    sys_ = decay(1e-6)
    alg = Algorithm(ROS3)
    mem = alg.new_memory()
    Y = np.array([[1.0]])
    c2 = Counts()
    for _ in range(5):
        Y, _ = alg.solve(sys_, Y, 600.0, np.array([1e-10]), 1e-3, c2, mem)
    c3 = Counts()
    alg.solve(sys_, Y, 600.0, np.array([1e-10]), 1e-3, c3, mem)
    assert c3.accepted == 1


def test_quantized_steps_land_on_the_interval_end(cuda):
    # tests/test_fastode.py:113-125
    from fastode_gb300 import ROS3, Algorithm, Counts
    sys_ = decay(1e-9)
    alg = Algorithm(ROS3, fac_max=1.0)
    mem = alg.new_memory()
    mem.h_next = 600.0 / 7
    Y = np.array([[1.0]])
    for _ in range(3):
        c = Counts()
        Y, st = alg.solve(sys_, Y, 600.0, np.array([1e-10]), 1e-3, c, mem)
        assert st == "converged" and c.steps == 7
        assert abs(mem.h_next - 600.0 / 7) < 1e-9


def test_a_rejection_shrinks_the_step(cuda):
    # tests/test_fastode.py:128-136
    from fastode_gb300 import ROS3, Algorithm, Counts
    alg = Algorithm(ROS3)
    mem = alg.new_memory()
    mem.h_next, mem.err_prev, mem.h_prev = 1.0, 1e-8, 1.0
    c = Counts()
    alg.solve(decay(1.0), np.array([[1.0]]), 1.0, np.array([1e-12]), 4e-3, c, mem)
    assert c.rejected == 1


def test_no_forced_acceptance_below_minimum_step(cuda):
    # tests/test_fastode.py:152-169
    from fastode_gb300 import ROS3, Algorithm, Counts
    alg = Algorithm(ROS3, max_steps=10)
    mem = alg.new_memory()
    mem.h_next = 1e-15
    initial, counts = np.array([[1.0]]), Counts()
    result, status = alg.solve(decay(1e15), initial, 1.0, np.array([1e-30]), 1e-12, counts, mem)
    assert status == "step too small"
    assert counts.steps == counts.rejected == 1
    assert counts.accepted == 0
    np.testing.assert_array_equal(result, initial)


@pytest.mark.parametrize("budget", [0, 1, 2])
def test_budget_includes_rejected_retries(cuda, budget):
    # tests/test_fastode.py:172-187
    from fastode_gb300 import ROS3, Algorithm, Counts
    alg = Algorithm(ROS3, max_steps=budget)
    mem = alg.new_memory()
    mem.h_next = 1.0
    initial, counts = np.array([[1.0]]), Counts()
    result, status = alg.solve(decay(1.0), initial, 1.0, np.array([1e-30]), 1e-13, counts, mem)
    assert status == "too many steps"
    assert counts.steps == counts.rejected == budget
    assert counts.accepted == 0
    np.testing.assert_array_equal(result, initial)


@pytest.mark.parametrize("budget, expected_status", [(2, "too many steps"), (10, "converged")])
def test_budget_includes_accepted_steps(cuda, budget, expected_status):
    # tests/test_fastode.py:190-208
    from fastode_gb300 import ROS3, Algorithm, Counts
    alg = Algorithm(ROS3, max_steps=budget, fac_max=1.0)
    mem = alg.new_memory()
    mem.h_next = 0.1
    counts = Counts()
    _, status = alg.solve(decay(1e-6), np.array([[1.0]]), 1.0, np.array([1e-10]), 1e-3, counts, mem)
    assert status == expected_status
    assert counts.steps == counts.accepted == budget
    assert counts.rejected == 0


@pytest.mark.parametrize("bad", [np.nan, np.inf])
def test_nan_or_inf_status(cuda, bad):
    """A non-finite state ends the call with "nan or inf" after one counted
    attempt, and the returned state is the (clamped) input."""
    from fastode_gb300 import ROS3, Algorithm, Counts
    from oracle import rosenbrock as O
    from fastode_gb300 import Mechanism
    mech = Mechanism(["A", "B"], [(["A"], [("B", 1.0)])])
    from fastode_gb300 import ChemSystem
    y0 = np.array([[bad, 1.0], [1.0, 2.0]])
    c = Counts()
    y, st = Algorithm(ROS3).solve(ChemSystem(mech, np.array([[1e-3]])), y0, 10.0, np.full(2, 1e-12), 1e-3, c)
    co = O.OCounts()
    yo, sto = O.OAlgorithm().solve(O.OChem(mech, np.array([[1e-3]])), y0, 10.0, np.full(2, 1e-12), 1e-3, co)
    assert st == sto == "nan or inf"
    assert tuple(c.as_dict().values()) == co.as_tuple()
    np.testing.assert_array_equal(np.isnan(y), np.isnan(yo))
    np.testing.assert_array_equal(y[np.isfinite(yo)], yo[np.isfinite(yo)])


def test_rodas3_without_constraints_matches_oracle(cuda):
    """RODAS3 (four stages, the forcing reuse of stage 1) on a small mechanism."""
    from fastode_gb300 import RODAS3, Algorithm, ChemSystem, Counts, Mechanism
    from oracle import rosenbrock as O
    mech = Mechanism(["A", "B", "C"], [(["A"], [("B", 1.0)]), (["B", "B"], [("B", 1.0), ("C", 1.0)]),
                                       (["B", "C"], [("A", 1.0), ("C", 1.0)])])
    k = np.array([[0.04, 3.0e7, 1.0e4]])
    Y = np.array([[1.0, 0.0, 0.0]])
    Yo = Y.copy()
    alg = Algorithm(RODAS3)
    oalg = O.OAlgorithm(O.ORODAS3)
    mem, omem = alg.new_memory(), O.OMemory()
    c, co = Counts(), O.OCounts()
    for _ in range(10):
        Y, st = alg.solve(ChemSystem(mech, k), Y, 1.0, np.full(3, 1e-12), 1e-4, c, mem)
        Yo, sto = oalg.solve(O.OChem(mech, k), Yo, 1.0, np.full(3, 1e-12), 1e-4, co, omem)
        assert st == sto
    assert tuple(c.as_dict().values()) == co.as_tuple()
    assert np.max(np.abs(Y - Yo) / np.maximum(np.abs(Yo), 1e-14)) < 1e-10


def test_dense_system_is_rejected(cuda):
    """A system given by Python callables cannot run on the device, and there
    is no CPU fallback."""
    from fastode_gb300 import ROS3, Algorithm, Counts

    class Lambdas:
        n = 1
        mass = np.ones(1)

        def rhs(self, Y):
            return -Y

    with pytest.raises(TypeError):
        Algorithm(ROS3).solve(Lambdas(), np.array([[1.0]]), 1.0, np.array([1e-10]), 1e-3, Counts())
