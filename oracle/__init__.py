"""CPU oracle for the Rosenbrock hot path — TEST INFRASTRUCTURE ONLY.

A NumPy/SciPy restatement of the reference's integrator
(davidfillmore/Fast-ODE-Atmospheric-Chem, fastode/solvers.py, chem.py,
linalg.py). Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline
legs may import it, and only as the checker or the timed CPU baseline; the
product package never imports it.

Pinned: tests/test_oracle_pin.py checks the oracle against golden vectors made
by running the reference itself (tests/golden/make_golden.py): identical
Counts, statuses and memory, and bit-identical states where both sides run the
same NumPy/SciPy operations.
"""
