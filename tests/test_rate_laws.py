"""TS1's rate laws as fo_rate_law records (scenario.rate_law_table), checked on
the CPU: the oracle's NumPy restatement of fastode.ts1.TS1.rate_constants
(fastode/ts1.py:66-103) over those records reproduces the reference's own rate
constants bit for bit (tests/golden/ts1_rate_laws.npz, made by running the
reference), and the records compiled from the reference's TS1 object equal
the fixture's."""
import sys
from pathlib import Path

import numpy as np
import pytest

from golden_cases import load

REFERENCE = Path("/root/reference")


def test_law_records_reproduce_the_reference_rate_constants():
    from oracle.ts1_rates import rate_constants
    f = load("ts1_rate_laws")
    k = rate_constants(f["law_type"], f["law_column"], f["law_c"], f["params"], f["T"], f["P"], f["power"])
    np.testing.assert_array_equal(k, f["k"])


def test_law_table_compiled_from_the_reference_mechanism():
    if not (REFERENCE / "fastode").is_dir():
        pytest.skip("the reference checkout is not on this host")
    sys.path.insert(0, str(REFERENCE))
    from fastode.ts1 import TS1
    from fastode_gb300.scenario import rate_law_table
    f = load("ts1_rate_laws")
    laws, columns = rate_law_table(TS1())
    np.testing.assert_array_equal(laws["type"], f["law_type"])
    np.testing.assert_array_equal(laws["column"], f["law_column"])
    np.testing.assert_array_equal(laws["c"], f["law_c"])
    assert list(columns) == [str(c) for c in f["columns"]]


def test_unknown_rate_type_is_not_compiled():
    from fastode_gb300.scenario import rate_law_table

    class Mech:
        reactions = [{"type": "ARRHENIUS", "A": 1.0}, {"type": "WENNBERG_NO_RO2"}]
        props = {}
    assert rate_law_table(Mech()) is None
