"""TS1 (209 species, 547 reactions with three-reactant rows) through the device
integrator on the reference's tier1-30s scenario: 64 cells in groups of 32,
101 intervals of 30 s, Algorithm(ROS3) at rtol 1e-3, atol 1e-17. The fixture
was made by running the reference's run_scenario (tests/golden/make_golden.py)
and its Counts equal the archived record reference-results/ts1/runs.csv
(alg, rtol 1e-3, tier1-30s: 334 steps, 330 accepted, 4 rejected)."""
import numpy as np
import pytest

from golden_cases import load, rel_err, table_mechanism, ts1_k

pytestmark = pytest.mark.gpu


# States within 1e-10 relative (floor a = 1e-14): the Counts and step sequences
# are the reference's, and what remains is roundoff of different summation
# orders (the reference's BLAS forcing and dense LU, the device's CSR sums and
# sparse LU) carried through 334 steps of a stiff system; the largest measured
# on a GB300 is 2.5e-11 (alg-nomemory), 1.8e-11 for the default controller.
STATE_TOL = 1e-10


@pytest.mark.parametrize("kernel", ["pipelined", "plain", "compact", "generated"])
def test_ts1_tier1_counts_match_the_archive(cuda, kernel):
    from fastode_gb300 import Algorithm
    from fastode_gb300.batch import Batch
    torch = cuda
    f = load("ts1_tier1_30s")
    mech = table_mechanism(f)
    b = Batch(mech, f["Y0"], group_size=int(f["group_size"]), algorithm=Algorithm(kernel=kernel))
    atol = torch.from_numpy(f["atol"]).cuda()
    for i in range(int(f["intervals"])):
        b.step(torch.from_numpy(np.ascontiguousarray(ts1_k(f, i).T)).cuda(), float(f["dt"]), atol, float(f["rtol"]))
        assert all(s == "converged" for s in b.statuses())
    total = b.counts.cpu().numpy().sum(axis=0)
    np.testing.assert_array_equal(total, f["counts"])
    assert total[0] == 334 and total[1] == 330 and total[2] == 4
    err = rel_err(b.state(), f["Y"])
    print(f"TS1 {kernel}: largest state difference {err.max():.3e}")
    assert err.max() <= STATE_TOL, err.max()


VARIANTS = {
    # name: (solver factory, fixture key)
    "alg-elementary": (lambda A, R, T: A(T, controller="elementary"), "alg_elementary"),
    "alg-noquant": (lambda A, R, T: A(T, quantize=False), "alg_noquant"),
    "alg-nomemory": (lambda A, R, T: A(T, carry_memory=False), "alg_nomemory"),
    "alg-reset": (lambda A, R, T: A(T, carry=False, quantize=False), "alg_reset"),
    "restart": (lambda A, R, T: R(T), "restart"),
}


@pytest.mark.parametrize("variant", sorted(VARIANTS))
def test_ts1_controller_variants_and_restarting_loop(cuda, variant):
    """The controller options of Algorithm (elementary controller, no
    quantization, no carried filter memory, no carried step) and the
    restarting loop on TS1 tier1-30s: the reference's Counts, which equal the
    archived rows of reference-results/ts1/runs.csv for these configurations
    (experiments/ts1_experiments.py:49-70)."""
    from fastode_gb300 import ROS3, Algorithm, RestartingLoop
    from fastode_gb300.batch import Batch
    torch = cuda
    f = load("ts1_tier1_30s")
    make, key = VARIANTS[variant]
    rtol, atol_v = f[f"{key}_tol"]
    mech = table_mechanism(f)
    b = Batch(mech, f["Y0"], group_size=int(f["group_size"]), algorithm=make(Algorithm, RestartingLoop, ROS3))
    atol = torch.full((mech.n,), float(atol_v), dtype=torch.float64, device="cuda")
    for i in range(int(f["intervals"])):
        b.step(torch.from_numpy(np.ascontiguousarray(ts1_k(f, i).T)).cuda(), float(f["dt"]), atol, float(rtol))
    np.testing.assert_array_equal(b.counts.cpu().numpy().sum(axis=0), f[f"{key}_counts"])
    worst = rel_err(b.state(), f[f"{key}_Y"]).max()
    print(f"TS1 {variant}: largest state difference {worst:.3e}")
    assert worst <= STATE_TOL


def _device_k(cuda, f):
    """TS1's first-interval rate constants on the device (fo_rate_laws) from
    the law records of tests/golden/ts1_rate_laws.npz."""
    import ctypes as C
    from fastode_gb300 import _abi
    from fastode_gb300.scenario import RATE_DTYPE
    torch = cuda
    laws = np.zeros(len(f["law_type"]), dtype=RATE_DTYPE)
    laws["type"], laws["column"], laws["c"] = f["law_type"], f["law_column"], f["law_c"]
    d = {name: torch.from_numpy(np.ascontiguousarray(v)).cuda() for name, v in
         dict(T=f["T"], P=f["P"], params=f["params"], power=f["power"]).items()}
    d_laws = torch.from_numpy(np.frombuffer(laws.tobytes(), dtype=np.uint8).copy()).cuda()
    Cc, R = f["k"].shape
    k = torch.empty((R, Cc), dtype=torch.float64, device="cuda")
    _abi.check(_abi.lib().fo_rate_laws(Cc, R, d_laws.data_ptr(), d["T"].data_ptr(), d["P"].data_ptr(),
                                       d["params"].data_ptr(), Cc, d["power"].data_ptr(), k.data_ptr(), 1, Cc,
                                       None), "fo_rate_laws")
    torch.cuda.synchronize()
    return k.cpu().numpy().T


# Largest difference from the reference's rate constants, in units in the last
# place; exp, pow and log10 on the device and in NumPy are each within an ulp
# or two of the exact value, and a Troe row chains several of them.
RATE_ULPS = 16


def test_device_rate_laws_match_the_reference(cuda):
    f = load("ts1_rate_laws")
    got, ref = _device_k(cuda, f), f["k"]
    assert np.array_equal(got == 0.0, ref == 0.0)
    nz = ref != 0.0
    ulps = np.abs(got[nz] - ref[nz]) / np.spacing(np.abs(ref[nz]))
    exact = float(np.mean(got[nz] == ref[nz]))
    print(f"rate laws: largest difference {ulps.max():.1f} ulp, {100 * exact:.1f}% bit-identical")
    assert ulps.max() <= RATE_ULPS, ulps.max()


@pytest.mark.parametrize("kernel", ["generated", "compact"])
def test_ts1_with_device_rate_constants_reproduces_the_archive(cuda, kernel):
    """The archived run (334 steps, 330 accepted, 4 rejected) with every rate
    constant made on the device: the first interval's from the rate laws, the
    photolysis columns of later intervals patched as run_scenario does."""
    from fastode_gb300 import Algorithm
    from fastode_gb300.batch import Batch
    torch = cuda
    f = load("ts1_tier1_30s")
    k0 = _device_k(cuda, load("ts1_rate_laws"))
    mech = table_mechanism(f)
    b = Batch(mech, f["Y0"], group_size=int(f["group_size"]), algorithm=Algorithm(kernel=kernel))
    atol = torch.from_numpy(f["atol"]).cuda()
    for i in range(int(f["intervals"])):
        k = np.array(k0, copy=True)
        if i > 0:
            k[:, f["photo"]] = (f["base"] * f["f"][i]) * f["scaling"][None, :]
        b.step(torch.from_numpy(np.ascontiguousarray(k.T)).cuda(), float(f["dt"]), atol, float(f["rtol"]))
    total = b.counts.cpu().numpy().sum(axis=0)
    np.testing.assert_array_equal(total, f["counts"])
    assert total[0] == 334 and total[1] == 330 and total[2] == 4
    worst = rel_err(b.state(), f["Y"]).max()
    print(f"TS1 device rate constants {kernel}: largest state difference {worst:.3e}")
    assert worst <= STATE_TOL
