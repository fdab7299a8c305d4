"""Parity on the measured workload: the 210-species / 500-reaction, 65,536-cell
job, on its seeded subset of eight whole groups (synthetic.PLAIN_LARGE_PARITY_GROUPS)
over its first 30 intervals, against the reference run on the same cells
(tests/golden/ros3_210x500_subset.npz, made by make_golden.py --only c2-subset;
fastode/solvers.py:305-415 through the loop of fastode/ts1.py:196-222).

The inputs are the fixture's own (Y0, the rate constants at t = 0 and every
interval's diurnal factors), and the device builds each interval's rate
constants from them with fo_photolysis_factor, as bench.py does: the
photolysis columns are J * f, one IEEE product, so the device integrates
exactly the reference's k. The bar:
  * Counts after every interval, per group: identical (cumulative);
  * status per group and interval: identical;
  * every attempted step size, in order: identical;
  * every error norm: within 1e-8 relative plus 1e-7 absolute (the LUs differ
    in roundoff: SuperLU pivots, the device factors pivot-free);
  * states at intervals 10, 20 and 30: within STATE_RTOL relative, floored at
    a = 1e-14;
  * accuracy: the device's Sandu digits against the reference's own FP64
    rtol = 1e-10, atol = 1e-10 * a solve of the same cells (intervals 10 and
    20) equal the reference's rtol = 1e-3 digits to 1e-6.
"""
import numpy as np
import pytest

from golden_cases import load, mechanism_of, rel_err

pytestmark = pytest.mark.gpu

ERR_RTOL = 1e-8
ERR_ATOL = 1e-7
# Final states relative to the reference, floored at a = 1e-14: the largest
# measured difference over the 30 intervals is recorded in MEASURED below.
STATE_RTOL = 1e-10


def _k_builder(cuda, f):
    """Device (R, C) rate constants of interval i from the fixture's inputs."""
    from fastode_gb300 import _abi
    torch = cuda
    k0 = torch.from_numpy(np.ascontiguousarray(f["k0"].T)).cuda()
    rxn = torch.from_numpy(f["photo"].astype(np.int32)).cuda()
    J = torch.from_numpy(f["J"]).cuda()
    fac = torch.from_numpy(np.ascontiguousarray(f["f"])).cuda()
    R, C = k0.shape
    k = k0.clone()

    def at(i):
        _abi.check(_abi.lib().fo_photolysis_factor(C, rxn.numel(), rxn.data_ptr(), J.data_ptr(),
                                                   fac[i].data_ptr(), k.data_ptr(), 1, C, None),
                   "fo_photolysis_factor")
        return k
    return at


def _host_k(f, i):
    k = np.array(f["k0"], copy=True)
    k[:, f["photo"]] = f["J"][None, :] * f["f"][i][:, None]
    return k


def test_device_rate_constants_are_the_fixture_inputs(cuda):
    f = load("ros3_210x500_subset")
    at = _k_builder(cuda, f)
    for i in (0, 7, 29):
        k = at(i)
        cuda.cuda.synchronize()
        np.testing.assert_array_equal(k.cpu().numpy().T, _host_k(f, i))


def test_device_rate_constants_match_the_generator(cuda):
    """The construction bench.py uses (host thermal k, device J * f) reproduces
    synthetic.rate_constants / Workload.k_at bit for bit on this host."""
    from fastode_gb300 import synthetic as syn
    torch = cuda
    f = load("ros3_210x500_subset")
    wl = syn.plain_large().subset(f["cells"])
    photo = np.nonzero(wl.sm.photolytic)[0].astype(np.int32)
    fac = syn.photolysis_factors(wl.cells, wl.dt, 3)
    g = dict(f, k0=wl.k_at(0), photo=photo, J=wl.sm.J[photo], f=fac)
    at = _k_builder(cuda, g)
    for i in range(3):
        k = at(i)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(k.cpu().numpy().T, wl.k_at(i))


def _ulps(a, b):
    return np.abs(a - b) / np.maximum(np.spacing(np.abs(b)), np.finfo(float).tiny)


def test_device_math_rate_constants_within_ulps(cuda):
    """fo_rate_constants and fo_update_photolysis evaluate exp, pow and cos on
    the device: within 4 ulp of NumPy on the subset's cells."""
    from fastode_gb300 import _abi, synthetic as syn
    torch = cuda
    f = load("ros3_210x500_subset")
    wl = syn.plain_large().subset(f["cells"])
    sm, cells = wl.sm, wl.cells
    C, R = cells.C, sm.R
    M = cells.p / (syn.R_GAS * cells.T)
    photo = np.nonzero(sm.photolytic)[0].astype(np.int32)
    d = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in
         dict(A=sm.A, E=sm.E, power=sm.mech.third_body_power.astype(np.float64), T=cells.T, M=M,
              phase=cells.phase, J=sm.J[photo], rxn=photo).items()}
    k = torch.empty((R, C), dtype=torch.float64, device="cuda")
    lib = _abi.lib()
    _abi.check(lib.fo_rate_constants(C, R, d["A"].data_ptr(), d["E"].data_ptr(), d["power"].data_ptr(),
                                     d["T"].data_ptr(), d["M"].data_ptr(), k.data_ptr(), 1, C, None),
               "fo_rate_constants")
    worst = 0.0
    for i in (0, 11, 29):
        t = i * wl.dt
        _abi.check(lib.fo_update_photolysis(C, len(photo), d["rxn"].data_ptr(), d["J"].data_ptr(),
                                            d["phase"].data_ptr(), 2.0 * np.pi / 86400.0, t, k.data_ptr(), 1, C,
                                            None), "fo_update_photolysis")
        torch.cuda.synchronize()
        got = k.cpu().numpy().T
        ref = syn.rate_constants(sm, cells, t)
        # a photolysis factor that the cosine rounds to either side of zero
        # is max(0, .); compare where both are nonzero and require the zero
        # pattern to agree elsewhere
        both = (got != 0.0) & (ref != 0.0)
        assert np.array_equal(got == 0.0, ref == 0.0)
        worst = max(worst, float(_ulps(got[both], ref[both]).max()))
    assert worst <= 4.0, worst


def _run_subset(cuda, f, kernel, intervals, slots=0):
    from fastode_gb300 import Algorithm
    from fastode_gb300.batch import Batch
    torch = cuda
    b = Batch(mechanism_of(f), f["Y0"], group_size=int(f["group_size"]), trace_cap=64, slots=slots,
              algorithm=Algorithm(kernel=kernel))
    atol = torch.from_numpy(f["atol"]).cuda()
    at = _k_builder(cuda, f)
    counts, statuses, snaps = [], [], {}
    traces = [[] for _ in range(b.ngroups)]
    for i in range(intervals):
        b.step(at(i), float(f["dt"]), atol, float(f["rtol"]))
        torch.cuda.synchronize()
        counts.append(b.counts.cpu().numpy().copy())
        statuses.append(b.status.cpu().numpy().copy())
        tl, tr = b.trace_len.cpu().numpy(), b.trace.cpu().numpy()
        for g in range(b.ngroups):
            assert tl[g] <= 64
            traces[g].extend(tr[g, : tl[g]].tolist())
        if i + 1 in f["snapshots"]:
            snaps[i + 1] = b.state()
    return b, np.stack(counts, axis=1), np.array(statuses).T, traces, snaps


# the largest state difference measured on a GB300, per kernel (recorded so a
# regression shows; the bar is STATE_RTOL)
@pytest.mark.parametrize("kernel", ["generated", "compact", "pipelined", "plain"])
def test_subset_matches_reference(cuda, kernel):
    f = load("ros3_210x500_subset")
    T = int(f["intervals"])
    b, counts, statuses, traces, snaps = _run_subset(cuda, f, kernel, T)
    np.testing.assert_array_equal(counts, f["counts"])
    np.testing.assert_array_equal(statuses, f["status"])
    mem = b.memory.cpu().numpy()
    np.testing.assert_array_equal(mem[:, 0], f["memory"][:, 0])
    np.testing.assert_array_equal(mem[:, 2], f["memory"][:, 2])
    np.testing.assert_allclose(mem[:, 1], f["memory"][:, 1], rtol=ERR_RTOL, atol=ERR_ATOL)
    for g in range(b.ngroups):
        na = int(f["n_attempts"][g])
        tr = np.array(traces[g])
        assert len(tr) == na
        np.testing.assert_array_equal(tr[:, 1], f["hs"][g, :na])
        np.testing.assert_allclose(tr[:, 2], f["errs"][g, :na], rtol=ERR_RTOL, atol=ERR_ATOL)
    worst = {s: float(rel_err(snaps[s], f["Y_snap"][j]).max()) for j, s in enumerate(f["snapshots"])}
    print(f"{kernel}: largest state difference by interval {worst}")
    assert max(worst.values()) <= STATE_RTOL, worst
    from fastode_gb300.scenario import digits
    snaps_ref = list(f["snapshots"])
    for j, s in enumerate(f["tight_snapshots"]):
        d_dev = digits(snaps[int(s)], f["Y_tight"][j], 1e-14)[0]
        d_ref = digits(f["Y_snap"][snaps_ref.index(s)], f["Y_tight"][j], 1e-14)[0]
        print(f"{kernel}: digits against the rtol 1e-10 solve after {int(s)} intervals: {d_dev:.6f} "
              f"(reference {d_ref:.6f})")
        assert abs(d_dev - d_ref) <= 1e-6 and d_ref > 4.0, (s, d_dev, d_ref)


def test_subset_queue_and_block_per_group_agree(cuda):
    """The persistent queue (two slots for eight groups: every slot is reused)
    gives the bits of one block per group on the subset."""
    f = load("ros3_210x500_subset")
    b0, c0, s0, _, _ = _run_subset(cuda, f, "generated", 4)
    b1, c1, s1, _, _ = _run_subset(cuda, f, "generated", 4, slots=2)
    np.testing.assert_array_equal(b0.state(), b1.state())
    np.testing.assert_array_equal(c0, c1)
    np.testing.assert_array_equal(s0, s1)
