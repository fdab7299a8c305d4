"""The generated variant (FO_VARIANT_GENERATED): each mechanism's factorization
of alpha*M - J and its triangular solves generated as straight-line code from
the fill pattern, linked with the integrator kernel per mechanism.

Its factors are those of every other variant bit for bit, and its solves sum
each row in the order of the plain variant's loops, so a whole integration
must give the plain variant's bits: states, Counts, statuses, controller
memory and every attempt's step size and error norm. Parity with the
reference itself is in test_gpu_parity.py and test_gpu_c2_subset.py, which run
this variant against the reference-made fixtures.
"""
import ctypes as C

import numpy as np
import pytest

from golden_cases import DAE_CASES, load, mechanism_of, table_mechanism
from test_gpu_parity import run_batch

pytestmark = pytest.mark.gpu


def _same(a, b):
    np.testing.assert_array_equal(a[0].state(), b[0].state())
    np.testing.assert_array_equal(a[0].counts.cpu().numpy(), b[0].counts.cpu().numpy())
    np.testing.assert_array_equal(a[0].memory.cpu().numpy(), b[0].memory.cpu().numpy())
    np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("case", ["ros3_20x40", "ros3_210x500"])
def test_generated_gives_the_plain_variants_bits(cuda, case):
    f = load(case)
    plain = run_batch(cuda, f, kernel="plain")
    gen = run_batch(cuda, f, kernel="generated")
    _same(plain, gen)
    for tp, tg in zip(plain[2], gen[2]):
        np.testing.assert_array_equal(np.array(tp), np.array(tg))


def test_generated_queue_gives_the_same_bits(cuda):
    f = load("ros3_210x500")
    a = run_batch(cuda, f, trace_cap=0, kernel="generated")
    b = run_batch(cuda, f, trace_cap=0, slots=1, kernel="generated")
    _same(a, b)


def test_generated_plan_module(cuda, tmp_path):
    """fo_plan_generate: the kernel stays within its register budget without
    spilling to local memory, the module is cached on disk, and a second plan
    of the same mechanism loads it from the cache."""
    from fastode_gb300.plan import Plan
    f = load("ros3_20x40")
    mech = mechanism_of(f)
    first = Plan(mech).generate(tmp_path)
    assert first["from_cache"] == 0
    assert first["registers"] <= 128
    second = Plan(mech).generate(tmp_path)
    assert second["from_cache"] == 1
    assert second["cubin_bytes"] == first["cubin_bytes"]
    assert len(list(tmp_path.glob("gen-*.cubin"))) == 1


def test_generated_needs_its_module_and_small_groups(cuda):
    """FO_VARIANT_GENERATED on a plan that was not generated, or with groups
    above 32 cells, is refused by the C-ABI (FO_E_UNSUPPORTED); the Python
    layer runs groups above 32 cells on the compact variant."""
    from fastode_gb300 import Algorithm, _abi
    from fastode_gb300.batch import Batch, group_offsets
    from fastode_gb300.plan import Plan
    torch = cuda
    f = load("ros3_20x40")
    plan = Plan(mechanism_of(f))
    Cc = f["Y0"].shape[0]
    offs = torch.from_numpy(group_offsets(Cc, 32)).cuda()
    G = len(offs) - 1
    Y = torch.from_numpy(np.ascontiguousarray(f["Y0"].T)).cuda()
    k = torch.from_numpy(np.ascontiguousarray(f["k"][0].T)).cuda()
    atol = torch.from_numpy(f["atol"]).cuda()
    mem = torch.zeros((G, 3), dtype=torch.float64, device="cuda")
    cnt = torch.zeros((G, 13), dtype=torch.int64, device="cuda")
    st = torch.zeros(G, dtype=torch.int32, device="cuda")
    ws = torch.empty(plan.workspace_bytes(G, 64), dtype=torch.uint8, device="cuda")
    opts = Algorithm(kernel="generated").options()

    def call(cells):
        return _abi.lib().fo_solve(plan.handle, C.byref(opts), G, offs.data_ptr(), cells, Y.data_ptr(), 1, Cc,
                                   k.data_ptr(), 1, Cc, atol.data_ptr(), float(f["rtol"]), float(f["dt"]),
                                   mem.data_ptr(), cnt.data_ptr(), st.data_ptr(), ws.data_ptr(), ws.numel(), 0,
                                   None, 0, None, None)

    assert call(32) == _abi.FO_E_UNSUPPORTED
    plan.generate()
    assert call(64) == _abi.FO_E_UNSUPPORTED
    assert call(32) == 0
    torch.cuda.synchronize()
    b = Batch(mechanism_of(f), f["Y0"], group_size=64, algorithm=Algorithm(kernel="generated"))
    assert b.opts.variant == _abi.VARIANTS["compact"]


@pytest.mark.parametrize("case", DAE_CASES)
def test_generated_constrained_systems(cuda, case):
    """RODAS3 with algebraic species: the projection factors its
    algebraic-rows-only matrix with the row loop and solves with the generated
    solves; the step factorizations are generated. Plain variant's bits."""
    from fastode_gb300 import Algorithm, RODAS3
    from fastode_gb300.batch import Batch
    torch = cuda
    f = load(case)
    mech = table_mechanism(f)
    out = []
    for kernel in ("plain", "generated"):
        b = Batch(mech, f["Y0"], group_size=32, algorithm=Algorithm(RODAS3, kernel=kernel), mass=f["mass"])
        atol = torch.from_numpy(f["atol"]).cuda()
        k = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(f["k"], (f["Y0"].shape[0], mech.R)).T)).cuda()
        for _ in range(int(f["intervals"])):
            b.step(k, float(f["dt"]), atol, float(f["rtol"]))
        torch.cuda.synchronize()
        out.append(b)
    np.testing.assert_array_equal(out[0].state(), out[1].state())
    np.testing.assert_array_equal(out[0].counts.cpu().numpy(), out[1].counts.cpu().numpy())
    np.testing.assert_array_equal(out[0].status.cpu().numpy(), out[1].status.cpu().numpy())


def _subset_run(cuda, f, lockstep, intervals, trace=True):
    from fastode_gb300 import Algorithm, _abi
    from fastode_gb300.batch import Batch
    torch = cuda
    b = Batch(mechanism_of(f), f["Y0"], group_size=32, trace_cap=64 if trace else 0,
              algorithm=Algorithm(kernel="generated", lockstep=lockstep))
    atol = torch.from_numpy(f["atol"]).cuda()
    k = torch.from_numpy(np.ascontiguousarray(f["k0"].T)).cuda()
    rxn = torch.from_numpy(f["photo"].astype(np.int32)).cuda()
    J = torch.from_numpy(f["J"]).cuda()
    fac = torch.from_numpy(np.ascontiguousarray(f["f"])).cuda()
    traces = []
    for i in range(intervals):
        _abi.check(_abi.lib().fo_photolysis_factor(b.C, rxn.numel(), rxn.data_ptr(), J.data_ptr(),
                                                   fac[i].data_ptr(), k.data_ptr(), 1, b.C, None),
                   "fo_photolysis_factor")
        b.step(k, float(f["dt"]), atol, float(f["rtol"]))
        if trace:
            tl, tr = b.trace_len.cpu().numpy(), b.trace.cpu().numpy()
            traces.append([tr[g, : tl[g]].copy() for g in range(b.ngroups)])
    torch.cuda.synchronize()
    return b, traces


def test_lockstep_rounds_give_the_same_bits(cuda):
    """Attempts in lockstep rounds (a cooperative launch with a grid-wide
    barrier after every attempt, fo_options.lockstep) against the same
    integration without rounds, on the measured workload's parity subset over
    its first 12 intervals (12 to 26 attempts per group in the first): states,
    Counts, memory, statuses and every attempt's step size and error norm."""
    f = load("ros3_210x500_subset")
    a, ta = _subset_run(cuda, f, True, 12)
    b, tb = _subset_run(cuda, f, False, 12)
    np.testing.assert_array_equal(a.state(), b.state())
    for x, y in ((a.counts, b.counts), (a.memory, b.memory), (a.status, b.status)):
        np.testing.assert_array_equal(x.cpu().numpy(), y.cpu().numpy())
    for ia, ib in zip(ta, tb):
        for ga, gb in zip(ia, ib):
            np.testing.assert_array_equal(ga, gb)
    np.testing.assert_array_equal(a.counts.cpu().numpy(), f["counts"][:, 11])


def test_lockstep_falls_back_when_the_groups_do_not_fit(cuda):
    """More groups than the GPU holds at once: the cooperative launch is
    refused and the groups run without rounds, with the same results."""
    import torch
    from fastode_gb300 import Algorithm, synthetic as syn
    from fastode_gb300.batch import Batch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    wl = syn.plain_small(n_cells=32 * (16 * sms + 64), intervals=2)
    at = torch.from_numpy(wl.atol).cuda()
    out = []
    for lockstep in (True, False):
        b = Batch(wl.sm.mech, wl.cells.Y0, group_size=32, algorithm=Algorithm(kernel="generated", lockstep=lockstep))
        for i in range(2):
            b.step(torch.from_numpy(np.ascontiguousarray(wl.k_at(i).T)).cuda(), wl.dt, at, wl.rtol)
        torch.cuda.synchronize()
        out.append((b.state(), b.counts.cpu().numpy()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
