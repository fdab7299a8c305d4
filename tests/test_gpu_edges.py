"""Edge cases of the device integrator through the C-ABI: the largest group
(256 cells in eight warps, whose norm and decisions are block-wide), a group
of one cell, zero groups, groups that do not fit, and invalid arguments."""
import ctypes as C

import numpy as np
import pytest

from golden_cases import load, mechanism_of, rel_err

pytestmark = pytest.mark.gpu


def _oracle(mech, Y0, ks, dt, atol, rtol, group_size, intervals):
    from oracle import rosenbrock as O
    return O.run_groups(mech, Y0, lambda i: ks[i], dt, intervals, atol, rtol, group_size=group_size)


@pytest.mark.parametrize("group_size", [1, 256])
def test_group_sizes_one_and_256_match_the_oracle(cuda, group_size):
    from fastode_gb300 import synthetic as syn
    from fastode_gb300.batch import Batch
    torch = cuda
    wl = syn.plain_small(n_cells=256, intervals=4)
    cells = 256 if group_size == 256 else 4
    Y0 = wl.cells.Y0[:cells]
    ks = [wl.k_at(i)[:cells] for i in range(wl.intervals)]
    b = Batch(wl.sm.mech, Y0, group_size=group_size)
    atol = torch.from_numpy(wl.atol).cuda()
    for i in range(wl.intervals):
        b.step(torch.from_numpy(np.ascontiguousarray(ks[i].T)).cuda(), wl.dt, atol, wl.rtol)
    Yo, co, so, _, _ = _oracle(wl.sm.mech, Y0, ks, wl.dt, wl.atol, wl.rtol, group_size, wl.intervals)
    counts = b.counts.cpu().numpy()
    for g in range(b.ngroups):
        assert tuple(counts[g]) == co[g].as_tuple()
    assert b.statuses() == ["converged"] * b.ngroups
    assert rel_err(b.state(), Yo).max() <= 1e-10


def _solve_call(torch, plan, ngroups, max_cells, Yd, kd, atol, dt, opts=None):
    from fastode_gb300 import Algorithm, _abi
    opts = opts if opts is not None else plan.options_for(Algorithm(), max(max_cells, 1))
    Cc = Yd.shape[1]
    offs = torch.tensor([0, Cc] if ngroups else [0], dtype=torch.int32, device="cuda")
    mem = torch.zeros((max(ngroups, 1), 3), dtype=torch.float64, device="cuda")
    cnt = torch.zeros((max(ngroups, 1), 13), dtype=torch.int64, device="cuda")
    st = torch.zeros(max(ngroups, 1), dtype=torch.int32, device="cuda")
    ws = plan.workspace(1, min(max(max_cells, 1), 256))
    return _abi.lib().fo_solve(plan.handle, C.byref(opts), ngroups, offs.data_ptr(), max_cells, Yd.data_ptr(), 1, Cc,
                               kd.data_ptr(), 1, Cc, atol.data_ptr(), 1e-3, dt, mem.data_ptr(), cnt.data_ptr(),
                               st.data_ptr(), ws.data_ptr(), ws.numel(), 0, None, 0, None, None), cnt


def test_zero_groups_and_invalid_arguments(cuda):
    from fastode_gb300 import Algorithm, _abi
    from fastode_gb300.plan import plan_for
    torch = cuda
    f = load("ros3_20x40")
    mech = mechanism_of(f)
    plan = plan_for(mech)
    Yd = torch.from_numpy(np.ascontiguousarray(f["Y0"][:32].T)).cuda()
    kd = torch.from_numpy(np.ascontiguousarray(f["k"][0][:32].T)).cuda()
    atol = torch.from_numpy(f["atol"]).cuda()
    before = Yd.clone()
    rc, cnt = _solve_call(torch, plan, 0, 32, Yd, kd, atol, 30.0)      # nothing to do, nothing touched
    torch.cuda.synchronize()
    assert rc == _abi.FO_OK and torch.equal(Yd, before)
    rc, _ = _solve_call(torch, plan, 1, 32, Yd, kd, atol, 0.0)         # dt must be positive
    assert rc == -1 and b"dt" in _abi.lib().fo_last_error()
    rc, _ = _solve_call(torch, plan, 1, 257, Yd, kd, atol, 30.0)       # groups hold at most 256 cells
    assert rc == -3
    o = Algorithm().options()
    o.variant = 7
    rc, _ = _solve_call(torch, plan, 1, 32, Yd, kd, atol, 30.0, o)
    assert rc == -1 and b"variant" in _abi.lib().fo_last_error()
    o = Algorithm().options()
    o.tableau = 5
    rc, _ = _solve_call(torch, plan, 1, 32, Yd, kd, atol, 30.0, o)
    assert rc == -1 and b"tableau" in _abi.lib().fo_last_error()
    torch.cuda.synchronize()
    assert torch.equal(Yd, before)


def test_group_too_large_for_shared_memory_is_rejected(cuda):
    """210 species x 256 cells of whole work rows (the pipelined kernel) do
    not fit in one block's shared memory: the call fails with
    FO_E_UNSUPPORTED instead of launching. (The compact kernel's half rows
    do fit.)"""
    from fastode_gb300 import Algorithm, _abi
    from fastode_gb300.batch import Batch
    f = load("ros3_210x500")
    mech = mechanism_of(f)
    Y0 = np.repeat(f["Y0"], 4, axis=0)                       # 256 cells
    b = Batch(mech, Y0, group_size=256, algorithm=Algorithm(kernel="pipelined"))
    torch = cuda
    k = torch.from_numpy(np.ascontiguousarray(np.repeat(f["k"][0], 4, axis=0).T)).cuda()
    atol = torch.from_numpy(f["atol"]).cuda()
    with pytest.raises(_abi.FastodeError, match="shared memory"):
        b.step(k, float(f["dt"]), atol, float(f["rtol"]))


@pytest.mark.parametrize("kernel", ["compact", "pipelined", "plain"])
@pytest.mark.parametrize("n,R", [(1, 1), (2, 2), (3, 4)])
def test_tiny_mechanisms_match_the_oracle(cuda, kernel, n, R):
    """One, two and three species: the compact kernel's halves are empty or a
    single row; every kernel gives the oracle's Counts and states."""
    from fastode_gb300 import Algorithm
    from fastode_gb300 import synthetic as syn
    from fastode_gb300.batch import Batch
    torch = cuda
    sm = syn.synthetic_mechanism(n, R, seed=3)
    wl = syn.Workload("tiny", sm, syn.synthetic_cells(sm, 32, seed=4), 30.0, 3, 1e-3, 32, True)
    ks = [wl.k_at(i) for i in range(wl.intervals)]
    b = Batch(sm.mech, wl.cells.Y0, group_size=32, algorithm=Algorithm(kernel=kernel))
    atol = torch.from_numpy(wl.atol).cuda()
    for i in range(wl.intervals):
        b.step(torch.from_numpy(np.ascontiguousarray(ks[i].T)).cuda(), wl.dt, atol, wl.rtol)
    Yo, co, so, _, _ = _oracle(sm.mech, wl.cells.Y0, ks, wl.dt, wl.atol, wl.rtol, 32, wl.intervals)
    assert tuple(b.counts.cpu().numpy()[0]) == co[0].as_tuple()
    assert b.statuses() == [so[0][-1]]
    assert rel_err(b.state(), Yo).max() <= 1e-10
