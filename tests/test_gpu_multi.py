"""Several mechanisms in one persistent launch, replayed as a CUDA graph per
interval (the batched uneven workload's machinery), against separate launches
per mechanism and against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_parts():
    from fastode_gb300 import synthetic as syn
    return syn.batched_uneven(n_cells=32 * 6, intervals=4, sizes=((20, 40), (60, 40), (30, 70)))


def make_parts(wls, cuda, kernel="generated", lockstep=True):
    from fastode_gb300 import Algorithm
    from fastode_gb300.multi import Part
    parts = []
    for wl in wls:
        photo = np.nonzero(wl.sm.photolytic)[0]
        parts.append(Part(wl.sm.mech, wl.cells.Y0, wl.k_at(0), wl.atol, wl.rtol, wl.dt, group_size=32,
                          algorithm=Algorithm(kernel=kernel, lockstep=lockstep),
                          photolysis=(photo, wl.sm.J[photo], wl.cells.phase)))
    return parts


@pytest.mark.parametrize("kernel", ["generated", "compact"])
@pytest.mark.parametrize("graph", [True, False])
def test_multi_launch_matches_separate_batches(cuda, graph, kernel):
    """One persistent launch over three mechanisms (with the generated kernel,
    one module holding the three mechanisms' code) against one launch per
    mechanism."""
    from fastode_gb300 import Algorithm
    from fastode_gb300.batch import Batch
    from fastode_gb300.multi import MultiBatch
    torch = cuda
    wls = small_parts()
    mb = MultiBatch(make_parts(wls, cuda, kernel))
    intervals = 4
    mb.run(intervals, graph=graph)
    torch.cuda.synchronize()
    for wl, part in zip(wls, mb.parts):
        b = Batch(wl.sm.mech, wl.cells.Y0, group_size=32, algorithm=Algorithm(kernel=kernel))
        atol = torch.from_numpy(wl.atol).cuda()
        for i in range(intervals):
            # the device clock and the photolysis kernel against host-made k:
            # the cosine may differ in the last bit, so compare loosely below
            b.step(torch.from_numpy(np.ascontiguousarray(wl.k_at(i).T)).cuda(), wl.dt, atol, wl.rtol)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(part.counts.cpu().numpy(), b.counts.cpu().numpy())
        Y, Yb = part.state(), b.state()
        assert np.all(np.abs(Y - Yb) <= 1e-10 * np.maximum(np.abs(Yb), 1e-14))
    assert all(s == 0 for p in mb.parts for s in p.status.cpu().numpy())


def test_multi_graph_replay_is_deterministic(cuda):
    """Replaying the captured interval graph gives the bits of the eager
    launches."""
    from fastode_gb300.multi import MultiBatch
    torch = cuda
    wls = small_parts()
    a = MultiBatch(make_parts(wls, cuda))
    a.run(3, graph=True)
    b = MultiBatch(make_parts(wls, cuda))
    b.run(3, graph=False)
    torch.cuda.synchronize()
    for pa, pb in zip(a.parts, b.parts):
        np.testing.assert_array_equal(pa.state(), pb.state())
        np.testing.assert_array_equal(pa.counts.cpu().numpy(), pb.counts.cpu().numpy())
    assert float(a.t.item()) == float(b.t.item()) == 3 * wls[0].dt


def test_multi_matches_oracle_on_dark_and_lit_cells(cuda):
    """Half the cells are dark (J = 0): the device counts per group equal the
    oracle's on host-made rate constants."""
    from oracle import rosenbrock as O
    wls = small_parts()
    mb = MultiBatch_from(wls, cuda)
    mb.run(2, graph=True)
    cuda.cuda.synchronize()
    for wl, part in zip(wls, mb.parts):
        assert np.any(wl.k_at(0)[:, wl.sm.photolytic] == 0.0)      # some cells dark
        Yo, co, _, _, _ = O.run_groups(wl.sm.mech, wl.cells.Y0, wl.k_at, wl.dt, 2, wl.atol, wl.rtol)
        counts = part.counts.cpu().numpy()
        for g, c in enumerate(co):
            assert tuple(counts[g]) == c.as_tuple()
        assert np.all(np.abs(part.state() - Yo) <= 1e-9 * np.maximum(np.abs(Yo), 1e-14))


def MultiBatch_from(wls, cuda):
    from fastode_gb300.multi import MultiBatch
    return MultiBatch(make_parts(wls, cuda))


@pytest.mark.parametrize("slots", [0, 4])
def test_multi_lockstep_rounds_give_the_same_bits(cuda, slots):
    """Lockstep rounds in the several-mechanism launch (a cooperative launch;
    each mechanism makes as many attempts per round as the largest one's
    attempt costs over its own), captured in the interval graph and replayed,
    against the same launch without rounds: every part's states, Counts,
    memory and statuses bit for bit; with four slots for eighteen groups the
    slots also pull further groups between rounds."""
    from fastode_gb300.multi import MultiBatch
    torch = cuda
    wls = small_parts()
    runs = []
    for lockstep in (True, False):
        mb = MultiBatch(make_parts(wls, cuda, lockstep=lockstep), slots=slots)
        mb.run(4, graph=True)
        torch.cuda.synchronize()
        runs.append([(p.state(), p.counts.cpu().numpy(), p.memory.cpu().numpy(), p.status.cpu().numpy())
                     for p in mb.parts])
    for a, b in zip(*runs):
        for x, y in zip(a, b):
            np.testing.assert_array_equal(x, y)
