"""The autotuner on the device: measure_on_device over kernel variants,
group sizes, launch shapes and the generated code's register tiles picks a
configuration that fits, and that configuration keeps parity with the oracle
(the reference's algorithm) at its own grouping. Register tiles change no
result: every tile gives the same bits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(cuda, wl, kernel, group_size, tile, slots=0):
    from fastode_gb300 import Algorithm
    from fastode_gb300.batch import Batch
    torch = cuda
    b = Batch(wl.sm.mech, wl.cells.Y0, group_size=group_size, slots=slots,
              algorithm=Algorithm(kernel=kernel, tile=tile))
    atol = torch.from_numpy(wl.atol).cuda()
    for i in range(wl.intervals):
        b.step(torch.from_numpy(np.ascontiguousarray(wl.k_at(i).T)).cuda(), wl.dt, atol, wl.rtol)
    torch.cuda.synchronize()
    return b


def test_tuner_choice_fits_and_keeps_parity(cuda):
    from fastode_gb300 import synthetic as syn
    from fastode_gb300.plan import plan_for
    from fastode_gb300.tune import autotune, candidates, fits, measure_on_device
    from oracle import rosenbrock as O
    wl = syn.batched_uneven(n_cells=32 * 12, intervals=3, sizes=((60, 40),))[0]
    measure = measure_on_device(wl.sm.mech, wl.cells.Y0, wl.k_at, wl.dt, wl.atol, wl.rtol)
    bp = plan_for(wl.sm.mech)
    smem = {k: bp.smem_items(k) for k in ("pipelined", "plain", "compact")}
    smem["generated"] = 0
    cs = candidates(smem, group_sizes=(16, 32, 64), kernels=("generated", "compact"), persistent=(False, True),
                    tiles=(4, 6))
    r = autotune(measure, smem, cs)
    best = r.best
    assert fits(smem, best.group_size, best.kernel)
    assert all(v is None for c, v in r.table if c.kernel == "generated" and c.group_size == 64)
    assert all(v is not None and v > 0.0 for c, v in r.table if c.kernel == "compact")
    b = _run(cuda, wl, best.kernel, best.group_size, best.tile)
    Yo, co, so, _, _ = O.run_groups(wl.sm.mech, wl.cells.Y0, wl.k_at, wl.dt, wl.intervals, wl.atol, wl.rtol,
                                    group_size=best.group_size)
    counts = b.counts.cpu().numpy()
    for g, c in enumerate(co):
        assert tuple(counts[g]) == c.as_tuple(), (best, g)
    assert np.all(np.abs(b.state() - Yo) <= 1e-10 * np.maximum(np.abs(Yo), 1e-14))


@pytest.mark.parametrize("tile", [3, 4, 8])
def test_register_tiles_give_the_same_bits(cuda, tile):
    from fastode_gb300 import synthetic as syn
    wl = syn.plain_small(n_cells=64, intervals=3)
    a = _run(cuda, wl, "generated", 32, 6)
    b = _run(cuda, wl, "generated", 32, tile)
    assert b.plan.tile == tile and a.plan.tile == 6
    np.testing.assert_array_equal(a.state(), b.state())
    np.testing.assert_array_equal(a.counts.cpu().numpy(), b.counts.cpu().numpy())
