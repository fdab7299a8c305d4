"""The autotuner's host logic (CPU): candidates, shared-memory fit, choice."""
import pytest

from fastode_gb300.tune import Config, autotune, candidates, fits


def test_fits_follows_shared_memory():
    # 210 species: 4 warps of 32 lanes fit (217 KB), 8 do not
    assert fits(210, 32) and fits(210, 128)
    assert not fits(210, 256)
    assert fits(20, 256)


def test_autotune_picks_the_fastest_that_fits():
    speed = {("pipelined", 32, False): 10.0, ("pipelined", 64, True): 12.0, ("plain", 32, False): 5.0}

    def measure(c):
        return speed.get((c.kernel, c.group_size, c.persistent), 1.0)

    r = autotune(measure, 210)
    assert r.best == Config("pipelined", 64, True)
    assert len(r.table) == len(candidates(210))


def test_autotune_skips_configs_that_do_not_fit():
    calls = []

    def measure(c):
        calls.append(c)
        return float(c.group_size)

    r = autotune(measure, 400, [Config("pipelined", 32), Config("pipelined", 128)])
    assert r.best == Config("pipelined", 32)
    assert [c for c, v in r.table if v is None] == [Config("pipelined", 128)]
    assert calls == [Config("pipelined", 32)]


def test_autotune_raises_when_nothing_fits():
    with pytest.raises(ValueError):
        autotune(lambda c: 1.0, 5000, [Config("pipelined", 64)])


def test_per_kernel_shared_memory():
    """With one figure per kernel, a group size that only the compact
    kernel's half rows fit is measured for compact and skipped for the
    others (210 species, 256 lanes: 105 doubles per cell fit, 210 do not)."""
    smem = {"compact": 105, "pipelined": 210, "plain": 210}
    assert fits(smem, 256, "compact") and not fits(smem, 256, "pipelined")
    measured = []

    def measure(c):
        measured.append(c)
        return 1.0

    r = autotune(measure, smem, candidates(smem, group_sizes=(256,), persistent=(False,)))
    assert measured == [Config("compact", 256, False)]
    assert r.best == Config("compact", 256, False)
    assert [c.kernel for c, v in r.table if v is None] == ["pipelined", "plain"]


def test_generated_candidates_carry_tiles_and_small_groups():
    """The generated variant is tuned over its register tile and runs groups
    of at most 32 cells; the table-driven kernels have no tile."""
    smem = {"generated": 0, "compact": 105, "pipelined": 210, "plain": 210}
    cs = candidates(smem, group_sizes=(16, 32, 64), kernels=("generated", "compact"), persistent=(True,),
                    tiles=(4, 6, 8))
    gen = [c for c in cs if c.kernel == "generated"]
    assert sorted({c.tile for c in gen}) == [4, 6, 8]
    assert {c.tile for c in cs if c.kernel == "compact"} == {6}
    assert not fits(smem, 64, "generated") and fits(smem, 32, "generated")

    def measure(c):
        return 100.0 + c.tile if c.kernel == "generated" else 50.0

    r = autotune(measure, smem, cs)
    assert r.best == Config("generated", 16, True, 8)
    assert [c for c, v in r.table if v is None] == [c for c in gen if c.group_size == 64]
