"""The bench's model of the build: the pass plan it mirrors from the library
(passes.cuh run_pass_pipeline, wt_build.cu run_passes) and the algorithmic
bytes per pass launch that its roofline divides by.  CPU only."""
import pytest

import bench


@pytest.mark.parametrize("L", range(1, 17))
def test_pass_plan_covers_the_levels_below_level_0(L):
    plan = bench.pass_plan(L)
    assert sum(plan) == max(L - 1, 0)
    assert all(1 <= k <= 4 for k in plan)
    if L in (6, 8):
        # octal group levels at 0 and 3: a first pass of levels 1-3 whose
        # level-3 order feeds octal level 3
        assert plan == [3, L - 4]
    elif L > 1:
        assert len(plan) == -(-(L - 1) // 4)
        assert max(plan) - min(plan) <= 1


def test_pass_bytes_per_launch():
    n = 1 << 30
    # sigma = 256: levels 1-3 with the level-3 order written, then levels 4-7
    want = ((n + 3 * n / 8 + n) + (n + 4 * n / 8)) / 2
    assert bench.pass_bytes_per_launch(n, 8) == pytest.approx(want)
    # sigma = 16: one pass of levels 1-3, no order written
    assert bench.pass_bytes_per_launch(n, 4) == pytest.approx(n + 3 * n / 8)
    assert bench.pass_bytes_per_launch(n, 1) == 0.0
