"""The window's automatic checkpoint spacing (every = 0) as a pure function of
free device memory (vibe_gb300_window_plan): both branches and the refusal,
without a GPU."""
import pytest

GB = 1 << 30


def test_store_every_step_when_it_fits(vg):
    # 120 states + a 3-state segment in 80 % of 200 GB
    assert vg.window_plan(200 * GB, GB, 120, 3) == 1
    assert vg.window_plan(200 * GB, GB, 120, 2) == 1


def test_sqrt_spacing_with_recomputation(vg):
    # 120 states do not fit in 80 % of 100 GB; ceil(sqrt(120 / 3)) = 7:
    # 18 checkpoints + 3 x 7 segment states = 39 states fit
    assert vg.window_plan(100 * GB, GB, 120, 3) == 7
    assert vg.window_plan(100 * GB, GB, 120, 2) == 8  # ceil(sqrt(60)); 15 + 16 states


def test_refuses_when_checkpoints_do_not_fit(vg):
    with pytest.raises(vg.VibeError) as e:
        vg.window_plan(20 * GB, GB, 120, 3)  # 39 states > 16
    assert "do not fit" in str(e.value)


def test_rejects_bad_arguments(vg):
    with pytest.raises(vg.VibeError):
        vg.window_plan(GB, 0, 10, 3)
