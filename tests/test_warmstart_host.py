"""Host-side logic of the learned warm start's trainer (no GPU)."""
import math

import numpy as np

from eikonalxx_gb300 import warmstart as ws


def test_learning_rate_warms_up_then_decays_to_the_floor():
    steps, lr = 1000, 1e-3
    r = [ws.learning_rate(k, steps, lr) for k in range(steps)]
    w = int(0.05 * steps)
    assert r[0] == lr / w and math.isclose(r[w - 1], lr)
    assert all(b <= a + 1e-18 for a, b in zip(r[w:], r[w + 1:]))      # non-increasing after warm-up
    assert math.isclose(r[w], lr) and r[-1] >= 0.05 * lr and r[-1] < 0.06 * lr


def test_random_smooth_models_stay_in_the_velocity_range():
    rng = np.random.default_rng(3)
    for _ in range(3):
        v = ws.random_smooth_model(32, 24, 16, 100.0, rng)
        assert v.shape == (16, 24, 32) and v.dtype == np.float32
        assert v.min() >= 1500.0 and v.max() <= 8000.0 and v.std() > 0


def test_net_config_is_checked_before_any_device_is_touched(lib):
    import pytest
    import eikonalxx_gb300 as ex
    good = (16, 16, 8, 50.0, 50.0, 50.0)
    for grid, batch in [((20, 16, 8, 50.0, 50.0, 50.0), 1),          # not a multiple of 8
                        ((16, 16, 8, float("inf"), 50.0, 50.0), 1),  # spacing not finite
                        ((16, 16, 8, 50.0, -1.0, 50.0), 1),          # spacing not positive
                        (good + (0.0, float("nan"), 0.0), 1),        # origin not finite
                        (good, 0)]:
        with pytest.raises(ex.InvalidArgument):
            ws.WarmNet(grid, batch=batch)
