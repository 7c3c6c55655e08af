"""Trajectories written from the device in the binary results format."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_plan_save_results_matches_arrays(gpu_lib, tmp_path):
    from magpy_gb300 import core
    E, n = 4, 3
    rng = np.random.default_rng(9)
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    plan = core.EnsemblePlan(E, np.full(n, 7e-9), np.full(n, 2e4), axes, axes.copy(),
                             np.arange(3 * n).reshape(n, 3) * 1e-8, 4e5, 0.1, 300.0, False,
                             True, False, 1e-13, 3e-11, 13, np.arange(E) + 5, "sine", 1e4, 3e8,
                             precision="mixed")
    plan.run()
    arr = plan.arrays()
    plan.save_results(tmp_path / "run", 1, 3)
    for e in range(E):
        for i in range(n):
            exists = (tmp_path / f"run_{e}_{i}.mz").exists()
            assert exists == (1 <= e < 3)
            if not exists:
                continue
            back = core.load_results(tmp_path / f"run_{e}_{i}")
            col = e * n + i
            np.testing.assert_array_equal(back["mx"], arr.mx[:, col])
            np.testing.assert_array_equal(back["my"], arr.my[:, col])
            np.testing.assert_array_equal(back["mz"], arr.mz[:, col])
            np.testing.assert_array_equal(back["time"], arr.time[e])
            np.testing.assert_array_equal(back["field"], arr.field[e])
    with pytest.raises(Exception):
        plan.save_results(tmp_path / "bad", 3, 5)
    plan.close()
