"""The C-ABI library without a GPU: it loads, exports every entry point that
include/magpy_gpu.h declares, and validates arguments before any device work."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def _declared():
    src = open(os.path.join(ROOT, "include", "magpy_gpu.h")).read()
    return sorted(set(re.findall(r"\b(magpy_[a-z_0-9]+)\s*\(", src)))


def test_library_exports_every_declared_symbol():
    from magpy_gb300 import _lib
    L = _lib.lib()
    names = _declared()
    assert len(names) >= 8
    for name in names:
        assert hasattr(L, name), name
    assert set(names) == set(_lib.SYMBOLS)


def test_version_and_error_string():
    from magpy_gb300 import _lib
    assert b"sm_103a" in _lib.lib().magpy_version()
    assert isinstance(_lib.lib().magpy_last_error_string(), bytes)


@pytest.mark.parametrize("dt,end,S", [(1.7e-3, 0.5, 21), (1e-3, 0.05, 6), (1e-2, 0.05, 23),
                                      (2e-3, 0.2, 9), (1e-3, 0.03, 4), (0.1, 0.0, 1)])
def test_step_count_matches_oracle(oracle, dt, end, S):
    from magpy_gb300 import core
    from oracle.pyoracle import reduced_inputs
    k = core.step_count(dt, end, S)
    if S > 1:
        inp = reduced_inputs(np.random.default_rng(0), 1)
        out = oracle.full_dynamics_reduced(inp, dt=dt, end_time=end, max_samples=S,
                                           noise=np.zeros(3 * (k + 5)))
        assert out["steps"] == k
    else:
        assert k == 0


def test_step_count_rejects_bad_input():
    from magpy_gb300 import core
    from magpy_gb300._lib import MagpyError
    with pytest.raises(MagpyError):
        core.step_count(0.0, 1.0, 10)
    with pytest.raises(MagpyError):
        core.step_count(1e-12, 1.0, 10)   # 1e12 steps would wrap the 32-bit counter
    with pytest.raises(MagpyError):
        core.step_count(1e-3, 1.0, 0)


def test_ensemble_validates_before_device_work():
    from magpy_gb300 import core
    from magpy_gb300._lib import MagpyError
    with pytest.raises(MagpyError, match="max_samples"):
        core.simulate_ensemble(2, [7e-9], [2e4], [[0, 0, 1]], [[0, 0, 1]], [[0, 0, 0]], 4e5, 0.1,
                               300, False, True, False, 1e-13, 1e-11, 0, [1, 2])
    with pytest.raises(KeyError):
        core.simulate_ensemble(2, [7e-9], [2e4], [[0, 0, 1]], [[0, 0, 1]], [[0, 0, 0]], 4e5, 0.1,
                               300, False, True, False, 1e-13, 1e-11, 5, [1, 2],
                               field_shape="triangle")
    with pytest.raises(MagpyError, match="tensor-core mode needs dipolar interactions"):
        core.simulate_ensemble(2, [7e-9, 7e-9], [2e4, 2e4], [[0, 0, 1]] * 2, [[0, 0, 1]] * 2,
                               [[0, 0, 0], [0, 0, 2e-8]], 4e5, 0.1, 300, False, False, True,
                               1e-13, 1e-11, 5, [1, 2], precision="mixed_tc")
    with pytest.raises(MagpyError, match="finite"):
        core.simulate_ensemble(1, [np.nan], [2e4], [[0, 0, 1]], [[0, 0, 1]], [[0, 0, 0]], 4e5,
                               0.1, 300, False, True, False, 1e-13, 1e-11, 5, [1])


def test_save_results_matches_reference_format(tmp_path, reference):
    """magpy_save_results writes the bytes of simulation::save_results."""
    from magpy_gb300 import core
    rng = np.random.default_rng(3)
    arrs = [rng.normal(size=17) for _ in range(5)]
    core.save_results(tmp_path / "ours", *arrs)
    reference.save_results(tmp_path / "ref", *arrs)
    for ext in ("mx", "my", "mz", "field", "time"):
        assert (tmp_path / f"ours.{ext}").read_bytes() == (tmp_path / f"ref.{ext}").read_bytes()
    back = core.load_results(tmp_path / "ours")
    for a, k in zip(arrs, ("mx", "my", "mz", "field", "time")):
        np.testing.assert_array_equal(back[k], a)


def test_save_results_errors(tmp_path):
    from magpy_gb300 import core
    from magpy_gb300._lib import MagpyError
    with pytest.raises(MagpyError, match="I/O error"):
        core.save_results(tmp_path / "missing_dir" / "x", [1.0], [2.0], [3.0], [4.0], [5.0])
    with pytest.raises(ValueError):
        core.save_results(tmp_path / "x", [1.0], [2.0], [3.0], [4.0], [5.0, 6.0])
    # zero samples: five empty files, as the reference writes
    core.save_results(tmp_path / "empty", [], [], [], [], [])
    assert (tmp_path / "empty.time").stat().st_size == 0


def test_dom_validates_before_device_work():
    from magpy_gb300 import core
    from magpy_gb300._lib import MagpyError
    with pytest.raises(MagpyError, match="max_samples"):
        core.simulate_dom_batch([1.0, 0.0], 1e-24, 2e4, 300.0, 4e5, 0.1, 1e-10, 1e-6, 0)
    with pytest.raises(MagpyError, match="time_step"):
        core.simulate_dom_batch([1.0, 0.0], 1e-24, 2e4, 300.0, 4e5, 0.1, -1e-10, 1e-6, 5)
    with pytest.raises(MagpyError, match="field_n_components"):
        core.simulate_dom_batch([1.0, 0.0], 1e-24, 2e4, 300.0, 4e5, 0.1, 1e-10, 1e-6, 5,
                                "square_f", 1e3, 1e5, 0)
    with pytest.raises(KeyError):
        core.simulate_dom_batch([1.0, 0.0], 1e-24, 2e4, 300.0, 4e5, 0.1, 1e-10, 1e-6, 5,
                                "triangle")


def test_generate_clusters_validates_before_device_work():
    from magpy_gb300 import core
    from magpy_gb300._lib import MagpyError
    with pytest.raises(MagpyError, match="n_particles"):
        core.generate_clusters(2, 0, [1, 2])
    with pytest.raises(MagpyError, match="packing_fraction"):
        core.generate_clusters(2, 8, [1, 2], packing_fraction=0.9)
    with pytest.raises(MagpyError, match="median_radius"):
        core.generate_clusters(2, 8, [1, 2], median_radius=-1.0)
    with pytest.raises(ValueError):
        core.generate_clusters(2, 8, [1])
    # no members: nothing to do, nothing launched
    out = core.generate_clusters(0, 8, [])
    assert out["radius"].shape == (0, 8)
