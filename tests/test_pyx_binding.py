"""The core.pyx binding a maintainer of the reference would compile
(magpy_gb300/pyx/core.pyx): the reference's `simulate` signature and result
dictionary (magpy/core.pyx:128-203) over simulation::full_dynamics of
include/magpy_simulation.hpp.  Cythonised and compiled by
magpy_gb300/pyx/build_pyx.py where Cython exists (not on the GPU hosts, whose
image has no Cython: there these tests skip); the CPU tests check the
linkage and the argument handling, the GPU test the results against
magpy_gb300.core.simulate."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def pyx_core():
    pytest.importorskip("Cython")
    from magpy_gb300.pyx import build_pyx
    build_pyx.build()
    import importlib
    return importlib.import_module("magpy_gb300.pyx.core")


def _args():
    axes = np.array([[0, 0, 1.0], [0, 1.0, 0]])
    return (np.array([7e-9, 6e-9]), np.array([2e4, 2.2e4]), axes, axes.copy(),
            np.array([[0, 0, 0], [2e-8, 0, 0.0]]), 4e5, 0.1, 300.0, False, True, False, 1e-13,
            2e-11, 11, 77)


def test_binding_rejects_bad_arguments_before_any_run(pyx_core):
    a = _args()
    with pytest.raises(KeyError):  # the reference's lookup of the field shape
        pyx_core.simulate(*a, field_shape="triangle")
    with pytest.raises(ValueError):
        pyx_core.simulate(*a[:13], 0, 77)
    with pytest.raises(ValueError):  # std::invalid_argument from the C++ entry point
        pyx_core.simulate(a[0], a[1][:1], *a[2:])
    with pytest.raises(ValueError):
        pyx_core.simulate(a[0], a[1], np.zeros((2, 2)), *a[3:])


@pytest.mark.gpu
def test_binding_matches_python_entry(gpu_lib, pyx_core):
    from magpy_gb300 import core
    a = _args()
    b = pyx_core.simulate(*a, field_shape="sine", field_amplitude=1e4, field_frequency=3e9)
    g = core.simulate(*a, "sine", 1e4, 3e9)
    assert b["N"] == 2
    for k in ("time", "field"):
        assert np.array_equal(b[k], g[k])
    for c in "xyz":
        for i in range(2):
            assert np.array_equal(b[c][i], g[c][i])
