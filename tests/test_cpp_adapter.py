"""The reference's C++ entry point, simulation::full_dynamics with the
signature of include/simulation.hpp:74-94, as include/magpy_simulation.hpp
provides it over the C-ABI.  tests/cpp/test_simulation_adapter.cpp is
compiled here with the host C++ compiler and linked against
libmagpy_gpu.so: on the CPU it checks the argument handling (exceptions
before any device work), on the GPU it runs a cluster and is compared with
magpy_gb300.core.simulate on the same arguments and seed."""
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def adapter_exe(tmp_path_factory):
    cxx = os.environ.get("CXX") or shutil.which("g++")
    if not cxx:
        pytest.skip("no C++ compiler")
    from magpy_gb300 import build
    lib = build.build()
    libdir = os.path.dirname(lib)
    exe = str(tmp_path_factory.mktemp("cpp") / "test_simulation_adapter")
    cmd = [cxx, "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "test_simulation_adapter.cpp"), "-o", exe,
           f"-L{libdir}", "-lmagpy_gpu", f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_adapter_argument_checks(adapter_exe):
    r = subprocess.run([adapter_exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "checks ok" in r.stdout


@pytest.mark.gpu
def test_adapter_run_matches_python_entry(gpu_lib, adapter_exe):
    """The same three-particle run through the C++ adapter and through
    magpy_gb300.core.simulate: the same kernel on the same generator
    increments, so bit for bit."""
    from magpy_gb300 import core
    r = subprocess.run([adapter_exe, "run"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = np.array([[float(v) for v in line.split()] for line in r.stdout.split("\n") if line])
    axes = np.array([[0, 0, 1.0], [0, 1.0, 0], [1.0, 0, 0]])
    loc = np.array([[0, 0, 0], [2e-8, 0, 0], [0, 2.1e-8, 0]])
    g = core.simulate(np.array([7e-9, 6e-9, 6.5e-9]), np.array([2e4, 2.2e4, 1.9e4]), axes, axes,
                      loc, 4e5, 0.1, 300.0, False, True, False, 1e-13, 2e-11, 11, 4321, "sine",
                      1e4, 3e9, 1e-9)
    for i in range(3):
        sel = rows[rows[:, 0] == i]
        assert np.array_equal(sel[:, 2], g["x"][i])
        assert np.array_equal(sel[:, 3], g["y"][i])
        assert np.array_equal(sel[:, 4], g["z"][i])
        assert np.array_equal(sel[:, 5], g["field"])
        assert np.array_equal(sel[:, 6], g["time"])
