"""Builds magpy_gb300/pyx/core.pyx, the reference-style `magpy.core.simulate`
binding over include/magpy_simulation.hpp, into an importable extension
(magpy_gb300.pyx.core) linked against magpy_gb300/_lib/libmagpy_gpu.so.

Needs Cython and a C++ compiler; the GPU library is built first
(magpy_gb300/build.py).  Usage: python magpy_gb300/pyx/build_pyx.py
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def build() -> str:
    from Cython.Build import cythonize  # ImportError without Cython
    import numpy as np
    from magpy_gb300 import build as gpu_build
    lib = gpu_build.build()
    pyx = os.path.join(HERE, "core.pyx")
    cpp = os.path.join(HERE, "_build", "core.cpp")
    os.makedirs(os.path.dirname(cpp), exist_ok=True)
    cythonize([pyx], quiet=True, force=True, language_level=3)
    os.replace(os.path.join(HERE, "core.cpp"), cpp)
    out = os.path.join(HERE, "core" + sysconfig.get_config_var("EXT_SUFFIX"))
    libdir = os.path.dirname(lib)
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-shared", "-fPIC", "-w",
           f"-I{sysconfig.get_paths()['include']}", f"-I{np.get_include()}",
           f"-I{os.path.join(ROOT, 'include')}", cpp, "-o", out, f"-L{libdir}", "-lmagpy_gpu",
           f"-Wl,-rpath,{libdir}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        raise RuntimeError("compiling the core.pyx binding failed")
    return out


if __name__ == "__main__":
    print(build())
