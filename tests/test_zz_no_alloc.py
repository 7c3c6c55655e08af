"""The entry point that allocates no device memory.

magpy_ensemble_dynamics_noalloc serves callers that cannot let a library
allocate on the device (a framework that owns all GPU memory through its own
pool and budget, or a latency-critical loop where cudaFree would wait for the
whole device).  It keeps its tables in a fixed static device array instead.
These tests call it through the C-ABI with device buffers and compare it with
magpy_ensemble_dynamics, twice in a row so that the second call runs on the
array the first call left behind.  This file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest


def _desc(_lib, keep, E, geo, seeds, window_end, dt, samples, on_device):
    d = _lib.EnsembleDesc()
    d.n_members, d.n_particles = E, int(geo["radius"].shape[0])
    for k, v in geo.items():
        setattr(d, k, _lib.vptr(v))
    d.magnetisation, d.damping, d.temperature = 4e5, 0.1, 300.0
    d.field_amplitude, d.field_frequency = 1e4, 3e8
    d.field_shape = _lib.FIELD_SHAPES["sine"]
    d.renorm, d.interactions, d.use_implicit = 0, 1, 0
    d.eps, d.max_iter = 1e-9, 1000
    d.time_step, d.end_time, d.max_samples = dt, window_end, samples
    d.seeds = _lib.vptr(seeds)
    d.precision = _lib.PRECISIONS["mixed"]
    d.buffers_on_device = int(on_device)
    keep.append((geo, seeds))
    return d


def _geometry(rng, n):
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    side = int(np.ceil(n ** (1 / 3)))
    grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    return {"radius": rng.uniform(6e-9, 9e-9, n), "anisotropy": rng.uniform(1.5e4, 2.5e4, n),
            "anisotropy_axis": axes, "magnetisation_direction": axes.copy(),
            "location": grid * 22e-9 + rng.uniform(-1e-9, 1e-9, size=(n, 3))}


@pytest.mark.gpu
def test_noalloc_matches_allocating_entry_point():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from magpy_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(99)
    keep = []
    # two calls in a row with different shapes, so the second reuses the array
    for E, n, window in ((48, 8, 300), (20, 40, 150)):
        geo = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in _geometry(rng, n).items()}
        seeds = rng.integers(0, 2**31 - 1, size=E).astype(np.int64)
        dt, S = 5e-14, 7
        end = dt * window
        # existing entry point, host buffers
        P = E * n
        ref = {k: np.empty((S, P)) for k in ("mx", "my", "mz")}
        ref_t, ref_f = np.empty((E, S)), np.empty((E, S))
        ref_st, ref_k = np.empty(E, dtype=np.int32), np.empty(E, dtype=np.int64)
        d = _desc(_lib, keep, E, geo, seeds, end, dt, S, False)
        o = _lib.EnsembleOut(ref["mx"].ctypes.data, ref["my"].ctypes.data, ref["mz"].ctypes.data,
                             ref_t.ctypes.data, ref_f.ctypes.data, ref_st.ctypes.data,
                             ref_k.ctypes.data)
        _lib.check(L.magpy_ensemble_dynamics(C.byref(d), C.byref(o), None))
        # no-allocation entry point, device buffers
        dev = {k: torch.from_numpy(v).cuda() for k, v in geo.items()}
        dseeds = torch.from_numpy(seeds).cuda()
        out = {k: torch.full((S, P), float("nan"), dtype=torch.float64, device="cuda")
               for k in ("mx", "my", "mz")}
        t = torch.empty((E, S), dtype=torch.float64, device="cuda")
        f = torch.empty((E, S), dtype=torch.float64, device="cuda")
        st = torch.full((E,), -1, dtype=torch.int32, device="cuda")
        k = torch.full((E,), -1, dtype=torch.int64, device="cuda")
        d2 = _desc(_lib, keep, E, dev, dseeds, end, dt, S, True)
        o2 = _lib.EnsembleOut(out["mx"].data_ptr(), out["my"].data_ptr(), out["mz"].data_ptr(),
                              t.data_ptr(), f.data_ptr(), st.data_ptr(), k.data_ptr())
        stream = torch.cuda.current_stream().cuda_stream
        _lib.check(L.magpy_ensemble_dynamics_noalloc(C.byref(d2), C.byref(o2), stream))
        torch.cuda.synchronize()
        for c in ("mx", "my", "mz"):
            np.testing.assert_allclose(out[c].cpu().numpy(), ref[c], rtol=1e-12, atol=0)
        np.testing.assert_allclose(t.cpu().numpy(), ref_t, rtol=1e-12, atol=0)
        np.testing.assert_allclose(f.cpu().numpy(), ref_f, rtol=1e-12, atol=0)
        assert np.array_equal(st.cpu().numpy(), ref_st)
        assert np.array_equal(k.cpu().numpy(), ref_k)
        assert np.all(ref_st == 0)


def test_noalloc_rejects_ensembles_beyond_its_scratch():
    """An ensemble larger than the static array is refused with a message
    (checked before any device work, so this runs without a GPU)."""
    from magpy_gb300 import _lib
    L = _lib.lib()
    E, n = 200_000, 64  # 12.8 M particles: far beyond 32 MiB of tables
    geo = {"radius": np.zeros(n), "anisotropy": np.zeros(n), "anisotropy_axis": np.zeros((n, 3)),
           "magnetisation_direction": np.zeros((n, 3)), "location": np.zeros((n, 3))}
    seeds = np.zeros(E, dtype=np.int64)
    d = _desc(_lib, [], E, geo, seeds, 1e-11, 5e-14, 5, True)
    o = _lib.EnsembleOut()
    rc = L.magpy_ensemble_dynamics_noalloc(C.byref(d), C.byref(o), None)
    assert rc == -1
    assert b"MAGPY_NOALLOC_SCRATCH_BYTES" in L.magpy_last_error_string()
