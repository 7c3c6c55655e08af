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


def _desc(_lib, keep, E, geo, seeds, window_end, dt, samples, on_device, shape="sine",
          per_member=False, noise=None, noise_per_member=0):
    d = _lib.EnsembleDesc()
    n = int(geo["radius"].shape[0]) // (E if per_member else 1)
    d.n_members, d.n_particles = E, n
    d.per_member_geometry = int(per_member)
    for k, v in geo.items():
        setattr(d, k, _lib.vptr(v))
    d.magnetisation, d.damping, d.temperature = 4e5, 0.1, 300.0
    d.field_amplitude, d.field_frequency = 1e4, 3e8
    d.field_shape = _lib.FIELD_SHAPES[shape]
    d.renorm, d.interactions, d.use_implicit = 0, 1, 0
    d.eps, d.max_iter = 1e-9, 1000
    d.time_step, d.end_time, d.max_samples = dt, window_end, samples
    d.seeds = _lib.vptr(seeds)
    if noise is not None:
        d.noise = _lib.vptr(noise)
        d.noise_per_member = noise_per_member
    d.precision = _lib.PRECISIONS["mixed"]
    d.buffers_on_device = int(on_device)
    keep.append((geo, seeds, noise))
    return d


def _geometry(rng, n, members=1):
    rows = n * members
    axes = rng.normal(size=(rows, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    side = int(np.ceil(n ** (1 / 3)))
    grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    grid = np.tile(grid, (members, 1))
    # the members' anisotropy constants are the same set (one mean K, so one
    # reduced time step for the launch); radii, axes and positions differ
    k = np.tile(rng.uniform(1.5e4, 2.5e4, n), members)
    return {"radius": rng.uniform(6e-9, 9e-9, rows), "anisotropy": k,
            "anisotropy_axis": axes, "magnetisation_direction": axes.copy(),
            "location": grid * 22e-9 + rng.uniform(-1e-9, 1e-9, size=(rows, 3))}


# (members, particles, window steps, waveform, one geometry per member, injected noise)
CASES = [
    ((48, 8, 300, "sine", False, False), (20, 40, 150, "sine", False, False)),
    ((12, 6, 200, "square", True, False), (9, 33, 120, "constant", True, False)),
    ((16, 5, 180, "constant", False, True), (10, 12, 90, "sine", True, True)),
]


@pytest.mark.gpu
@pytest.mark.parametrize("calls", CASES, ids=["shared-geometry", "per-member-geometry",
                                              "injected-noise"])
def test_noalloc_matches_allocating_entry_point(calls):
    """Two calls in a row (different shapes, so the second runs on what the
    first left in the array), each against the allocating entry point with
    host buffers on the same inputs: trajectories to 1e-12 relative (the
    same kernel on the same tables), times, fields, status and steps."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from magpy_gb300 import _lib
    L = _lib.lib()
    rng = np.random.default_rng(99)
    keep = []
    for E, n, window, shape, per_member, injected in calls:
        geo = {k: np.ascontiguousarray(v, dtype=np.float64)
               for k, v in _geometry(rng, n, E if per_member else 1).items()}
        seeds = rng.integers(0, 2**31 - 1, size=E).astype(np.int64)
        dt, S = 5e-14, 7
        end = dt * window
        noise, npm = None, 0
        if injected:
            npm = 3 * n * (window + 2)
            noise = rng.normal(size=(E, npm))
        # existing entry point, host buffers
        P = E * n
        ref = {k: np.empty((S, P)) for k in ("mx", "my", "mz")}
        ref_t, ref_f = np.empty((E, S)), np.empty((E, S))
        ref_st, ref_k = np.empty(E, dtype=np.int32), np.empty(E, dtype=np.int64)
        d = _desc(_lib, keep, E, geo, seeds, end, dt, S, False, shape, per_member, noise, npm)
        o = _lib.EnsembleOut(ref["mx"].ctypes.data, ref["my"].ctypes.data, ref["mz"].ctypes.data,
                             ref_t.ctypes.data, ref_f.ctypes.data, ref_st.ctypes.data,
                             ref_k.ctypes.data)
        _lib.check(L.magpy_ensemble_dynamics(C.byref(d), C.byref(o), None))
        # no-allocation entry point, device buffers, on a non-default stream
        # whose queued work produced the inputs
        stream = torch.cuda.Stream()
        with torch.cuda.stream(stream):
            dev = {k: torch.from_numpy(v).to("cuda", non_blocking=False) for k, v in geo.items()}
            dseeds = torch.from_numpy(seeds).cuda()
            dnoise = torch.from_numpy(noise).cuda() if injected else None
            out = {k: torch.full((S, P), float("nan"), dtype=torch.float64, device="cuda")
                   for k in ("mx", "my", "mz")}
            t = torch.empty((E, S), dtype=torch.float64, device="cuda")
            f = torch.empty((E, S), dtype=torch.float64, device="cuda")
            st = torch.full((E,), -1, dtype=torch.int32, device="cuda")
            k = torch.full((E,), -1, dtype=torch.int64, device="cuda")
        d2 = _desc(_lib, keep, E, dev, dseeds, end, dt, S, True, shape, per_member,
                   dnoise, npm)
        o2 = _lib.EnsembleOut(out["mx"].data_ptr(), out["my"].data_ptr(), out["mz"].data_ptr(),
                              t.data_ptr(), f.data_ptr(), st.data_ptr(), k.data_ptr())
        _lib.check(L.magpy_ensemble_dynamics_noalloc(C.byref(d2), C.byref(o2),
                                                     stream.cuda_stream))
        torch.cuda.synchronize()
        for c in ("mx", "my", "mz"):
            np.testing.assert_allclose(out[c].cpu().numpy(), ref[c], rtol=1e-12, atol=0)
        np.testing.assert_allclose(t.cpu().numpy(), ref_t, rtol=1e-12, atol=0)
        np.testing.assert_allclose(f.cpu().numpy(), ref_f, rtol=1e-12, atol=0)
        assert np.array_equal(st.cpu().numpy(), ref_st)
        assert np.array_equal(k.cpu().numpy(), ref_k)
        assert np.all(ref_st == 0)


def _tiny(_lib, E=4, n=3):
    geo = {"radius": np.full(n, 7e-9), "anisotropy": np.full(n, 2e4),
           "anisotropy_axis": np.tile([0.0, 0.0, 1.0], (n, 1)),
           "magnetisation_direction": np.tile([0.0, 0.0, 1.0], (n, 1)),
           "location": np.arange(3 * n, dtype=np.float64).reshape(n, 3) * 2e-8}
    return geo, np.zeros(E, dtype=np.int64)


def test_noalloc_rejects_ensembles_beyond_its_scratch():
    """An ensemble larger than the static array is refused with a message
    (checked before any device work, so this runs without a GPU)."""
    from magpy_gb300 import _lib
    L = _lib.lib()
    E, n = 200_000, 64  # 12.8 M particles: far beyond 32 MiB of tables
    geo, seeds = _tiny(_lib, E, n)
    d = _desc(_lib, [], E, geo, seeds, 1e-11, 5e-14, 5, True)
    o = _lib.EnsembleOut()
    rc = L.magpy_ensemble_dynamics_noalloc(C.byref(d), C.byref(o), None)
    assert rc == -1
    assert b"MAGPY_NOALLOC_SCRATCH_BYTES" in L.magpy_last_error_string()


def test_noalloc_rejects_sizes_whose_products_would_wrap():
    """Member and sample counts so large that E * n or S * 8 would wrap a
    64-bit product are refused by the division-first bounds."""
    from magpy_gb300 import _lib
    L = _lib.lib()
    geo, seeds = _tiny(_lib)
    for E, S in ((2**61, 5), (4, 2**62)):
        d = _desc(_lib, [], 4, geo, seeds, 1e-11, 5e-14, 5, True)
        d.n_members, d.max_samples = E, S
        rc = L.magpy_ensemble_dynamics_noalloc(C.byref(d), C.byref(_lib.EnsembleOut()), None)
        assert rc == -1
        assert b"MAGPY_NOALLOC_SCRATCH_BYTES" in L.magpy_last_error_string()


def test_noalloc_rejects_partial_trajectory_outputs():
    """The kernel writes mx, my and mz together: a caller giving some of them
    and NULL for the others is refused before any device work."""
    from magpy_gb300 import _lib
    L = _lib.lib()
    geo, seeds = _tiny(_lib)
    d = _desc(_lib, [], 4, geo, seeds, 1e-11, 5e-14, 5, True)
    fake = C.c_void_p(0x1000)  # never dereferenced: the call is refused first
    for o in (_lib.EnsembleOut(mx=fake), _lib.EnsembleOut(mx=fake, my=fake),
              _lib.EnsembleOut(mz=fake)):
        rc = L.magpy_ensemble_dynamics_noalloc(C.byref(d), C.byref(o), None)
        assert rc == -1
        assert b"all set or all NULL" in L.magpy_last_error_string()
