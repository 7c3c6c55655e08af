"""Seeded cluster geometries drawn on the device (magpy_generate_clusters)."""
import numpy as np
import pytest

from philox_ref import philox4x32_10

pytestmark = pytest.mark.gpu


def _u53(hi, lo):
    b = (hi.astype(np.uint64) >> np.uint64(5)) << np.uint64(26) | (lo.astype(np.uint64) >> np.uint64(6))
    return (b.astype(np.float64) + 0.5) * 2.0 ** -53


def _draw(seed, i, j, tag):
    i = np.asarray(i, dtype=np.uint64)
    z = np.zeros_like(i)
    return philox4x32_10(i, z + np.uint64(j), z + np.uint64(tag), z + np.uint64(0x9E01),
                         seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)


def test_radii_and_axes_match_numpy_statement(gpu_lib):
    from magpy_gb300 import core
    seeds = np.array([7, 123456789, 2**40 + 3], dtype=np.int64)
    n = 37
    g = core.generate_clusters(3, n, seeds, median_radius=8e-9, sigma=0.25, moments="random")
    assert np.all(g["status"] == 0)
    for e, s in enumerate(seeds):
        r = _draw(int(s), np.arange(n), 0, 0x6E01)
        z = np.sqrt(-2.0 * np.log(_u53(r[0], r[1]))) * np.cos(2 * np.pi * _u53(r[2], r[3]))
        np.testing.assert_allclose(g["radius"][e], 8e-9 * np.exp(0.25 * z), rtol=1e-13)
        for tag, key in ((0x6E02, "anisotropy_axis"), (0x6E03, "magnetisation_direction")):
            a = _draw(int(s), np.arange(n), 0, tag)
            zz = 2.0 * _u53(a[0], a[1]) - 1.0
            ph = 2 * np.pi * _u53(a[2], a[3])
            sz = np.sqrt(np.maximum(0.0, 1.0 - zz * zz))
            want = np.stack([sz * np.cos(ph), sz * np.sin(ph), zz], 1)
            np.testing.assert_allclose(g[key][e], want, rtol=0, atol=1e-14)


def test_sphere_packing_constraints_and_determinism(gpu_lib):
    from magpy_gb300 import core
    E, n, spacing, phi = 48, 64, 2.2, 0.3
    seeds = np.arange(E) * 7919 + 5
    g = core.generate_clusters(E, n, seeds, spacing=spacing, packing_fraction=phi)
    assert np.all(g["status"] == 0)
    for e in range(E):
        r, loc = g["radius"][e], g["location"][e]
        R = 0.5 * spacing * r.mean() * (n / phi) ** (1 / 3)
        assert np.all(np.linalg.norm(loc, axis=1) <= R * (1 + 1e-12))
        d = np.linalg.norm(loc[:, None] - loc[None], axis=2)
        need = spacing * 0.5 * (r[:, None] + r[None])
        np.fill_diagonal(d, np.inf)
        assert np.all(d >= need * (1 - 1e-12))
        np.testing.assert_allclose(g["anisotropy_axis"][e], g["magnetisation_direction"][e])
    g2 = core.generate_clusters(E, n, seeds, spacing=spacing, packing_fraction=phi)
    for k in ("radius", "anisotropy_axis", "location"):
        np.testing.assert_array_equal(g[k], g2[k])
    g3 = core.generate_clusters(E, n, seeds + 1, spacing=spacing, packing_fraction=phi)
    assert not np.array_equal(g["location"], g3["location"])


def test_axes_are_uniform_on_the_sphere(gpu_lib):
    from magpy_gb300 import core
    g = core.generate_clusters(256, 64, np.arange(256) + 1, layout="chain")
    a = g["anisotropy_axis"].reshape(-1, 3)
    np.testing.assert_allclose(np.linalg.norm(a, axis=1), 1.0, atol=1e-14)
    M = a.shape[0]
    assert np.all(np.abs(a.mean(0)) < 5 / np.sqrt(3 * M))
    cov = a.T @ a / M
    np.testing.assert_allclose(cov, np.eye(3) / 3, atol=5 * np.sqrt(2 / 15 / M))


def test_chain_layout(gpu_lib):
    from magpy_gb300 import core
    g = core.generate_clusters(3, 5, [1, 2, 3], layout="chain", spacing=2.5)
    for e in range(3):
        mr = g["radius"][e].mean()
        want = np.stack([np.zeros(5), np.zeros(5), 2.5 * mr * np.arange(5)], 1)
        np.testing.assert_allclose(g["location"][e], want, rtol=1e-15, atol=0)


def test_overfull_packing_reports_and_stops(gpu_lib):
    from magpy_gb300 import core
    # 0.6 of exclusion-sphere packing with 2.2x spacing cannot be reached by
    # random sequential placement: members stop with status 1 and NaN tails
    g = core.generate_clusters(4, 200, [1, 2, 3, 4], packing_fraction=0.6, max_rounds=8)
    assert np.all(g["status"] == 1)
    for e in range(4):
        loc = g["location"][e]
        bad = np.isnan(loc[:, 0])
        assert bad.any() and not bad[0]
        first = np.argmax(bad)
        assert np.all(bad[first:]) and not np.any(bad[:first])


def test_device_outputs_equal_host_outputs_and_feed_an_ensemble(gpu_lib):
    torch = pytest.importorskip("torch")
    from magpy_gb300 import core
    E, n = 8, 27
    seeds = np.arange(E) + 100
    h = core.generate_clusters(E, n, seeds)
    d = core.generate_clusters(E, n, seeds, device="cuda")
    for k in ("radius", "anisotropy_axis", "magnetisation_direction", "location"):
        np.testing.assert_array_equal(d[k].cpu().numpy(), h[k])
    arr = core.simulate_ensemble(E, h["radius"], np.full((E, n), 2e4), h["anisotropy_axis"],
                                 h["magnetisation_direction"], h["location"], 4e5, 0.1, 300.0,
                                 False, True, False, 5e-14, 5e-14 * 200, 3, seeds,
                                 per_member_geometry=True, precision="mixed")
    assert np.all(arr.status == 0)
