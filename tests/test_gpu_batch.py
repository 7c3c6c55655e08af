"""Uneven-size ensembles in one CUDA-graph launch with the autotuner."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lattice(n, spacing=20e-9):
    side = int(np.ceil(n ** (1 / 3)))
    grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    return grid * spacing


def _group(n, E, precision, rng, end_steps=300):
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    return dict(n_members=E, radius=np.full(n, 7e-9), anisotropy=np.full(n, 2e4),
                anisotropy_axis=axes, magnetisation_direction=axes, location=_lattice(n),
                magnetisation=4e5, damping=0.1, temperature=300.0, renorm=False,
                interactions=True, use_implicit=False, time_step=1e-13,
                end_time=1e-13 * end_steps, max_samples=7,
                seeds=rng.integers(0, 2**31 - 1, size=E), field_shape="sine",
                field_amplitude=5e3, field_frequency=1e9, precision=precision)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_matches_single_groups(gpu_lib, precision):
    from magpy_gb300 import core
    rng = np.random.default_rng(7)
    groups = [_group(n, E, precision, rng) for n, E in ((1, 70), (8, 33), (27, 20), (64, 40),
                                                         (125, 9))]
    batch = core.EnsembleBatch(groups, autotune=True)
    for rep in range(2):  # graph replays give the same results
        batch.run()
        for i, g in enumerate(groups):
            prec, bw, mpw, ms = batch.choice(i)
            if precision == "fp64":
                assert prec == "fp64"
            arr = batch.groups[i].arrays()
            assert np.all(arr.status == 0)
            single = core.simulate_ensemble(*[g[k] for k in core.EnsembleBatch._POS],
                                            g["field_shape"], g["field_amplitude"],
                                            g["field_frequency"], precision=prec)
            # same kernel, same increments: identical except for the CTA shape,
            # which does not change any arithmetic
            np.testing.assert_array_equal(arr.mz, single.mz)
            np.testing.assert_array_equal(arr.mx, single.mx)
    batch.close()
