"""Members split over two processes (gloo on CPU) against one process.

Each rank integrates its member range with the FP64 oracle (the reference's
algorithm and its mt19937 noise per member seed), the ranks exchange their
partial cluster magnetisations, and the ensemble statistics must equal the
single-process run of all members: per-member trajectories bit for bit,
the ensemble magnetisation and the energy dissipated to 1e-13 relative (the
sums are added in another order).  A GPU test runs the same split with the
default member integrator (the GPU kernels) in both ranks.
"""
import os
import socket
import tempfile

import numpy as np
import pytest

from magpy_gb300.replicas import member_range


def test_member_range_partitions():
    for E in (0, 1, 2, 5, 7, 64, 1001):
        for W in (1, 2, 3, 4, 8):
            spans = [member_range(E, W, r) for r in range(W)]
            assert spans[0][0] == 0 and spans[-1][1] == E
            for (a, b), (c, d) in zip(spans, spans[1:]):
                assert b == c
            sizes = [b - a for a, b in spans]
            assert max(sizes) - min(sizes) <= 1
            assert sizes == sorted(sizes, reverse=True)
    with pytest.raises(ValueError):
        member_range(4, 2, 2)


def _model():
    from magpy_gb300.model import EnsembleModel, Model
    base = Model(radius=[6e-9, 7e-9], anisotropy=[2e4, 2.2e4],
                 anisotropy_axis=[[0, 0, 1.0], [0.6, 0, 0.8]],
                 magnetisation_direction=[[0, 0, 1.0], [0, 0.6, 0.8]],
                 location=[[0, 0, 0.0], [0, 0, 2e-8]], magnetisation=4e5, damping=0.1,
                 temperature=300.0, field_shape="sine", field_frequency=3e8,
                 field_amplitude=1e4)
    return EnsembleModel(5, base)


SIM = dict(end_time=2e-11, time_step=1e-13, max_samples=21, random_state=7)


def _oracle_members(oracle):
    from magpy_gb300.results import EnsembleResults, Results

    def run(members, seeds, end_time, time_step, max_samples, **kw):
        model = _model()
        out = []
        for e, seed in zip(members, seeds):
            m = model.models[e]
            r = oracle.full_dynamics(m.radius, m.anisotropy, m.anisotropy_axis,
                                     m.magnetisation_direction, m.location, m.magnetisation,
                                     m.damping, m.temperature, use_implicit=False,
                                     time_step=time_step, end_time=end_time,
                                     max_samples=max_samples, seed=int(seed),
                                     field_shape=m.field_shape,
                                     field_amplitude=m.field_amplitude,
                                     field_frequency=m.field_frequency)
            n = r["x"].shape[0]
            out.append(Results(time=r["time"], field=r["field"],
                               x={i: r["x"][i] for i in range(n)},
                               y={i: r["y"][i] for i in range(n)},
                               z={i: r["z"][i] for i in range(n)}, N=n, status=r["status"]))
        return EnsembleResults(out)
    return run


def _worker(rank, world, port, outdir):
    import torch.distributed as dist
    from oracle import pyoracle
    from magpy_gb300.replicas import max_over_ranks, simulate_shard
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", world_size=world,
                            rank=rank)
    try:
        res = simulate_shard(_model(), group=None,
                             simulate_members=_oracle_members(pyoracle.Oracle()), **SIM)
        z = np.stack([np.stack([r.z[i] for i in sorted(r.z)]) for r in res.local.results])
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), start=res.start, stop=res.stop,
                 M=np.stack([res.ensemble_magnetisation(d) for d in "xyz"]),
                 sar=res.energy_dissipated(), z=z, time=res.time, field=res.field,
                 tmax=max_over_ranks(1.5 + rank))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sharded_ensemble_matches_one_process(oracle):
    import torch.multiprocessing as mp
    world = 2
    with tempfile.TemporaryDirectory() as d:
        ctx = mp.get_context("spawn")
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, world, port, d)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        parts = [dict(np.load(os.path.join(d, f"rank{r}.npz"))) for r in range(world)]
    single = _oracle_members(oracle)(range(5), _model().seeds(SIM["random_state"]),
                                     SIM["end_time"], SIM["time_step"], SIM["max_samples"])
    M1 = np.stack([single.ensemble_magnetisation(d) for d in "xyz"])
    sar1 = single.energy_dissipated()
    z1 = np.stack([np.stack([r.z[i] for i in sorted(r.z)]) for r in single.results])
    assert [(int(p["start"]), int(p["stop"])) for p in parts] == [(0, 3), (3, 5)]
    np.testing.assert_array_equal(np.concatenate([p["z"] for p in parts]), z1)
    for p in parts:
        np.testing.assert_allclose(p["M"], M1, rtol=1e-13, atol=1e-13 * np.abs(M1).max())
        np.testing.assert_allclose(p["sar"], sar1, rtol=1e-12)
        np.testing.assert_array_equal(p["time"], single.time)
        np.testing.assert_array_equal(p["field"], single.field)
        assert float(p["tmax"]) == 1.5 + world - 1
    # the ranks agree bit for bit
    np.testing.assert_array_equal(parts[0]["M"], parts[1]["M"])


def test_max_over_ranks_single_process():
    from magpy_gb300.replicas import max_over_ranks
    assert max_over_ranks(3.5) == 3.5


def _gpu_worker(rank, world, port, outdir):
    import torch.distributed as dist
    from magpy_gb300.replicas import simulate_shard
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", world_size=world,
                            rank=rank)
    try:
        res = simulate_shard(_model(), group=None, **SIM)  # the default GPU member path
        z = np.stack([np.stack([r.z[i] for i in sorted(r.z)]) for r in res.local.results])
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), start=res.start, stop=res.stop,
                 M=np.stack([res.ensemble_magnetisation(d) for d in "xyz"]),
                 sar=res.energy_dissipated(), z=z)
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_sharded_gpu_members_match_one_process(gpu_lib):
    """The replica path with its default member integrator (the GPU kernels):
    two ranks, each integrating its member range on the GPU, against one
    process running every member.  The ranks share this machine's one GPU;
    their kernels are independent (the only exchange is the host-side gloo
    all-gather of the partial magnetisations), so nothing on the device waits
    for another rank.  Per-member trajectories bit for bit (the same kernel on
    the same seeds), ensemble statistics to 1e-13."""
    import torch.multiprocessing as mp
    world = 2
    with tempfile.TemporaryDirectory() as d:
        ctx = mp.get_context("spawn")
        port = _free_port()
        procs = [ctx.Process(target=_gpu_worker, args=(r, world, port, d)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(300)
            assert p.exitcode == 0
        parts = [dict(np.load(os.path.join(d, f"rank{r}.npz"))) for r in range(world)]
    single = _model().simulate(SIM["end_time"], SIM["time_step"], SIM["max_samples"],
                               SIM["random_state"])
    M1 = np.stack([single.ensemble_magnetisation(c) for c in "xyz"])
    z1 = np.stack([np.stack([r.z[i] for i in sorted(r.z)]) for r in single.results])
    np.testing.assert_array_equal(np.concatenate([p["z"] for p in parts]), z1)
    for p in parts:
        np.testing.assert_allclose(p["M"], M1, rtol=1e-13, atol=1e-13 * np.abs(M1).max())
        np.testing.assert_allclose(p["sar"], single.energy_dissipated(), rtol=1e-12)
