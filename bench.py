"""Benchmark: LLG particle-steps/s on the interacting-cluster workload.

Workload (seeded, synthetic): N=64 particles placed uniformly in a sphere with
centre spacing >= 2.2 x the pair's mean radius, log-normal radii (median 8 nm,
sigma 0.2), easy axes uniform on the sphere, initial moments along the easy
axes, full dipolar coupling, AC field 10 kA/m at 300 kHz along z, T = 300 K,
alpha = 0.1, Ms = 400 kA/m, K = 2e4 J/m^3, E = 4096 members sharing the
geometry, dt = 5e-14 s.  The 20 field cycles of that workload are 1.33e9
steps; one benchmark step integrates a fixed window of the trajectory
(default 2000 Heun steps) for the whole ensemble.

value:  particle-steps/s of the chosen (mixed-precision) kernel with the plan,
        inputs and outputs resident on the device (CUDA events on the launch
        stream; L2 flushed between steps).
e2e:    the same metric through the public API (magpy_gb300.core.simulate_ensemble
        on host numpy buffers: planning, host->device copies, the run and the
        device->host copy of the trajectories inside the timed region).
plain:  the FP64-faithful kernel on the same workload (shorter window), and the
        strong error of the chosen form against it on identical increments.

--impl reference runs the CPU restatement of the reference (oracle/, OpenMP
over members, all host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LLG particle-steps/s"
UNIT = "particle-steps/s"
MU0 = 1.25663706e-6


# ---------------------------------------------------------------------------
# workload
# ---------------------------------------------------------------------------
def cluster_geometry(n=64, seed=2024, median_r=8e-9, sigma=0.2, spacing=2.2):
    rng = np.random.default_rng(seed)
    radius = median_r * np.exp(sigma * rng.normal(size=n))
    # sphere sized for a ~30% packing of the exclusion spheres
    r_excl = 0.5 * spacing * radius.mean()
    R = r_excl * (n / 0.3) ** (1 / 3)
    loc = np.empty((n, 3))
    i = 0
    tries = 0
    while i < n:
        tries += 1
        if tries > 1_000_000:
            raise RuntimeError("sphere packing failed")
        p = rng.uniform(-R, R, 3)
        if np.dot(p, p) > R * R:
            continue
        d = np.sqrt(np.sum((loc[:i] - p) ** 2, axis=1))
        if np.all(d >= spacing * 0.5 * (radius[i] + radius[:i])):
            loc[i] = p
            i += 1
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    return dict(radius=radius, anisotropy=np.full(n, 2e4), anisotropy_axis=axes,
                magnetisation_direction=axes.copy(), location=loc)


def workload(members=4096, n=64, window=2000, samples=11):
    geo = cluster_geometry(n)
    dt = 5e-14
    np.random.seed(1234)  # member seeds as magpy/model.py:202-203 derives them
    seeds = np.random.randint(np.iinfo(np.int32).max, size=members).astype(np.int64)
    return dict(geo=geo, E=members, n=n, dt=dt, end_time=dt * window, samples=samples,
                seeds=seeds, ms=4e5, damping=0.1, temperature=300.0, field_shape="sine",
                field_amplitude=1e4, field_frequency=3e5)


def flops_per_particle_step(n):
    # Heun local work 251 flop + two dipolar evaluations, each the dense
    # (3N x 3N)(3N) product counted at 2 flop per entry: 2 * 18 N
    return 251.0 + 36.0 * n


def tc_issued_flops_per_member_step(n, members_per_cta=32):
    # tensor-core kernel: per field evaluation and CTA, D_hi [B_hi | B_lo]
    # (N = 64) and D_lo B_hi (N = 32) over 3N rows padded to 128-row tiles and
    # 3N columns padded to 16; two evaluations per Heun step
    rows = 128 * ((3 * n + 127) // 128)
    kp = 16 * ((3 * n + 15) // 16)
    return 2 * 2.0 * rows * kp * (2 * members_per_cta + members_per_cta) / members_per_cta


# DRAM traffic of one headline launch (N=64, E=4096, 2001 steps, 11 samples)
# from one ncu capture of dram__bytes_read.sum and dram__bytes_write.sum (one
# pass, `-k regex:sllg_tc -s 3 -c 1` over `python bench.py --steps 1 --warmup 3
# --no-plain --no-e2e --no-cpu --no-side`), with the hash of the kernel
# sources it was taken on; the bench reports it only while that hash matches.
DRAM_CAPTURE = {"read": 8.38e6, "write": 10.49e6, "source_sha16": "c017a222e0ef8c14",
                "command": "ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum "
                           "--clock-control none -k regex:sllg_tc -s 3 -c 1"}
KERNEL_SOURCES = ("sllg_tc.cu", "tc_ptx.cuh", "common.cuh", "llg32.cuh", "llg64.cuh")


def kernel_source_hash():
    import hashlib
    h = hashlib.sha256()
    for f in KERNEL_SOURCES:
        with open(os.path.join(ROOT, "magpy_gb300", "csrc", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()[:16]


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
class Plan:
    """A device-resident plan through the C-ABI (magpy_plan_*)."""

    def __init__(self, wl, precision, window_end=None, seeds=None):
        import ctypes as C
        from magpy_gb300 import _lib
        self.C, self._lib = C, _lib
        g = wl["geo"]
        self.keep = {k: np.ascontiguousarray(v, dtype=np.float64) for k, v in g.items()}
        d = _lib.EnsembleDesc()
        d.n_members, d.n_particles = wl["E"], wl["n"]
        for k, v in self.keep.items():
            setattr(d, k, v.ctypes.data)
        d.magnetisation, d.damping, d.temperature = wl["ms"], wl["damping"], wl["temperature"]
        d.field_amplitude, d.field_frequency = wl["field_amplitude"], wl["field_frequency"]
        d.field_shape = _lib.FIELD_SHAPES[wl["field_shape"]]
        d.renorm, d.interactions, d.use_implicit = 0, 1, 0
        d.eps, d.max_iter = 1e-9, 1000
        d.time_step = wl["dt"]
        d.end_time = window_end if window_end is not None else wl["end_time"]
        d.max_samples = wl["samples"]
        self.seeds = np.ascontiguousarray(seeds if seeds is not None else wl["seeds"], dtype=np.int64)
        d.seeds = self.seeds.ctypes.data
        d.precision = _lib.PRECISIONS[precision]
        d.buffers_on_device = 0
        self.handle = C.c_void_p()
        _lib.check(_lib.lib().magpy_plan_create(C.byref(d), C.byref(self.handle), None))
        E, n, S, K = (C.c_int64() for _ in range(4))
        _lib.lib().magpy_plan_shape(self.handle, C.byref(E), C.byref(n), C.byref(S), C.byref(K))
        self.E, self.n, self.S, self.K = E.value, n.value, S.value, K.value

    def run(self, stream_ptr):
        self._lib.check(self._lib.lib().magpy_plan_run(self.handle, stream_ptr))

    def final_state(self):
        C = self.C
        S, P = self.S, self.E * self.n
        mx, my, mz = (np.empty((S, P)) for _ in range(3))
        st = np.empty(self.E, dtype=np.int32)
        o = self._lib.EnsembleOut(mx.ctypes.data, my.ctypes.data, mz.ctypes.data, None, None,
                                  st.ctypes.data, None)
        self._lib.check(self._lib.lib().magpy_plan_copy_out(self.handle, C.byref(o), None))
        return np.stack([mx[-1], my[-1], mz[-1]], 1), st

    def close(self):
        if self.handle:
            self._lib.lib().magpy_plan_destroy(self.handle)
            self.handle = None


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        # the raw samples go to MAGPY_CLOCKS_DIR (default: the temp directory);
        # the JSON line carries their summary
        import tempfile
        out_dir = os.environ.get("MAGPY_CLOCKS_DIR", tempfile.gettempdir())
        self.path = os.path.join(out_dir, f"magpy_clocks_rank{gpu_index}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait(timeout=10)
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


def l2_flush(torch, buf):
    buf.add_(1.0)  # 256 MiB write, larger than the 129 MB L2


def time_plan(torch, plan, steps, warmup, stream, flush):
    sp = stream.cuda_stream
    for _ in range(warmup):
        plan.run(sp)
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            l2_flush(torch, flush)
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        plan.run(sp)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
    return times


def gpu_arm(args):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import magpy_gb300  # noqa: F401  (loads libmagpy_gpu.so)
    from magpy_gb300 import core

    wl = workload(args.members, 64, args.window, args.samples)
    # every rank runs a full ensemble (weak scaling), with its own seeds
    seeds = wl["seeds"] + rank * 1_000_003
    stream = torch.cuda.Stream()
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    plan = Plan(wl, args.precision, seeds=seeds)
    units_per_step = plan.E * plan.n * plan.K

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        times = time_plan(torch, plan, args.steps, args.warmup, stream, flush)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    clocks = clk.summary()
    ms = float(np.sum(times)) / args.steps
    if dist:
        t = torch.tensor([ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = units_per_step * world / (ms * 1e-3)

    out = {}
    if rank == 0:
        flops = flops_per_particle_step(64) * units_per_step
        achieved = flops / (ms * 1e-3) / 1e12
        peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
        peaks = json.load(open(peaks_path)) if os.path.exists(peaks_path) else {}
        fp32_nominal = 152 * 128 * 2 * 2.07e9 / 1e12
        traffic_bytes = (3 * plan.S * plan.E * plan.n * 8)
        tensor_peak = peaks.get("bf16_tflops")
        # DRAM bytes of one launch of the headline workload: a figure from one
        # ncu capture of the two DRAM counters (one pass), valid only for the
        # kernel source it was taken on (checked by hash); the trajectory
        # writes mostly stay in L2
        headline = (args.precision == "mixed_tc" and wl["E"] == 4096 and plan.K == 2001
                    and wl["samples"] == 11)
        src_hash = kernel_source_hash()
        cap = DRAM_CAPTURE
        traffic, traffic_source = None, None
        if headline and src_hash == cap["source_sha16"]:
            traffic = cap["read"] + cap["write"]
            traffic_source = (f"fixed figure: ncu dram__bytes_read.sum + dram__bytes_write.sum "
                              f"of the headline launch, captured on kernel source "
                              f"{cap['source_sha16']} ({cap['command']})")
        elif headline:
            traffic_source = (f"no capture of the current kernel source {src_hash} (last capture "
                              f"on {cap['source_sha16']})")
        out["roofline"] = {
            "achieved": round(achieved, 3), "unit": "TFLOP/s",
            "traffic": traffic, "traffic_source": traffic_source,
            "kernel_source_sha16": src_hash,
            "algorithmic_flops_per_launch": flops,
            "algorithmic_bytes_per_launch": traffic_bytes,
            "hbm_achieved_gbs": round(traffic_bytes / (ms * 1e-3) / 1e9, 3),
            "hbm_peak_gbs": peaks.get("hbm_gbs"),
            "fp32_nominal_tflops": round(fp32_nominal, 1),
            "fp32_nominal_frac": round(achieved / fp32_nominal, 4),
        }
        if args.precision == "mixed_tc" and tensor_peak:
            # the dipolar products run on the tensor cores: the roofline is the
            # measured dense FP16/BF16 rate; the issued MMA work (hi/lo split,
            # padded tiles) is reported beside the algorithmic figure
            mma = tc_issued_flops_per_member_step(64) * plan.E * plan.K
            out["roofline"].update({
                "bound": "tensor", "peak": tensor_peak, "frac": round(achieved / tensor_peak, 4),
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst, of measured)",
                "issued_mma_tflops": round(mma / (ms * 1e-3) / 1e12, 3),
                "issued_mma_frac": round(mma / (ms * 1e-3) / 1e12 / tensor_peak, 4)})
        else:
            out["roofline"].update({
                "bound": "fp32", "peak": round(fp32_nominal, 1),
                "frac": round(achieved / fp32_nominal, 4),
                "peak_source": "nominal FP32 CUDA-core rate, 152 SMs x 128 lanes x 2 flop x "
                               "2.07 GHz (MEASURED_PEAKS.json has no FP32 figure)"})
        # The FP64-faithful form on the window, seeds and in-kernel increments
        # of the timed launch, timed the same way (warm-up, then
        # --plain-repeats launches with the L2 flushed between them), and the
        # strong error of the chosen form against it over that whole window
        # for every member.  Both kernels are deterministic: the chosen
        # plan's final state is the one every timed launch produced.
        # The side measurements characterise one GPU: taken at N = 1 only.
        single = world == 1
        if single and not args.no_plain:
            p64 = Plan(wl, "fp64", seeds=seeds)
            t64 = time_plan(torch, p64, args.plain_repeats, 1, stream, flush)
            a64, s64 = p64.final_state()
            am, sm_ = plan.final_state()
            err = np.linalg.norm(am - a64, axis=1) / np.linalg.norm(a64, axis=1)
            per = p64.E * p64.n * p64.K
            ms64 = float(np.median(t64))
            plain_value = per / (ms64 * 1e-3)
            # GB300's FP64 rate is 1.25 TFLOP/s nominal counting an FMA as two
            # flops; the FP64-faithful kernel is built without contraction (bit
            # parity), so each flop is one FP64 instruction: half that rate
            fp64_nominal = 1.25
            fp64_ceiling = fp64_nominal / 2
            a64_tflops = flops_per_particle_step(64) * per / (ms64 * 1e-3) / 1e12
            out["plain_fp64"] = {
                "value": plain_value, "unit": UNIT, "window_steps": p64.K, "members": p64.E,
                "ms_per_step": ms64, "repeats": len(t64), "ms_all": [float(t) for t in t64],
                "roofline": {"bound": "fp64", "achieved": round(a64_tflops, 4),
                             "unit": "TFLOP/s", "peak": fp64_ceiling,
                             "frac": round(a64_tflops / fp64_ceiling, 4),
                             "frac_of_nominal_with_fma": round(a64_tflops / fp64_nominal, 4),
                             "peak_source": "nominal GB300 FP64 rate 1.25 TFLOP/s (FMA = 2 flop), "
                                            "halved: no contraction in this kernel (not in "
                                            "MEASURED_PEAKS.json)",
                             "note": "algorithmic flop as the headline's; ncu puts the FP64 pipe "
                                     "83.5 % busy on active SMs for this kernel"}}
            out["chosen_vs_plain"] = value / world / plain_value
            out["strong_error_vs_fp64"] = {
                "max_rel": float(err.max()), "mean_rel": float(err.mean()),
                "frac_below_1e-5": float(np.mean(err <= 1e-5)),
                "window_steps": p64.K, "members": p64.E, "particles": int(err.size),
                "status_nonzero": int(np.count_nonzero(s64) + np.count_nonzero(sm_)),
                "note": "final state of the timed window, every particle of every member: "
                        "|m_chosen - m_fp64| / |m_fp64| on identical in-kernel increments; the "
                        "FP64 kernel is bit-identical to the reference CPU path on identical "
                        "increments"}
            p64.close()
        # the CUDA-core mixed form on the same workload, for comparison
        if single and args.precision != "mixed" and not args.no_plain:
            ps = Plan(wl, "mixed", seeds=seeds)
            ts = time_plan(torch, ps, 3, 1, stream, flush)
            out["mixed_cuda_cores"] = {"value": units_per_step / (float(np.mean(ts)) * 1e-3),
                                       "unit": UNIT, "ms_per_step": float(np.mean(ts))}
            ps.close()
    # end to end through the public API with host buffers, on every rank at
    # once (a barrier before each call, the slowest rank's time)
    if not args.no_e2e:
        g = wl["geo"]
        e2e_t = []
        h2d = sum(np.asarray(v, dtype=np.float64).nbytes for v in g.values()) + seeds.nbytes
        for it in range(args.e2e_steps + 1):
            if dist:
                dist.barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            arr = core.simulate_ensemble(
                wl["E"], g["radius"], g["anisotropy"], g["anisotropy_axis"],
                g["magnetisation_direction"], g["location"], wl["ms"], wl["damping"],
                wl["temperature"], False, True, False, wl["dt"], wl["end_time"],
                wl["samples"], seeds, wl["field_shape"], wl["field_amplitude"],
                wl["field_frequency"], precision=args.precision)
            dt_ = time.perf_counter() - t0
            if dist:
                t = torch.tensor([dt_], device="cuda")
                dist.all_reduce(t, op=dist.ReduceOp.MAX)
                dt_ = float(t.item())
            if it > 0:
                e2e_t.append(dt_)
        d2h = arr.mx.nbytes * 3 + arr.status.nbytes + arr.steps.nbytes + \
            arr.time.nbytes + arr.field.nbytes
        es = float(np.median(e2e_t))
        if rank == 0:
            out["e2e"] = {"value": units_per_step * world / es, "unit": UNIT,
                          "h2d_bytes_per_step": int(h2d) * world,
                          "d2h_bytes_per_step": int(d2h) * world,
                          "ms_per_step": es * 1e3,
                          "path": "magpy_gb300.core.simulate_ensemble -> magpy_ensemble_dynamics "
                                  "(host numpy buffers)"}
    # the other configurations and the CPU baseline: one GPU, N = 1 only
    if rank == 0 and world == 1:
        if not args.no_side:
            out["config_single_particle"] = single_particle_config(torch, stream)
            out["config_batched_uneven"] = batched_uneven_config(torch, stream)
            out["config_adjoint"] = adjoint_config(torch, stream)
            out["config_dom"] = dom_config(torch, cpu=not args.no_cpu)
            out["config_implicit_n512"] = implicit_config(torch, stream, cpu=not args.no_cpu)
            out["config_geometry"] = geometry_config(torch)
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline(wl, args.cpu_seconds)
    plan.close()
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 (compensated state), f64 schedule", "data": "synthetic",
            "config": {
                "workload": "interacting cluster: N=64 in a sphere, log-normal radii "
                            "(median 8 nm, sigma 0.2), full dipolar, AC 10 kA/m 300 kHz, "
                            "T=300 K, alpha=0.1, dt=5e-14 s, E=4096 per GPU, Heun, "
                            f"{plan.K}-step window per benchmark step",
                "members_per_gpu": wl["E"], "particles": 64, "window_steps": plan.K,
                "samples": wl["samples"], "precision": args.precision,
                "l2": "flushed between timed steps (256 MiB write)",
                "parallelism": f"replicas x{world} (independent members, no collective)"},
            "clocks": clocks,
            "gpu_launches": args.steps,
            "wall_s": wall,
        }
        line.update(out)
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


def single_particle_config(torch, stream):
    """Single-particle ensemble, FP64-faithful Heun: N=1, E=1000, r=7 nm, K=2e4,
    Ms=4e5, alpha=0.1, T=300 K, easy axis and m0 along z, no field,
    dt=1e-13 s, 1e5 steps (the full run), 1001 samples."""
    from magpy_gb300 import core
    E, dt, steps = 1000, 1e-13, 100_000
    np.random.seed(99)
    seeds = np.random.randint(np.iinfo(np.int32).max, size=E)
    args = (E, [7e-9], [2e4], [[0, 0, 1.0]], [[0, 0, 1.0]], [[0, 0, 0.0]], 4e5, 0.1, 300.0,
            False, True, False, dt, dt * steps, 1001, seeds)
    names = ("n_members", "radius", "anisotropy", "anisotropy_axis",
                                 "magnetisation_direction", "location", "magnetisation",
                                 "damping", "temperature", "renorm", "interactions",
                                 "use_implicit", "time_step", "end_time", "max_samples", "seeds")
    batch = core.EnsembleBatch([dict(zip(names, args), precision="fp64")], autotune=True)
    plan = batch.groups[0]
    batch.run(stream.cuda_stream)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    batch.run(stream.cuda_stream)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b)
    mz = plan.ensemble_magnetisation("z") / 4e5
    choice = batch.choice(0)[:3]
    a64 = plan.arrays()
    batch.close()
    out = {"value": E * plan.max_steps / (ms * 1e-3), "unit": UNIT, "ms": ms,
           "precision": "fp64", "steps": plan.max_steps, "launch_choice": choice,
           "mz_mean_final": float(mz[-1]), "mz_mean_first_sample": float(mz[1]),
           "workload": "N=1, E=1000, r=7 nm, K=2e4, Ms=4e5, alpha=0.1, T=300 K, "
                       "dt=1e-13 s, 1e5 steps, FP64-faithful kernel"}
    # the same run in the mixed-precision form (FP32 evaluation, compensated
    # state) on the same in-kernel increments
    bm = core.EnsembleBatch([dict(zip(names, args), precision="mixed")], autotune=True)
    pm = bm.groups[0]
    bm.run(stream.cuda_stream)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    bm.run(stream.cuda_stream)
    b.record(stream)
    b.synchronize()
    msm = a.elapsed_time(b)
    am = pm.arrays()
    # strong error at every one of the 1001 samples: how it grows with the
    # horizon, and the horizon up to which every member is within 1e-5
    tm = np.stack([am.mx, am.my, am.mz], -1)      # [S][E][3]
    t64 = np.stack([a64.mx, a64.my, a64.mz], -1)
    err_t = np.linalg.norm(tm - t64, axis=-1) / np.linalg.norm(t64, axis=-1)  # [S][E]
    worst = err_t.max(axis=1)
    S = worst.size
    steps_at = np.round(np.arange(S) * pm.max_steps / (S - 1)).astype(np.int64)
    over = np.nonzero(worst > 1e-5)[0]
    horizon = int(steps_at[over[0] - 1]) if over.size else int(pm.max_steps)
    err = err_t[-1]
    marks = {str(k): {"max_rel": float(worst[i]), "frac_below_1e-5": float(np.mean(err_t[i] <= 1e-5))}
             for k in (1000, 10000, 30000, 100000)
             for i in [int(np.searchsorted(steps_at, k))] if i < S}
    matched = over.size == 0
    out["mixed"] = {"value": E * pm.max_steps / (msm * 1e-3), "unit": UNIT, "ms": msm,
                    "launch_choice": bm.choice(0)[:3],
                    "at_matched_error": bool(matched),
                    "strong_error_vs_fp64": {
                        "max_rel": float(err.max()), "median_rel": float(np.median(err)),
                        "frac_below_1e-5": float(np.mean(err <= 1e-5)), "steps": pm.max_steps,
                        "horizon_steps_all_members_within_1e-5": horizon,
                        "by_horizon": marks,
                        "note": "sigma = 6.9: trajectories that approach the barrier top amplify "
                                "the FP32 rounding of the step increments (a few 1e-10 per "
                                "step); a member whose two trajectories reach the top apart can "
                                "settle in different wells.  Beyond the stated horizon the mixed "
                                "number is not at matched error."}}
    bm.close()
    return out


def implicit_config(torch, stream, cpu=True):
    """Large cluster, implicit midpoint: N=512 in a sphere (as the headline
    cluster: log-normal radii, 2.2x spacing), alpha=0.01, E=512 members sharing
    the geometry, dt=2e-13 s, FP64 block-3x3 Newton (eps 1e-9, max_iter 1000),
    AC field 10 kA/m at 300 kHz.  The full run is 5000 steps; the FP64-faithful
    kernel is timed over a 20-step window, the mixed mode (FP64 Newton, FP32
    dipolar sum) over 100 steps, and the tensor-core mode (FP64 Newton, the
    dipolar field as a cluster GEMM) over 100 steps and over the full run,
    plans resident on the device."""
    from magpy_gb300 import core
    n, E, dt = 512, 512, 2e-13
    g = cluster_geometry(n, seed=512)
    np.random.seed(5)
    seeds = np.random.randint(np.iinfo(np.int32).max, size=E)

    def plan(precision, steps):
        return core.EnsemblePlan(E, g["radius"], g["anisotropy"], g["anisotropy_axis"],
                                 g["magnetisation_direction"], g["location"], 4e5, 0.01, 300.0,
                                 False, True, True, dt, dt * (steps - 0.5), 3, seeds, "sine",
                                 1e4, 3e5, 1e-9, precision=precision)

    def timed(p):
        p.run(stream.cuda_stream)  # warm-up
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        p.run(stream.cuda_stream)
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    out = {"workload": "N=512 sphere cluster, E=512, alpha=0.01, dt=2e-13 s, implicit midpoint "
                       "(FP64 block-3x3 Newton, eps 1e-9), AC 10 kA/m 300 kHz"}
    p64 = plan("fp64", 20)
    ms64 = timed(p64)
    out["fp64"] = {"value": E * n * p64.max_steps / (ms64 * 1e-3), "unit": UNIT,
                   "window_steps": p64.max_steps, "ms": ms64}
    a64 = p64.arrays()
    pm20 = plan("mixed", 20)
    pm20.run(stream.cuda_stream)
    torch.cuda.synchronize()
    am = pm20.arrays()
    m64 = np.stack([a64.mx[-1], a64.my[-1], a64.mz[-1]], 1)
    mm = np.stack([am.mx[-1], am.my[-1], am.mz[-1]], 1)
    err = np.linalg.norm(mm - m64, axis=1) / np.linalg.norm(m64, axis=1)
    out["strong_error_mixed_vs_fp64"] = {"max_rel": float(err.max()),
                                         "mean_rel": float(err.mean()), "window_steps": 20}
    out["status_nonzero"] = int(np.count_nonzero(a64.status) + np.count_nonzero(am.status))
    p64.close()
    pm20.close()
    pm = plan("mixed", 100)
    msm = timed(pm)
    out["mixed"] = {"value": E * n * pm.max_steps / (msm * 1e-3), "unit": UNIT,
                    "window_steps": pm.max_steps, "ms": msm}
    out["mixed_vs_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    out["full_run_seconds_mixed"] = msm * 1e-3 * 5000 / pm.max_steps
    pm.close()
    # the dipolar field on the tensor cores (a thread-block cluster of 13 CTAs
    # per 64 members, one GEMM per Newton iteration; FP64 state and residual):
    # strong error on the 20-step window, the rate on 100 steps, and the
    # whole 5000-step run executed once
    pt20 = plan("mixed_tc", 20)
    pt20.run(stream.cuda_stream)
    torch.cuda.synchronize()
    at = pt20.arrays()
    mt = np.stack([at.mx[-1], at.my[-1], at.mz[-1]], 1)
    errt = np.linalg.norm(mt - m64, axis=1) / np.linalg.norm(m64, axis=1)
    out["strong_error_mixed_tc_vs_fp64"] = {"max_rel": float(errt.max()),
                                            "mean_rel": float(errt.mean()), "window_steps": 20,
                                            "status_nonzero": int(np.count_nonzero(at.status))}
    pt20.close()
    pt = plan("mixed_tc", 100)
    mst = timed(pt)
    out["mixed_tc"] = {"value": E * n * pt.max_steps / (mst * 1e-3), "unit": UNIT,
                       "window_steps": pt.max_steps, "ms": mst}
    out["mixed_tc_vs_fp64"] = out["mixed_tc"]["value"] / out["fp64"]["value"]
    out["mixed_tc_vs_mixed"] = out["mixed_tc"]["value"] / out["mixed"]["value"]
    pt.close()
    pf = plan("mixed_tc", 5000)
    a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_.record(stream)
    pf.run(stream.cuda_stream)
    b_.record(stream)
    b_.synchronize()
    af = pf.arrays()
    full_ms = a_.elapsed_time(b_)
    out["full_run_mixed_tc"] = {"seconds": full_ms * 1e-3, "steps": pf.max_steps,
                                "status_nonzero": int(np.count_nonzero(af.status)),
                                "value": E * n * pf.max_steps / (full_ms * 1e-3), "unit": UNIT}
    pf.close()
    # the same path at the sizes where the reference's dense implicit solver
    # still runs (oracle/time_reference_implicit.py times it on one core)
    scaling = {}
    for ns in (27, 64, 125):
        gs = cluster_geometry(ns, seed=512)
        row = {}
        for prec in ("fp64", "mixed", "mixed_tc"):
            ps = core.EnsemblePlan(E, gs["radius"], gs["anisotropy"], gs["anisotropy_axis"],
                                   gs["magnetisation_direction"], gs["location"], 4e5, 0.01,
                                   300.0, False, True, True, dt, dt * 19.5, 3, seeds, "sine",
                                   1e4, 3e5, 1e-9, precision=prec)
            mss = timed(ps)
            row[prec] = E * ns * ps.max_steps / (mss * 1e-3)
            ps.close()
        scaling[str(ns)] = row
    out["scaling_fp64_mixed"] = {"unit": UNIT, "members": E, "window_steps": 20,
                                 "by_n": scaling}
    if cpu:
        # the restated reference (block 3x3 Newton; the reference's dense
        # (3N)^3 Jacobian path is far slower) on one member of the same cluster
        O = _oracle()
        t0 = time.perf_counter()
        r = O.full_dynamics(g["radius"], g["anisotropy"], g["anisotropy_axis"],
                            g["magnetisation_direction"], g["location"], 4e5, 0.01, 300.0,
                            use_implicit=True, time_step=dt, end_time=dt * 4.5, max_samples=2,
                            seed=int(seeds[0]), field_shape="sine", field_amplitude=1e4,
                            field_frequency=3e5)
        csec = time.perf_counter() - t0
        out["cpu_port_one_member"] = {"value": n * r["steps"] / csec, "unit": UNIT,
                                      "cores": 1, "sample": f"1 member x {r['steps']} steps",
                                      "kind": "port"}
    return out


def geometry_config(torch):
    """Seeded cluster geometries on the device: 4096 members x 64 particles,
    log-normal radii (8 nm, 0.2), random packing at 25 % of 2.2x exclusion
    spheres, axes uniform; device outputs, one launch.  (At 30 % about 1 % of
    the clusters jam before the last particle finds a place; they report it.)"""
    from magpy_gb300 import core
    seeds = np.arange(4096, dtype=np.int64) + 17
    core.generate_clusters(64, 64, seeds[:64], packing_fraction=0.25, device="cuda")  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    g = core.generate_clusters(4096, 64, seeds, packing_fraction=0.25, device="cuda")
    torch.cuda.synchronize()
    sec = time.perf_counter() - t0
    return {"value": 4096 / sec, "unit": "clusters/s", "seconds": sec,
            "clusters_jammed": int(torch.count_nonzero(g["status"]).item()),
            "jammed_note": "status 1: the cluster's random packing found no place for its last "
                           "particle within the attempt limit (reported per cluster, not an error "
                           "of the launch)",
            "workload": "4096 clusters of 64: log-normal radii, sphere packing 0.25, spacing 2.2"}


def dom_config(torch, cpu=True):
    """Two-state master equation (DOModel) for a polydisperse batch: 65536
    particles, log-normal radii (median 8 nm, sigma 0.2), K=2e4, Ms=4e5,
    alpha=0.1, T=300 K, all starting up, sine 10 kA/m at 300 kHz for 20 cycles,
    tolerance (time_step) 1e-10 s, 201 samples; one launch through the C-ABI
    with host buffers (allocation and copies inside the timed region).  The
    unit is accepted adaptive RK45 steps per second."""
    from magpy_gb300 import core
    rng = np.random.default_rng(77)
    E = 65536
    radius = np.exp(rng.normal(np.log(8e-9), 0.2, E))
    vol = 4 / 3 * np.pi * radius ** 3
    p0 = np.tile([1.0, 0.0], (E, 1))
    kw = dict(time_step=1e-10, end_time=20 / 3e5, max_samples=201, field_shape="sine",
              field_amplitude=1e4, field_frequency=3e5)
    core.simulate_dom_batch(p0[:256], vol[:256], 2e4, 300.0, 4e5, 0.1, **kw)  # warm-up
    t0 = time.perf_counter()
    g = core.simulate_dom_batch(p0, vol, 2e4, 300.0, 4e5, 0.1, **kw)
    sec = time.perf_counter() - t0
    steps = int(g["steps"].sum())
    out = {"value": steps / sec, "unit": "RK45 steps/s", "seconds": sec,
           "particles": E, "steps_total": steps, "status_nonzero": int(np.count_nonzero(
               g["status"])),
           "M_final_cycle_mean": float(g["mz"][:, -21:].mean()),
           "workload": "DOModel batch: 65536 particles, log-normal radii (8 nm, 0.2), sine "
                       "10 kA/m 300 kHz, 20 cycles, tol 1e-10 s, FP64, C-ABI with host buffers"}
    if cpu:
        O = _oracle()
        threads = os.cpu_count() or 1
        sel = rng.choice(E, 2048, replace=False)
        t0 = time.perf_counter()
        o = O.dom_batch(vol[sel], 2e4, 300.0, 4e5, 0.1, p0[sel], kw["field_shape"],
                        kw["field_amplitude"], kw["field_frequency"], 1, kw["time_step"],
                        kw["end_time"], kw["max_samples"], n_threads=threads)
        csec = time.perf_counter() - t0
        out["cpu_port"] = {"value": float(o["steps"].sum()) / csec, "unit": "RK45 steps/s",
                           "cores": threads, "sample": "2048 of the particles",
                           "kind": "port"}
        diff = np.abs(g["mz"][sel] - o["mz"]).max(axis=1)
        out["max_abs_mz_diff_vs_port"] = float(diff.max())
        out["frac_particles_within_1e-9"] = float(np.mean(diff <= 1e-9))
        out["diff_note"] = ("adaptive steps: an ulp-level difference of the device exp/sin "
                            "can flip one accept/reject decision, after which the particle's "
                            "steps fall elsewhere and the first-order-hold samples differ "
                            "by up to the interpolation error")
    return out


def batched_uneven_config(torch, stream):
    """8192 members over N in {1, 8, 27, 64, 125} (1639, 1639, 1638, 1638, 1638), cubic lattices of
    20 nm spacing, r=7 nm, parameters as the single-particle case, mixed
    precision, 1e4 Heun steps, one CUDA-graph launch, autotuned per size."""
    from magpy_gb300 import core
    rng = np.random.default_rng(31)
    groups = []
    for n, E in ((1, 1639), (8, 1639), (27, 1638), (64, 1638), (125, 1638)):
        side = int(np.ceil(n ** (1 / 3)))
        grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
        axes = rng.normal(size=(n, 3))
        axes /= np.linalg.norm(axes, axis=1, keepdims=True)
        groups.append(dict(n_members=E, radius=np.full(n, 7e-9), anisotropy=np.full(n, 2e4),
                           anisotropy_axis=axes, magnetisation_direction=axes,
                           location=grid * 20e-9, magnetisation=4e5, damping=0.1,
                           temperature=300.0, renorm=False, interactions=True,
                           use_implicit=False, time_step=1e-13, end_time=1e-13 * 10_000,
                           max_samples=11, seeds=rng.integers(0, 2**31 - 1, size=E),
                           precision="mixed"))
    batch = core.EnsembleBatch(groups, autotune=True)
    batch.run(stream.cuda_stream)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    batch.run(stream.cuda_stream)
    b.record(stream)
    b.synchronize()
    ms = a.elapsed_time(b)
    units = sum(g["n_members"] * g["radius"].size for g in groups) * batch.groups[0].max_steps
    choices = {str(g["radius"].size): batch.choice(i)[:3] for i, g in enumerate(groups)}
    tuned_ms = {str(g["radius"].size): round(batch.choice(i)[3] * batch.groups[i].max_steps, 3)
                for i, g in enumerate(groups)}
    batch.close()
    return {"value": units / (ms * 1e-3), "unit": UNIT, "ms": ms, "launches": 1,
            "choices": choices, "group_ms_alone": tuned_ms,
            "workload": "8192 members, N in {1,8,27,64,125} (1639/1639/1638/1638/1638), 1e4 Heun steps, mixed "
                        "precision, one CUDA-graph launch, autotuned kernel/CTA shape"}


def adjoint_config(torch, stream):
    """Pathwise adjoint: N=27 cubic lattice (20 nm, r=8 nm), E=2048, 2e4 Heun
    steps (dt=5e-14 s), checkpoints every 256 steps, sine field 10 kA/m at
    300 kHz; one grad = d{SAR, final <m_z>}/d{K, alpha, H0} (a forward run and
    two backward sweeps).  Checked against central differences of the
    FP64-faithful forward on the same increments: at h = 1e-4 relative (the
    specified check), at h = 1e-5, and extrapolated from h = 1e-4 and 5e-5
    (Richardson: the difference's h^2 error term cancels)."""
    from magpy_gb300.adjoint import EnsembleAdjoint, sar, sar_grad_M
    n, E, steps, dt = 27, 2048, 20_000, 5e-14
    grid = np.stack(np.meshgrid(*[np.arange(3)] * 3, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(4)
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    seeds = rng.integers(0, 2**31 - 1, size=E)
    base = dict(K=2e4, alpha=0.1, H0=1e4)

    def make(K, alpha, H0):
        return EnsembleAdjoint(E, np.full(n, 8e-9), np.full(n, K), axes, axes, grid * 20e-9,
                               4e5, alpha, 300.0, dt, dt * (steps - 0.5), 21, seeds, "sine",
                               H0, 3e5, True, checkpoint_every=256)

    def objectives(field, M):
        return np.array([sar(field, M), M[-1]])

    adj = make(**base)
    adj.forward()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    t, field, M = adj.forward()
    g_sar, _ = adj.backward(sar_grad_M(field))
    J = objectives(field, M)
    g_sar[2] += J[0] / base["H0"]
    dM = np.zeros_like(M)
    dM[-1] = 1.0
    g_mz, _ = adj.backward(dM)
    el = time.perf_counter() - t0
    adj.close()
    # central differences of the FP64-faithful kernel (bit-identical to the
    # reference's arithmetic) on the same in-kernel increments
    from magpy_gb300 import core

    def J_fp64(K, alpha, H0):
        a = core.simulate_ensemble(E, np.full(n, 8e-9), np.full(n, K), axes, axes, grid * 20e-9,
                                   4e5, alpha, 300.0, False, True, False, dt,
                                   dt * (steps - 0.5), 21, seeds, "sine", H0, 3e5,
                                   precision="fp64")
        Mz = a.mz.reshape(a.mz.shape[0], E, n).sum(axis=2).mean(axis=1)
        return objectives(a.field[0], Mz)

    def central(name, rel):
        th = dict(base)
        h = rel * base[name]
        J2 = []
        for sgn in (1, -1):
            th[name] = base[name] + sgn * h
            J2.append(J_fp64(**th))
        return (J2[0] - J2[1]) / (2 * h)

    def row(i, fd):
        return {"SAR": [g_sar[i], fd[0], abs(g_sar[i] - fd[0]) / abs(fd[0])],
                "mean_mz": [g_mz[i], fd[1], abs(g_mz[i] - fd[1]) / abs(fd[1])]}

    agree, agree_small, agree_rich = {}, {}, {}
    t_fd = time.perf_counter()
    for i, name in enumerate(("K", "alpha", "H0")):
        fd4 = central(name, 1e-4)
        agree[name] = row(i, fd4)
        agree_small[name] = row(i, central(name, 1e-5))
        agree_rich[name] = row(i, (4 * central(name, 5e-5) - fd4) / 3)
    t_fd = time.perf_counter() - t_fd
    return {"value": 1.0 / el, "unit": "grads/s", "s_per_grad": el,
            "objectives": {"SAR_J_per_m3": J[0], "final_Mz_A_per_m": J[1]},
            "adjoint_vs_fd": agree, "adjoint_vs_fd_h1e-5": agree_small,
            "adjoint_vs_fd_richardson": agree_rich, "fd_seconds": t_fd,
            "fd_note": "[adjoint, central difference (FP64-faithful kernel), relative "
                       "difference]; h = 1e-4 relative (the specified check), 1e-5, and the "
                       "extrapolation (4 fd(5e-5) - fd(1e-4)) / 3.  The difference at 1e-4 is "
                       "the central difference's own h^2 error (it falls 11x from h = 1e-4 to "
                       "3e-5 for K, whose gradient runs through the steep switching events)",
            "workload": "N=27 lattice (20 nm, r=8 nm), E=2048, 2e4 Heun steps, dt=5e-14 s, "
                        "checkpoints every 256 steps, sine 10 kA/m 300 kHz, mixed precision; "
                        "grad of (SAR, final <m_z>) w.r.t. (K, alpha, H0)"}


# ---------------------------------------------------------------------------
# CPU arms (oracle port of the reference path, OpenMP over members)
# ---------------------------------------------------------------------------
def _oracle():
    from oracle import pyoracle
    if not os.path.exists(pyoracle.ORACLE_SO):
        pyoracle.build()
    return pyoracle.Oracle()


def cpu_sample(O, wl, members, steps, threads):
    g = wl["geo"]
    t0 = time.perf_counter()
    O.ensemble(wl["seeds"][:members], g["radius"], g["anisotropy"], g["anisotropy_axis"],
               g["magnetisation_direction"], g["location"], wl["ms"], wl["damping"],
               wl["temperature"], interactions=True, use_implicit=False,
               time_step=wl["dt"], end_time=wl["dt"] * steps, max_samples=2,
               field_shape=wl["field_shape"], field_amplitude=wl["field_amplitude"],
               field_frequency=wl["field_frequency"], n_threads=threads)
    el = time.perf_counter() - t0
    return members * wl["n"] * (steps + 1) / el, el


def cpu_baseline(wl, seconds):
    O = _oracle()
    threads = O.lib.oracle_max_threads()
    members = max(threads, 1) * 2
    rate, el = cpu_sample(O, wl, members, 50, threads)  # calibration
    steps = int(max(50, min(1_000_000, seconds * rate / (members * wl["n"]))))
    rate, el = cpu_sample(O, wl, members, steps, threads)
    return {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{members} members x {steps} Heun steps of the same workload, "
                      f"{el:.1f} s, oracle/sllg_oracle.cpp (FP64, OpenMP over members)"}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    wl = workload(args.members, 64, args.window, args.samples)
    O = _oracle()
    threads = O.lib.oracle_max_threads()
    members = max(threads, 1) * 2
    rate, _ = cpu_sample(O, wl, members, 20, threads)
    steps = int(max(20, min(1_000_000, args.ref_step_seconds * rate / (members * wl["n"]))))
    for _ in range(args.warmup):
        cpu_sample(O, wl, members, max(20, steps // 10), threads)
    rates, els = [], []
    for _ in range(args.steps):
        r, el = cpu_sample(O, wl, members, steps, threads)
        rates.append(r)
        els.append(el)
    value = float(np.median(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": float(np.median(els)) * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": "interacting cluster: N=64 in a sphere, log-normal radii "
                               "(median 8 nm, sigma 0.2), full dipolar, AC 10 kA/m 300 kHz, "
                               "T=300 K, alpha=0.1, dt=5e-14 s, Heun (the GPU arm's workload); "
                               "a bounded sample of its members and steps per benchmark step",
                   "members": members, "window_steps": steps, "particles": 64,
                   "precision": "fp64 (the reference's arithmetic)"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{members} members x {steps} Heun steps per benchmark step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--members", type=int, default=4096)
    ap.add_argument("--window", type=int, default=2000)
    ap.add_argument("--samples", type=int, default=11)
    ap.add_argument("--plain-repeats", type=int, default=3)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-step-seconds", type=float, default=3.0)
    ap.add_argument("--precision", default="mixed_tc", choices=["mixed_tc", "mixed", "fp64"])
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-side", action="store_true", help="skip the side workloads")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
