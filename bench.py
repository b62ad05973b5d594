"""Benchmark: Gcell-updates/s of the GB300 stepper on the benchmark workloads.

    python bench.py [--gpus N] [--steps K] [--warmup W]       # visco2d + every other workload as a sub-record
    python bench.py --workload visco2d|elastic2d|visco3d|fmc2d|adjoint2d ...   # one workload alone
    python bench.py --impl reference ...     # the CPU implementation of the same path

One bench "step" is one complete simulation of the workload (all its time
steps, e.g. 4000 steps of the 1024x1024 viscoelastic grid) from a zero state,
with every input resident in HBM.  K steps are timed with CUDA events on the
stream the kernels run on, bracketed by a barrier and synchronisations; L2 is
flushed (a 256 MiB write) after every simulation, inside the timed region.
Under torchrun each rank runs its own replica (the path shards over shots;
a single-shot workload has no exchange), and the time is the max over ranks.

The default line is the 2D viscoelastic workload (1024^2, L = 3, per-cell Q,
4000 steps); under "workloads" it carries one record per other benchmark
target, each timed the same way with its own step count: elastic2d (512^2,
Taichi semantics, 2000 steps), visco3d (256^3, 1000 steps), fmc2d (64 shots
x 3 phantoms, 3000 steps, with the per-shot loop it replaces) and adjoint2d
(16-shot gradient on 512x1024, 3000 steps, with t_grad / t_forward).

Each record adds:
  roofline      - HBM roofline of the dominant kernel, algorithmic bytes per
                  launch / mean launch time (CUDA events around single
                  launches), against the measured HBM peak, with the ncu DRAM
                  traffic per launch from profiles/traffic_<workload>.json;
  step_roofline - the whole time step at the benchmark's bytes per cell-update;
  e2e           - the same metric through the public C-ABI call sequence with
                  host buffers (creation with uploads, run, readback, destroy);
  clocks        - SM clocks and throttle reasons sampled during the timing;
and the headline a cpu_baseline: the CPU restatement of the reference
kernels (all host cores) on a bounded sample of the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from taichi_sim_gb300 import workloads  # noqa: E402

# Per-cell bytes each kernel must move at least once per step (float32),
# counting each array of its data layout once: stress: v read (2D 8, 3D 12),
# stresses r/w, memory variables r/w, and the coefficients as stored: a
# 2-byte palette index (2D order-2 WGSL stepper, 3D) or lambda, mu, mu_s
# (Taichi 2D); velocity: stresses read, v r/w, rho (2D, 4 B per node and
# component) or dt / rho as a (hi, lo) pair (3D, 8 B).  CPML strip memories
# are added per strip cell.
KERNEL_BYTES = {
    "visco2d": {"stress": 8 + 24 + 72 + 2, "velocity": 12 + 16 + 8, "psi_stress": 8 * 2, "psi_vel": 8 * 2},
    "elastic2d": {"stress": 8 + 24 + 12, "velocity": 12 + 16 + 8, "psi_stress": 8 * 2, "psi_vel": 8 * 2},
    "visco3d": {"stress": 12 + 48 + 144 + 2, "velocity": 24 + 24 + 16, "psi_stress": 8 * 3, "psi_vel": 8 * 3},
}
FAMILY = {"elastic2d": "TAICHI2D", "visco2d": "WGSL2D", "visco3d": "WGSL3D"}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def build_model(name, time_steps=None, grid=None):
    from taichi_sim_gb300.sim_support.simulator import Simulator
    from taichi_sim_gb300.sim_support.Simulator3D import Simulator3D
    kw = {}
    if time_steps is not None:
        kw["n_steps"] = time_steps
    if grid is not None:
        kw["n_grid"] = grid
    cfg = workloads.WORKLOADS[name](**kw)
    return (Simulator3D if name == "visco3d" else Simulator)(cfg)


def strip_fraction(sim):
    """Fraction of cells inside the CPML strips, per axis (a cell-weighted mean)."""
    frac = []
    for ax, n in zip("xyz", sim.grid_shape()):
        a = getattr(sim, f"_a_{ax}").flatten()
        b = getattr(sim, f"_b_{ax}").flatten()
        nonid = (a != 0) | (b != 1)
        frac.append(float(nonid.sum() + 2 * (sim._coefs.shape[0] - 1)) / n if nonid.any() else 0.0)
    return frac


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons while timing."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.out = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        self.out.flush()
        self.out.seek(0)
        rows = [l.strip().split(", ") for l in self.out.read().splitlines() if l.strip()]
        os.unlink(self.out.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        smax = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, name in enumerate(names):
                if len(r) > 4 + k and r[4 + k].strip().lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def cpu_baseline(sim, name, target_s=12.0):
    """The CPU restatement of the reference kernels, all host cores, on a
    bounded number of time steps of the same grid."""
    from oracle import oracle
    fam = {"elastic2d": oracle.TAICHI2D, "visco2d": oracle.WGSL2D, "visco3d": oracle.WGSL3D}[name]
    cores = len(os.sched_getaffinity(0))
    os.environ.setdefault("OMP_NUM_THREADS", str(cores))
    cells = int(np.prod(sim.grid_shape()))
    t = time.time()
    oracle.run(sim, fam, n_steps=4)
    probe = max(time.time() - t, 1e-3) / 4
    n = int(max(8, min(sim._n_steps, target_s / probe)))
    t = time.time()
    oracle.run(sim, fam, n_steps=n)
    dt = time.time() - t
    return {"value": cells * n / dt / 1e9, "unit": "Gcell/s", "cores": cores, "kind": "port",
            "sample": f"{n} of {sim._n_steps} time steps of the full {'x'.join(map(str, sim.grid_shape()))} grid "
                      f"(C restatement of the reference kernels, OpenMP, {dt:.1f} s)"}


def traffic(name, kernel):
    """ncu DRAM bytes (read + write) per launch of a workload's kernel, from
    the committed profile summary profiles/traffic_<name>.json, or None."""
    path = os.path.join(ROOT, "profiles", f"traffic_{name}.json")
    try:
        with open(path) as f:
            return json.load(f).get(kernel)
    except (OSError, ValueError):
        return None


def workload_config(name, sim):
    """The ``config`` of a workload's line (shared with the reference arm)."""
    return {"workload": name, "grid": list(sim.grid_shape()), "time_steps_per_step": int(sim._n_steps),
            "family": FAMILY[name], "receivers": int(sim._n_rec),
            "zener": "L=3 fitted 2-8 MHz, per-cell Q" if name != "elastic2d" else None,
            "arithmetic": ("every operation rounded on its own (TS_TAICHI_EXACT=1)"
                           if os.environ.get("TS_TAICHI_EXACT") == "1" else "the reference's constants, no rounding bias")
            if name == "elastic2d" else "unbiased (raw coefficients, 1/d as a pair, divisions by rho)",
            "l2": "256 MiB flush written after every simulation (inside the timed region)"}


def run_reference(args):
    """--impl reference: the reference's CPU path (the oracle port: the
    reference's own kernels need Taichi/wgpu, absent here) on the same metric."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    name = args.workload or "visco2d"
    if name == "adjoint2d":
        print(json.dumps({"impl": "reference", "unavailable": "the reference computes no gradients"}))
        return
    per_shot = name == "fmc2d"
    if per_shot:
        name = "visco2d"   # the reference runs one shot at a time: its per-shot path
    sim = build_model(name, args.time_steps)
    from oracle import oracle
    fam = {"elastic2d": oracle.TAICHI2D, "visco2d": oracle.WGSL2D, "visco3d": oracle.WGSL3D}[name]
    cores = len(os.sched_getaffinity(0))
    cells = int(np.prod(sim.grid_shape()))
    sample = args.ref_sample_steps
    for _ in range(args.warmup):
        oracle.run(sim, fam, n_steps=max(2, sample // 10))
    t = time.time()
    for _ in range(args.steps):
        oracle.run(sim, fam, n_steps=sample)
    dt = time.time() - t
    value = cells * sample * args.steps / dt / 1e9
    cfg = workload_config(name, sim)
    cfg["arithmetic"] = "strict IEEE float, the reference's operation order (CPU restatement)"
    cfg["parallelism"] = "single GPU"
    desc = (f"{sample} of the {sim._n_steps} time steps of the full {'x'.join(map(str, sim.grid_shape()))} grid "
            f"per bench step (C restatement of the reference kernels, OpenMP, {cores} threads)")
    line = {"impl": "reference", "metric": "Gcell-updates/s", "value": value, "unit": "Gcell/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded numpy default_rng(0); no public dataset exists)",
            "config": cfg,
            "cpu_baseline": {"value": value, "unit": "Gcell/s", "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": value, "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    if per_shot:
        line["note"] = "fmc2d: the reference runs one shot at a time; its per-shot rate on the 1024x1024 model"
    print(json.dumps(line))


def stepper_record(name, args, steps, warmup, world=1, rank=0, local=0, dist=None, with_cpu=False):
    """One workload on the single-simulation stepper: K complete simulations
    timed with CUDA events, the dominant kernel's roofline, the whole-step
    roofline at the benchmark's bytes per cell-update, and the same metric
    end to end through the C ABI with host buffers."""
    import torch
    from taichi_sim_gb300 import engine, shards

    sim = build_model(name, args.time_steps, args.grid)
    n_t = int(sim._n_steps)
    cells = int(np.prod(sim.grid_shape()))
    fam = getattr(engine, FAMILY[name])
    st = engine.Stepper(sim, family=fam)
    path = st.path
    stream = torch.cuda.Stream()
    h = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def one_simulation():
        st.reset(stream=h, wait=False)
        st.run(n_t, stream=h)
        with torch.cuda.stream(stream):
            flush.zero_()

    for _ in range(warmup):
        one_simulation()
    torch.cuda.synchronize()
    _, _, bad = st.status()
    if bad >= 0:
        raise RuntimeError(f"{name}: workload unstable at step {bad}")
    launches0 = st.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        start.record(stream)
        for _ in range(steps):
            one_simulation()
        end.record(stream)
        torch.cuda.synchronize()
    launches = st.launch_count() - launches0
    ms = start.elapsed_time(end)
    ms = shards.max_over_ranks(ms, device="cuda")   # the job's time: its slowest replica
    value = cells * n_t * steps * world / (ms / 1e3) / 1e9

    # ---- roofline of the dominant kernel (single launches between events) ----
    st.reset()
    n_prof = min(args.profile_steps, n_t)
    k_ms = st.profile_steps(n_prof, stream=h)
    kb = KERNEL_BYTES[name]
    frac = strip_fraction(sim)
    strip_share = sum(frac) / len(frac)
    bytes_stress = cells * (kb["stress"] + kb["psi_stress"] * 2 * strip_share)
    bytes_vel = cells * (kb["velocity"] + kb["psi_vel"] * 2 * strip_share)
    peak, peak_kind = peaks()
    if st.path == "persistent":
        # one cooperative launch runs every step with the wavefield in shared
        # memory: its algorithmic bytes are both updates' per step, while its
        # DRAM traffic is the slab load and store of the launch
        step_bytes = bytes_stress + bytes_vel
        achieved = step_bytes / (k_ms[0] / 1e3) / 1e9
        roofline = {"kernel": "persistent step (stress + velocity, wavefield in shared memory)", "bound": "hbm",
                    "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                    "traffic": traffic(name, "persistent"), "peak_kind": peak_kind,
                    "bytes_per_launch": int(step_bytes * n_t), "steps_per_launch": n_t,
                    "kernel_ms_per_step": {"persistent": round(k_ms[0], 6), "receiver_sums": round(k_ms[1], 6)},
                    "note": "state held on chip across steps: achieved counts the algorithmic bytes the "
                            "two-kernel step would move; traffic is the DRAM bytes of one launch"}
    else:
        dom = 0 if k_ms[0] >= k_ms[1] else 1
        dom_bytes = [bytes_stress, bytes_vel][dom]
        achieved = dom_bytes / (k_ms[dom] / 1e3) / 1e9
        kname = ["stress", "velocity"][dom]
        roofline = {"kernel": kname, "bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "traffic": traffic(name, kname), "peak_kind": peak_kind,
                    "bytes_per_launch": int(dom_bytes),
                    "kernel_ms": {"stress": round(k_ms[0], 5), "velocity": round(k_ms[1], 5)}}
    b_alg = workloads.B_ALG[name]
    step_roofline = {"b_alg_per_cell_update": b_alg, "achieved": round(value / world * b_alg, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(value / world * b_alg / peak, 4), "peak_kind": peak_kind,
                     "note": "whole time step (all kernels) at the benchmark's algorithmic bytes per cell-update"}
    st.close()

    # ---- end to end through the C ABI with host buffers ----
    e2e_times, h2d, d2h = [], 0, 0
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t0 = time.time()
        with engine.Stepper(sim, family=fam) as s2:
            s2.run(n_t)
            tr = s2.read("traces")
            fld = s2.read("szz" if sim._dims == 3 else "syy")
            h2d, d2h = s2.transfer_bytes()
        torch.cuda.synchronize()
        e2e_times.append(time.time() - t0)
    e2e_s = float(np.mean(e2e_times))
    e2e = {"value": cells * n_t * world / e2e_s / 1e9, "unit": "Gcell/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h), "seconds_per_step": round(e2e_s, 4),
           "path": "ts_create + ts_run + ts_read(traces, field) + ts_destroy"}
    cpu = cpu_baseline(sim, name) if with_cpu and rank == 0 and world == 1 and not args.no_cpu_baseline else None
    cfg = workload_config(name, sim)
    cfg["parallelism"] = f"replicas x{world}" if world > 1 else "single GPU"
    cfg["step_path"] = path
    return {"metric": "Gcell-updates/s", "value": round(value, 3), "unit": "Gcell/s", "n_gpus": world,
            "steps": steps, "warmup": warmup, "ms_per_step": round(ms / steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy default_rng(0); no public dataset exists)", "config": cfg,
            "roofline": roofline, "step_roofline": step_roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": int(launches), "clocks": clk.summary()}


def fmc_record(args, steps, warmup):
    """Batched full-matrix capture: 64 shots x 3 phantoms (512x768, 768x768,
    1024x768) in one launch per kernel per step, against the per-shot loop
    (the regular stepper run once per shot, as the reference's shot loop does)."""
    import torch
    from taichi_sim_gb300 import engine
    from taichi_sim_gb300.batch import BatchStepper, autotune, fmc_shot_sources
    from taichi_sim_gb300.sim_support.simulator import Simulator

    n_t = args.time_steps or 3000
    sims = [Simulator(c) for c in workloads.fmc2d_phantoms(n_steps=n_t)]
    shots = [fmc_shot_sources(s) for s in sims]
    cell_shots = sum(int(np.prod(s.grid_shape())) * sh.shape[0] for s, sh in zip(sims, shots))
    shape, tune = autotune(sims, shots, steps=8)
    b = BatchStepper(sims, shots, **shape)
    stream = torch.cuda.Stream()
    h = stream.cuda_stream
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def one():
        b.reset(stream=h)
        b.run(n_t, stream=h)
        with torch.cuda.stream(stream):
            flush.zero_()

    for _ in range(warmup):
        one()
    torch.cuda.synchronize()
    if b.status()[2] >= 0:
        raise RuntimeError("fmc2d: unstable")
    launches0 = b.launch_count()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        start.record(stream)
        for _ in range(steps):
            one()
        end.record(stream)
        torch.cuda.synchronize()
    ms = start.elapsed_time(end)
    launches = b.launch_count() - launches0
    value = cell_shots * n_t * steps / (ms / 1e3) / 1e9
    b.reset()
    k_ms = b.profile_steps(min(50, n_t))
    b.close()

    # end to end: a batch created from the host models (uploads), run, every trace read back
    torch.cuda.synchronize()
    t0 = time.time()
    with BatchStepper(sims, shots, **shape) as be:
        be.run(n_t)
        for q in range(len(sims)):
            be.traces(q)
        h2d, d2h = be.transfer_bytes()
    torch.cuda.synchronize()
    e2e_s = time.time() - t0

    # per-shot loop on a sample of shots of every phantom
    per_shot_s, sample = 0.0, 0
    for sim, sh in zip(sims, shots):
        saved = sim._source_term, sim._n_src
        sim._source_term, sim._n_src = sh[0], sh.shape[2]
        try:
            st = engine.Stepper(sim, family=engine.WGSL2D)
        finally:
            sim._source_term, sim._n_src = saved
        st.set_sources(sh[0])
        st.reset()
        st.run(n_t)
        st.status()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in range(args.loop_shots):
            st.set_sources(sh[s])
            st.reset()
            st.run(n_t)
            st.read("traces")
        torch.cuda.synchronize()
        per_shot_s += (time.perf_counter() - t0) / args.loop_shots * sh.shape[0]
        sample += args.loop_shots
        st.close()
    loop_value = cell_shots * n_t / per_shot_s / 1e9
    peak, peak_kind = peaks()
    b_alg = 115.6
    # stress launch: v 8, stresses 24 r/w, memory variables 72 r/w per cell-shot
    # (coefficients shared by the shots); velocity launch: stresses 12, v 16
    kb = {"stress": 8 + 24 + 72, "velocity": 12 + 16}
    dom = 0 if k_ms[0] >= k_ms[1] else 1
    kname = ["stress", "velocity"][dom]
    dom_bytes = cell_shots * kb[kname]
    achieved = dom_bytes / (k_ms[dom] / 1e3) / 1e9
    return {"metric": "Gcell-updates/s", "value": round(value, 3), "unit": "Gcell/s", "n_gpus": 1,
            "steps": steps, "warmup": warmup, "ms_per_step": round(ms / steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy default_rng)",
            "config": {"workload": "fmc2d", "phantoms": [list(s.grid_shape()) for s in sims],
                       "shots_per_phantom": [int(sh.shape[0]) for sh in shots], "time_steps_per_step": n_t,
                       "launch_shape": shape, "autotune_ms": tune,
                       "l2": "256 MiB flush written after every batch (inside the timed region)"},
            "roofline": {"kernel": f"batched {kname}", "bound": "hbm", "achieved": round(achieved, 1), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic("fmc2d", kname),
                         "peak_kind": peak_kind, "bytes_per_launch": int(dom_bytes),
                         "kernel_ms": {"stress": round(k_ms[0], 4), "velocity": round(k_ms[1], 4)}},
            "per_shot_loop": {"value": round(loop_value, 3), "unit": "Gcell/s",
                              "sample": f"{args.loop_shots} shots per phantom ({sample} total), extrapolated",
                              "path": "Stepper per phantom; per shot ts_set_sources + ts_reset + ts_run + ts_read"},
            "speedup_vs_per_shot_loop": round(value / loop_value, 3),
            "step_roofline": {"b_alg_per_cell_update": b_alg, "achieved": round(value * b_alg, 1), "peak": peak,
                              "unit": "GB/s", "frac": round(value * b_alg / peak, 4), "peak_kind": peak_kind},
            "e2e": {"value": round(cell_shots * n_t / e2e_s / 1e9, 3), "unit": "Gcell/s",
                    "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "seconds_per_step": round(e2e_s, 4),
                    "path": "ts_batch_create + ts_batch_run + ts_batch_read_traces (every phantom) + ts_batch_destroy"},
            "gpu_launches": int(launches), "clocks": clk.summary()}


ADJ_BYTES = {
    # adjoint step per cell (float32, L = 3 global relaxation times):
    # velocity kernel: vbar r/w 16, stress-node adjoints gathered 16, Bx By 8,
    # record 8, gBx gBy r/w 16, velocity-node adjoints written 16;
    # stress kernel: velocity-node adjoints 16, sbar r/w 24, L M Ms 12,
    # record 16, gL gM gMs r/w 24, Zener adjoints r/w 72, stress-node adjoints 16
    "adjoint_step": 80 + 180,
    # forward step of the same model (its algorithmic bytes) and the record it writes when recomputing
    "forward_step": 127.75, "record": 24,
}


def adjoint_record(args, steps, warmup, with_cpu=False):
    """Adjoint gradient: 16 shots of a 512 x 1024 viscoelastic model (3000
    steps, 256 receivers), gradient of the L2 trace misfit w.r.t. per-cell
    lambda, mu, rho summed over shots, checkpointing every ceil(sqrt(3000))
    = 55 steps; one bench step = the whole 16-shot gradient.  Reported next
    to one plain forward per shot (the regular stepper) as t_grad / t_forward."""
    import torch
    from taichi_sim_gb300 import engine
    from taichi_sim_gb300.adjoint import AdjointProblem, l2_misfit
    from taichi_sim_gb300.batch import fmc_shot_sources
    from taichi_sim_gb300.sim_support.simulator import Simulator

    n_t = args.time_steps or 3000
    true = Simulator(workloads.adjoint2d_512x1024(n_steps=n_t))
    start = Simulator(workloads.adjoint2d_512x1024(n_steps=n_t, true_model=False))
    shots = fmc_shot_sources(start)
    n_shots = shots.shape[0]
    cells = int(np.prod(start.grid_shape()))
    stream = torch.cuda.Stream()
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    # observed data: the true model through the same forward (untimed)
    with torch.cuda.stream(stream), AdjointProblem(true, checkpoint_every=64) as pt, torch.no_grad():
        obs = []
        for s in range(n_shots):
            pt.set_source_term(shots[s])
            obs.append(pt.traces(*pt.material()).clone())

    # t_forward: the plain stepper, one simulation per shot
    with engine.Stepper(start, family=engine.WGSL2D) as st:
        h = stream.cuda_stream

        def forward_all():
            for s in range(n_shots):
                st.set_sources(shots[s])
                st.reset(stream=h, wait=False)
                st.run(n_t, stream=h)
                with torch.cuda.stream(stream):
                    flush.zero_()

        forward_all()
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record(stream)
        forward_all()
        b.record(stream)
        torch.cuda.synchronize()
        t_fwd_ms = a.elapsed_time(b) / n_shots

    def gradient(prob, m):
        for t in m:
            t.grad = None
        for s in range(n_shots):
            prob.set_source_term(shots[s])
            l2_misfit(prob.traces(*m), obs[s]).backward()
            with torch.cuda.stream(stream):
                flush.zero_()

    ckpt = int(np.ceil(np.sqrt(n_t)))
    n_seg = -(-n_t // ckpt)
    # trailing segments whose per-step record (6 floats per node) the forward
    # pass keeps within the record budget; the others are recomputed
    seg_bytes = start.grid_shape()[0] * 4 * (-(-start.grid_shape()[1] // 32) * 32) * 6 * ckpt
    segs = int(min(n_seg, max(1, args.adjoint_record_gb * 1e9 // seg_bytes)))
    with torch.cuda.stream(stream), AdjointProblem(start, checkpoint_every=ckpt, record_segments=segs) as prob:
        m = [t.clone().requires_grad_(True) for t in prob.material()]
        for _ in range(warmup):
            gradient(prob, m)
        torch.cuda.synchronize()
        l0 = prob.launch_count()
        start_ev, end_ev = ev(), ev()
        with ClockSampler(0) as clk:
            start_ev.record(stream)
            for _ in range(steps):
                gradient(prob, m)
            end_ev.record(stream)
            torch.cuda.synchronize()
        ms = start_ev.elapsed_time(end_ev)
        launches = prob.launch_count() - l0
        grad_ref = [t.grad.detach().clone() for t in m]

        # end to end: material and observed traces from host memory, gradient back to host
        host_m = [t.detach().cpu().pin_memory() for t in m]
        host_obs = [o.cpu().pin_memory() for o in obs]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        md = [t.to("cuda", non_blocking=True).requires_grad_(True) for t in host_m]
        for s in range(n_shots):
            prob.set_source_term(shots[s])
            l2_misfit(prob.traces(*md), host_obs[s].to("cuda", non_blocking=True)).backward()
        g_host = [t.grad.cpu() for t in md]
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        h2d = sum(t.numel() * 4 for t in host_m) + sum(o.numel() * 4 for o in host_obs)
        d2h = sum(t.numel() * 4 for t in g_host)

    # the same gradient recomputing every segment but the last
    with torch.cuda.stream(stream), AdjointProblem(start, checkpoint_every=ckpt, record_segments=1) as prob1:
        m1 = [t.detach().clone().requires_grad_(True) for t in m]
        gradient(prob1, m1)
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record(stream)
        gradient(prob1, m1)
        b.record(stream)
        torch.cuda.synchronize()
        ms_one = a.elapsed_time(b)
        agree1 = max(float((x.grad - y).norm() / y.norm()) for x, y in zip(m1, grad_ref))

    # the same gradient with the whole record kept in HBM (no recomputation)
    with torch.cuda.stream(stream), AdjointProblem(start, checkpoint_every=0) as prob0:
        m0 = [t.detach().clone().requires_grad_(True) for t in m]
        gradient(prob0, m0)
        torch.cuda.synchronize()
        a, b = ev(), ev()
        a.record(stream)
        gradient(prob0, m0)
        b.record(stream)
        torch.cuda.synchronize()
        ms_keep = a.elapsed_time(b)
        agree = max(float((x.grad - y).norm() / y.norm()) for x, y in zip(m0, grad_ref))
        # one adjoint sweep alone (the record kept): backward of one shot
        prob0.set_source_term(shots[0])
        tr = prob0.traces(*m0)
        loss = l2_misfit(tr, obs[0])
        torch.cuda.synchronize()
        a.record(stream)
        loss.backward()
        b.record(stream)
        torch.cuda.synchronize()
        sweep_ms = a.elapsed_time(b)

    t_grad_ms = ms / steps / n_shots
    ratio = t_grad_ms / t_fwd_ms
    value = cells * n_t * n_shots * steps / (ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    adj_bytes = cells * ADJ_BYTES["adjoint_step"]
    achieved = adj_bytes / (sweep_ms / n_t / 1e3) / 1e9
    cpu = None if (args.no_cpu_baseline or not with_cpu) else cpu_baseline(start, "visco2d")
    if cpu:
        cpu["sample"] += "; the reference computes no gradient: this is its forward on the same grid"
    line = {"metric": "Gcell-updates/s", "value": round(value, 3), "unit": "Gcell/s", "n_gpus": 1,
            "steps": steps, "warmup": warmup, "ms_per_step": round(ms / steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded numpy default_rng(0); no public dataset exists)",
            "config": {"workload": "adjoint2d", "grid": list(start.grid_shape()), "time_steps": n_t,
                       "shots_per_step": n_shots, "receivers": int(start._n_rec), "checkpoint_every": ckpt,
                       "segments": n_seg, "segments_recorded_by_forward": segs,
                       "record_gb": round(segs * seg_bytes / 1e9, 2),
                       "zener": "L=3, fixed relaxation times",
                       "value_is": "forward cell-updates of the 16 shots per second of gradient time",
                       "l2": "256 MiB flush written after every shot (inside the timed region)"},
            "adjoint": {"t_grad_over_t_forward": round(ratio, 3), "t_forward_ms_per_shot": round(t_fwd_ms, 3),
                        "t_grad_ms_per_shot": round(t_grad_ms, 3),
                        "schedule": f"checkpoint every {ckpt} steps; the forward pass records the last {segs} "
                                    f"of {n_seg} segments ({segs * seg_bytes / 1e9:.1f} GB), the backward "
                                    f"pass recomputes the other {n_seg - segs}",
                        "one_segment_recorded": {"t_grad_over_t_forward": round(ms_one / n_shots / t_fwd_ms, 3),
                                                 "recomputed_segments": n_seg - 1,
                                                 "gradient_rel_diff": agree1},
                        "record_kept": {"t_grad_over_t_forward": round(ms_keep / n_shots / t_fwd_ms, 3),
                                        "record_gb": round(cells * n_t * 24 / 1e9, 1),
                                        "gradient_rel_diff_vs_checkpointed": agree},
                        "adjoint_step_ms": round(sweep_ms / n_t, 5)},
            "roofline": {"kernel": "adjoint step (k_adj_velocity + k_adj_stress)", "bound": "hbm",
                         "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic("adjoint2d", "adjoint_step"), "peak_kind": peak_kind,
                         "bytes_per_launch_pair": int(adj_bytes)},
            "cpu_baseline": cpu,
            "e2e": {"value": cells * n_t * n_shots / e2e_s / 1e9, "unit": "Gcell/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "seconds_per_step": round(e2e_s, 4),
                    "path": "material + observed traces from pinned host memory, 16 x (traces, misfit, "
                            "backward), gradient to host"},
            "gpu_launches": int(launches), "clocks": clk.summary()}
    return line


# Sub-records of the default line: (bench steps, warm-up steps) of each
# workload, sized so that the whole default run takes a few minutes.
SUB_RECORDS = {"elastic2d": (20, 3), "visco3d": (5, 3), "fmc2d": (2, 3), "adjoint2d": (1, 3)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default=None, choices=sorted(workloads.WORKLOADS) + ["fmc2d", "adjoint2d"],
                    help="one workload alone (default: visco2d, with every other workload as a sub-record)")
    ap.add_argument("--no-sub", action="store_true", help="default run without the sub-records")
    ap.add_argument("--loop-shots", type=int, default=4, help="fmc2d: shots per phantom timed in the per-shot loop")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-sample-steps", type=int, default=200)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--adjoint-record-gb", type=float, default=8.0,
                    help="adjoint2d: HBM for the records of the trailing segments the forward pass keeps")
    ap.add_argument("--profile-steps", type=int, default=200)
    ap.add_argument("--time-steps", type=int, default=None,
                    help="override the workload's time steps (small runs for profiler captures)")
    ap.add_argument("--grid", type=int, default=None,
                    help="elastic2d/visco2d/visco3d: nodes per side instead of the workload's (profiler captures)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "gb300":
        print("bench: at least 3 warm-up steps are required; using 3", file=sys.stderr)
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if args.workload == "fmc2d":
        print(json.dumps(fmc_record(args, args.steps, args.warmup)))
        return
    if args.workload == "adjoint2d":
        print(json.dumps(adjoint_record(args, args.steps, args.warmup, with_cpu=True)))
        return
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    name = args.workload or "visco2d"
    line = stepper_record(name, args, args.steps, args.warmup, world, rank, local, dist, with_cpu=True)
    if args.workload is None and world == 1 and not args.no_sub:
        # every other benchmark target, measured in the same run with its own
        # CUDA-event timing, rooflines, clocks and end-to-end figure
        subs = {}
        for sub, (k, w) in SUB_RECORDS.items():
            if sub == "fmc2d":
                subs[sub] = fmc_record(args, k, w)
            elif sub == "adjoint2d":
                subs[sub] = adjoint_record(args, k, w)
            else:
                subs[sub] = stepper_record(sub, args, k, w)
            torch.cuda.empty_cache()
        line["workloads"] = subs
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
