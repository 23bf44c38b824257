"""Benchmark of the SPH step: particle-steps/s on one GB300.

Workload (default): the 1,048,576-particle dam break with a held sphere
(128x64x128 lattice, spacing 0.02, seeded jitter, box 4x2x3, h 0.08,
rest density 8000, 4 PCISPH iterations, dt 0.008). A step is one substep of
the reference's SphSimulation3DGrid::step() over all particles. The timed
region replays K steps (from step W+1 of the rollout) as CUDA graphs; the
state (>= 250 MB) is larger than L2, so no flush is needed between steps.

Arms
  default           this library (libfluidsph.so) through its C ABI
  --impl reference  the reference step's CPU restatement (the oracle, the
                    only runnable form of the reference here: its WGSL needs
                    wgpu + a Vulkan adapter, which this machine lacks), all
                    host cores, on a bounded sample of the same workload
Multi-GPU: replicas only (each rank runs its own scene; no collective on the
data path); value = all ranks' particle-steps / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "fluid-toy_gb300", ROOT):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

METRIC = "particle-steps/s"
# A simulation whose particle-count bucket is not yet in the process-wide
# table measures its neighbour passes' load depths on its steps 8-17 and keeps
# the fastest per pass (same results either way); warm-ups run past that, so
# timed regions use the chosen kernels (the reported warm-up is the count run).
WARMUP_PAST_TUNING = 20


# sorted slots from which the force pass runs without its cooperative kernel
COOP_MAX_PARTICLES = 262144


def kernels_per_step(iterations: int, particles: int) -> int:
    """Kernel launches of one step without rigid-body coupling: hash, scan,
    scatter, sort/gather with the big-cell sort and rank (3), warp work +
    order (2), density dedupe (mark, scan, list, list work, order: 5),
    density, dedupe copy, hit keys, key bases, key scatter, XSPH, force +
    predict (below COOP_MAX_PARTICLES sorted slots two kernels: the heavy
    particles cooperatively, then the rest), one solve per PCISPH iteration
    and finalize + integrate: 21 + iterations (+1). The grid clear is a
    memset, not counted."""
    return 21 + iterations + (1 if particles < COOP_MAX_PARTICLES else 0)


# algorithmic bytes per particle-step and per stage (SoA, compulsory traffic)
STAGE_BYTES = {"hash": 16, "reorder": 60, "density": 32, "xsph": 40, "force_predict": 68 + 68,
               "pcisph_solve": 100, "finalize_integrate": 48 + 48}
CELL_BYTES = {"clear": 4, "hash": 8, "scan": 8}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---- distributed plumbing (replicas) -----------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local_rank)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        return self._reduce(x, "max")

    def sum(self, x: float) -> float:
        return self._reduce(x, "sum")

    def _reduce(self, x: float, op: str) -> float:
        if not self.pg:
            return x
        import torch
        dev = "cuda" if torch.cuda.is_available() and self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX if op == "max" else self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def aggregate(units_local: float, seconds_local: float, dist: Dist) -> tuple[float, float]:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    units = dist.sum(units_local)
    secs = dist.max(seconds_local)
    return units / secs if secs > 0 else 0.0, secs


# ---- clocks during the timed region --------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---- arms ------------------------------------------------------------------------
def make_scene(config: int):
    from fluidsph import scenes
    return scenes.CONFIGS[config]()


def fp32_peak_tflops(device: int) -> tuple[float, str, dict]:
    """The FP32 roofline denominator: measured on this GPU by the library's
    FP32 throughput kernel (fs_selftest_fp32_rate: independent fma.rn chains
    at 32 warps per SM, best of five CUDA-event-timed launches); the nominal
    152 SMs x 128 lanes x 2 FLOP x max SM clock only if that call fails."""
    import ctypes as C

    import torch
    from fluidsph import abi
    rates = (C.c_double * 2)()
    if abi.load().fs_selftest_fp32_rate(device, rates) == 0 and rates[0] > 0:
        info = {"fma_tflops": round(rates[0], 2), "mul_add_tflops": round(rates[1], 2)}
        return rates[0], ("measured: fs_selftest_fp32_rate (fma.rn chains, 32 warps/SM, "
                          "CUDA events, best of 5)"), info
    p = torch.cuda.get_device_properties(device)
    sms = p.multi_processor_count
    mhz = 2070.0
    try:
        out = subprocess.run(["nvidia-smi", f"--id={device}", "--query-gpu=clocks.max.sm",
                              "--format=csv,noheader,nounits"], capture_output=True, text=True,
                             timeout=10).stdout.strip()
        mhz = float(out.splitlines()[0])
    except Exception:
        pass
    peak = sms * 128 * 2 * mhz * 1e6 / 1e12
    return peak, f"nominal: {sms} SMs x 128 FP32 lanes x 2 FLOP x {mhz:.0f} MHz", {}


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except Exception:
            pass
    return {}


def profile_traffic(kernel: str) -> float | None:
    """dram bytes per launch of `kernel` from the committed ncu summary."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            if line.startswith(f"traffic_bytes_per_launch[{kernel}]"):
                try:
                    return float(line.split("=", 1)[1].split()[0])
                except (IndexError, ValueError):
                    return None
    return None


def cpu_sample(scene, parts_np, steps: int, threads: int = 0) -> dict:
    """The oracle on the host cores, from the given state, for `steps` steps."""
    from oracle import oracle
    nthreads = oracle.set_threads(threads)
    o = oracle.OracleSim(parts_np, scene.sph, scene.geom)
    o.update_gravity(scene.gravity)
    o.set_pcisph_iterations(scene.iterations)
    if scene.rigid is not None:
        o.update_rigid_body(scene.rigid)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    return {"value": scene.n * steps / dt, "unit": METRIC, "cores": nthreads, "kind": "port",
            "seconds": dt, "steps": steps}


def statistics_vs_fp64(scene, steps: int, dev: int, first: int = 105, every: int = 5,
                       band: float = 0.01) -> dict:
    """The multi-step check of the plain step: this library's rollout and the
    oracle's FP64 twin (all host cores) over `steps` steps, flow statistics
    (total mass, mean density deviation, mean kinetic energy, |v|^2
    percentiles) sampled every `every` steps from step `first` and averaged;
    the relative differences must stay within `band` (the rollouts are
    chaotic, so trajectories are not compared)."""
    from fluidsph.sim import SphSimulation3DGrid
    from oracle import oracle
    from oracle.flow_stats import NAMES, fp64_sample, gpu_sample
    oracle.set_threads(0)
    rho0, mass = float(scene.sph.rest_density), float(scene.sph.mass)
    sim = SphSimulation3DGrid(scene.particles, scene.sph, scene.geom, device=dev)
    sim.update_gravity(scene.gravity)
    sim.set_pcisph_iterations(scene.iterations)
    if scene.rigid is not None:
        sim.update_rigid_body(scene.rigid)
    o64 = oracle.oracle_for_scene(scene, precision=64)
    gs, os_ = [], []
    done, t_cpu = 0, 0.0
    while done < steps:
        k = min(every - done % every, steps - done)
        sim.step(k)
        t0 = time.perf_counter()
        o64.step(k)
        t_cpu += time.perf_counter() - t0
        done += k
        if done >= first and done % every == 0:
            gs.append(gpu_sample(sim, rho0, mass, scene.geom))
            os_.append(fp64_sample(o64, rho0, mass, scene.geom))
    sim.close()
    g, o = np.mean(gs, axis=0), np.mean(os_, axis=0)
    rel = np.abs(g - o) / np.abs(o)
    return {"steps": steps, "window": f"steps {first}..{steps}, every {every}", "band": band,
            "gpu": dict(zip(NAMES, map(float, g))), "fp64": dict(zip(NAMES, map(float, o))),
            "relative_difference": dict(zip(NAMES, map(float, rel))),
            "within_band": bool(g[0] == o[0] and (rel[1:] <= band).all()),
            "fp64_cpu_seconds": round(t_cpu, 1)}


def run_ours(args, dist: Dist) -> dict | None:
    import torch
    from fluidsph.sim import SphSimulation3DGrid

    dev = dist.local_rank
    torch.cuda.set_device(dev)
    scene = make_scene(args.config)
    n = scene.n
    K, W = args.steps, max(args.warmup, WARMUP_PAST_TUNING)

    def fresh():
        sim = SphSimulation3DGrid(scene.particles, scene.sph, scene.geom, device=dev)
        sim.update_gravity(scene.gravity)
        sim.set_pcisph_iterations(scene.iterations)
        if scene.rigid is not None:
            sim.update_rigid_body(scene.rigid)
        sim.clear_rigid_body_accum()
        return sim

    # --- headline: K graph-replayed steps after W warm-up steps -------------------
    sim = fresh()
    stream = torch.cuda.Stream(device=dev)  # events and steps on one stream
    sim.set_stream(stream.cuda_stream)
    sim.step(W)
    sim.prepare_steps(K)  # capture the step graphs outside the timed region
    depths = sim.kernel_forms()
    sim.sync()
    state_after_warmup = sim.particles() if dist.rank == 0 and not args.no_cpu else None
    sim.neighbor_stats(reset=True)
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    dist.barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    sim.step(K)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    dist.barrier()
    clk = clocks.stop()
    secs = e0.elapsed_time(e1) / 1e3
    stats = sim.neighbor_stats(reset=True)
    value, secs_max = aggregate(n * K, secs, dist)
    sim.close()

    # --- per-stage timing of the same K steps (roofline inputs) --------------------
    sim = fresh()
    sim.step(W)
    sim.enable_stage_timing(True)
    sim.stage_times(reset=True)
    sim.step(K)
    stages, timed = sim.stage_times(reset=True)
    sim.close()
    per_step_ms = {k: v / max(timed, 1) for k, v in stages.items()}

    # --- e2e through the public API with host buffers ------------------------------
    # the reference app's per-substep pattern (app.rs:962-1019, 1205-1220): upload
    # the parameter structs from host memory, step, read the rigid-body
    # accumulator back (synchronising)
    sim = fresh()
    sim.step(W)
    sim.sync()
    h2d = 64 + 128 + 16 + 48 + 96
    d2h = 32
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(K):
        sim.update_sph_params(scene.sph)
        sim.update_container_geometry(scene.geom)
        sim.update_gravity(scene.gravity)
        if scene.rigid is not None:
            sim.update_rigid_body(scene.rigid)
        sim.step(1)
        sim.read_rigid_body_accum()
    e2e_secs = time.perf_counter() - t0
    dist.barrier()
    e2e_value, _ = aggregate(n * K, e2e_secs, dist)
    sim.close()

    forms = None
    if not args.no_forms:
        # the two other forms of the metric, on their own workloads (every rank
        # takes part: the batched arm aggregates over ranks)
        import argparse as _ap
        b = run_batch(_ap.Namespace(steps=50, warmup=3, loop_steps=10), dist)
        a = run_adjoint(_ap.Namespace(steps=200, warmup=3), dist)
        ident = run_identify(_ap.Namespace(gd_iters=3, identify_only=True), dist)
        if dist.rank == 0:
            forms = {
                "batched": {k: b[k] for k in ("value", "unit", "ms_per_step", "looped_plain",
                                              "batched_over_looped", "config", "clocks",
                                              "gpu_launches")},
                "adjoint": {k: a[k] for k in ("value", "unit", "forward_ms_per_step",
                                              "fwd_adjoint_over_forward", "gradient_finite",
                                              "config")},
                "batched_adjoint": {k: ident[k] for k in ("value", "unit", "forward_ms_per_step",
                                                          "fwd_adjoint_over_forward", "config")},
            }

    if dist.rank != 0:
        return None

    # --- roofline of the dominant kernel -----------------------------------------------
    nb = {k: v for k, v in per_step_ms.items() if k != "step"}
    dom = max(nb, key=nb.get)
    cand = stats["cand_density"] / K
    hits = stats["hits_density"] / K
    nonself = stats["hits_nonself"] / K
    cand_s = stats["cand_solve"] / K
    hits_s = stats["hits_solve"] / K
    flops = {
        "density": 6 * cand + 16 * hits,
        "xsph": 6 * cand + 16 * nonself,
        "force_predict": 6 * cand + 64 * nonself,
        "pcisph_solve": 6 * cand_s + 32 * hits_s,
    }
    fp32_peak, fp32_src, fp32_rates = fp32_peak_tflops(dev)
    peaks = measured_peaks()
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    hbm_src = "measured (MEASURED_PEAKS.json hbm_gbs)" if "hbm_gbs" in peaks else "fallback 6.8 TB/s"
    G = 52 ** 3

    def hbm_achieved(stage):
        b = STAGE_BYTES.get(stage, 0) * n + CELL_BYTES.get(stage, 0) * G
        return b / (per_step_ms[stage] * 1e-3) / 1e9 if per_step_ms[stage] > 0 else 0.0

    stage_report = {}
    for st, ms in nb.items():
        r = {"ms": round(ms, 4)}
        if st in flops:
            tf = flops[st] / (ms * 1e-3) / 1e12
            r.update({"tflops": round(tf, 3), "fp32_frac": round(tf / fp32_peak, 4)})
        r.update({"hbm_gbs": round(hbm_achieved(st), 1),
                  "hbm_frac": round(hbm_achieved(st) / hbm_peak, 4)})
        stage_report[st] = r
    kernel_name = {"pcisph_solve": "k_solve",
                   "force_predict": ("k_force_all" if scene.n >= COOP_MAX_PARTICLES
                                     else "k_force_predict"),
                   "density": "k_density", "xsph": "k_xsph"}.get(dom, dom)
    if dom in flops:
        iters = scene.iterations if dom == "pcisph_solve" else 1
        achieved = flops[dom] / (per_step_ms[dom] * 1e-3) / 1e12
        traffic = profile_traffic(kernel_name)
        roofline = {"bound": "fp32", "achieved": round(achieved, 3), "peak": round(fp32_peak, 1),
                    "unit": "TFLOP/s", "frac": round(achieved / fp32_peak, 4),
                    "traffic": traffic, "kernel": kernel_name, "launches_per_step": iters,
                    "flop_per_step": flops[dom], "peak_source": fp32_src,
                    "peak_rates_measured": fp32_rates,
                    "flop_model": "6 per candidate pair test + per in-range pair 16 density, "
                                  "16 xsph, 64 force, 32 solve; counts measured each step"}
    else:
        achieved = hbm_achieved(dom)
        roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak,
                    "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                    "traffic": profile_traffic(kernel_name), "kernel": kernel_name,
                    "peak_source": hbm_src}

    out = {
        "metric": METRIC, "value": round(value, 1), "unit": METRIC, "n_gpus": dist.world,
        "steps": K, "warmup": W, "ms_per_step": round(secs_max / K * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 lattice jitter)",
        "config": {"workload": scene.name, "particles": n, "steps_timed": f"{W + 1}..{W + K}",
                   "kernel_radius": 0.08, "pcisph_iterations": scene.iterations,
                   "load_depths": {k: depths[k] for k in ("density_loads", "xsph_loads",
                                                          "solve_loads", "decided", "bucket")},
                   "parallelism": f"replicas{dist.world}" if dist.world > 1 else "single",
                   "l2": "state > 250 MB exceeds the 129 MB L2 (no flush)"},
        "roofline": roofline,
        "roofline_stages": stage_report,
        "neighbors_per_step": {"candidates": cand, "hits": hits, "solve_candidates": cand_s},
        "e2e": {"value": round(e2e_value, 1), "unit": METRIC, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "pattern": "per step: upload sph/geometry/gravity/rigid-body structs, "
                           "fs_step(1), read rigid-body accumulator (sync)"},
        "gpu_launches": K * kernels_per_step(scene.iterations, scene.n),
        "clocks": clk,
    }
    if forms is not None:
        out["forms"] = forms
    from fluidsph.sim import kernel_forms_table
    out["load_depth_table"] = kernel_forms_table()
    if args.config == 0 and args.stats_steps > 0:
        out["statistics_vs_fp64"] = statistics_vs_fp64(scene, args.stats_steps, dev)
    if state_after_warmup is not None:
        cs = cpu_sample(scene, state_after_warmup, args.cpu_steps)
        cs["sample"] = (f"{scene.name}: oracle (FP32 C++ restatement, OpenMP) from the GPU "
                        f"state after step {W}, {args.cpu_steps} steps")
        out["cpu_baseline"] = cs
    return out


def run_batch(args, dist: Dist) -> dict | None:
    """The batched ensemble: all scenes in one launch per stage, K steps from
    graphs, against looping the plain simulation over the same scenes (one
    stream, each scene's steps graph-replayed)."""
    import torch
    from fluidsph import scenes as S
    from fluidsph.sim import SphBatch3DGrid, SphSimulation3DGrid

    dev = dist.local_rank
    torch.cuda.set_device(dev)
    scenes = S.config2()
    counts = np.array([s.n for s in scenes])
    total = int(counts.sum())
    K, W = args.steps, max(args.warmup, WARMUP_PAST_TUNING)
    stream = torch.cuda.Stream(device=dev)

    b = SphBatch3DGrid([s.particles for s in scenes], [s.sph for s in scenes],
                       [s.geom for s in scenes], device=dev)
    for k, s in enumerate(scenes):
        b.update_scene(k, gravity=s.gravity)
    b.set_pcisph_iterations(scenes[0].iterations)
    b.set_stream(stream.cuda_stream)
    b.step(W)
    t0 = time.perf_counter()
    b.prepare_steps(K)
    capture_s = time.perf_counter() - t0
    b.sync()
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    dist.barrier()
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.step(K)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    dist.barrier()
    clk = clocks.stop()
    secs = e0.elapsed_time(e1) / 1e3
    value, secs_max = aggregate(total * K, secs, dist)
    b.enable_stage_timing(True)
    b.stage_times(reset=True)
    b.step(min(K, 20))
    stages, timed = b.stage_times(reset=True)
    depths = b.kernel_forms()
    b.close()

    # looped plain: the same scenes one after another on one stream, each for
    # k_loop graph-replayed steps after W warm-up steps
    k_loop = max(1, min(K, args.loop_steps))
    sims = []
    for s in scenes:
        sim = SphSimulation3DGrid(s.particles, s.sph, s.geom, device=dev)
        sim.update_gravity(s.gravity)
        sim.set_pcisph_iterations(s.iterations)
        sim.set_stream(stream.cuda_stream)
        sim.step(W)
        sim.prepare_steps(k_loop)
        sims.append(sim)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    for sim in sims:
        sim.step(k_loop)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    loop_secs = e0.elapsed_time(e1) / 1e3
    loop_value, _ = aggregate(total * k_loop, loop_secs, dist)
    for sim in sims:
        sim.close()
    if dist.rank != 0:
        return None
    per_step_ms = {k: round(v / max(timed, 1), 4) for k, v in stages.items()}
    return {
        "metric": METRIC, "value": round(value, 1), "unit": METRIC, "n_gpus": dist.world,
        "steps": K, "warmup": W, "ms_per_step": round(secs_max / K * 1e3, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 scene draws and lattice jitter)",
        "config": {"workload": f"batched_ensemble_{len(scenes)}_scenes", "scenes": len(scenes),
                   "particles": total, "count_range": [int(counts.min()), int(counts.max())],
                   "steps_timed": f"{W + 1}..{W + K}", "graph_capture_s": round(capture_s, 3),
                   "load_depths": {k: depths[k] for k in ("density_loads", "xsph_loads",
                                                          "solve_loads", "decided", "bucket")},
                   "l2": "state > 1 GB exceeds the 129 MB L2 (no flush)"},
        "stages_ms_per_step": per_step_ms,
        "looped_plain": {"value": round(loop_value, 1), "unit": METRIC, "steps": k_loop,
                         "ms_per_step": round(loop_secs / k_loop * 1e3, 4),
                         "pattern": "one SphSimulation3DGrid per scene on one stream, "
                                    "each fs_step(k) graph-replayed, scene after scene"},
        "batched_over_looped": round(value / loop_value, 3) if loop_value else None,
        "gpu_launches": K * kernels_per_step(scenes[0].iterations, total),
        "clocks": clk,
    }


def run_adjoint(args, dist: Dist) -> dict | None:
    """The differentiable rollout: forward-only ms/step (graph-replayed steps)
    against forward + reverse ms/step (fs_adj_forward with checkpoints every
    20 steps, the density-splat loss, fs_adj_backward), same workload."""
    import torch
    from fluidsph import scenes as S
    from fluidsph.adjoint import DifferentiableRollout
    from fluidsph.sim import SphSimulation3DGrid

    dev = dist.local_rank
    torch.cuda.set_device(dev)
    sc = S.config3()
    T = args.steps
    every = 20
    mc = S.loss_grid(sc)

    def fresh(sph=None):
        sim = SphSimulation3DGrid(sc.particles, sph or sc.sph, sc.geom, device=dev)
        sim.update_gravity(sc.gravity)
        sim.set_pcisph_iterations(sc.iterations)
        return sim

    hidden_p = type(sc.sph).from_buffer_copy(sc.sph)
    hidden_p.viscosity, hidden_p.stiffness = 12.0, 30.0
    hidden = fresh(hidden_p)
    hidden.step(T)
    target = hidden.density_splat(mc, sc.geom)  # the hidden run's field
    hidden.close()

    stream = torch.cuda.Stream(device=dev)
    sim = fresh()
    sim.set_stream(stream.cuda_stream)
    # warm-up past the simulation's load-depth measurement (steps 8-17),
    # back to the initial state, then the graphs with the chosen kernels
    sim.step(max(args.warmup, WARMUP_PAST_TUNING))
    sim.upload_particles(sc.particles)
    sim.prepare_steps(T)
    sim.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    sim.step(T)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    fwd_ms = e0.elapsed_time(e1) / T

    r = DifferentiableRollout(sim, every)
    sim.upload_particles(sc.particles)
    r.forward(T)  # warm-up of the recording path
    r.splat_mse_loss(mc, sc.geom, target)
    r.backward()
    sim.upload_particles(sc.particles)
    sim.sync()
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    r.forward(T)
    loss = r.splat_mse_loss(mc, sc.geom, target)
    dpos, dvel, _ = r.backward()
    torch.cuda.synchronize(dev)
    total_ms = (time.perf_counter() - t0) * 1e3 / T
    dpar = r.param_gradients()
    finite = bool(np.isfinite(dvel).all() and np.isfinite(dpar).all())
    r.close()
    sim.close()
    if dist.rank != 0:
        return None
    return {
        "metric": "fwd+adjoint ms/step", "value": round(total_ms, 4), "unit": "ms/step",
        "n_gpus": dist.world, "steps": T, "warmup": max(args.warmup, WARMUP_PAST_TUNING),
        "ms_per_step": round(total_ms, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded lattice, 8-mode Fourier initial velocity)",
        "config": {"workload": sc.name, "particles": sc.n, "steps": T, "checkpoint_every": every,
                   "loss": "MSE of the 64^3 density splat against a hidden run "
                           "(viscosity 12, stiffness 30)"},
        "forward_ms_per_step": round(fwd_ms, 4),
        "fwd_adjoint_over_forward": round(total_ms / fwd_ms, 3),
        "loss": loss, "gradient_finite": finite,
        "grad_params": {n: float(dpar[0, i])
                        for i, n in enumerate(DifferentiableRollout.PARAM_NAMES)},
    }


def _identify(scenes, hidden, steps, every, iters, grid_size, dev, timed=False, tape_budget=0):
    """Batched gradient descent on per-scene viscosity, pcisph_delta (the
    pressure strength the step reads) and surface tension against
    hidden-parameter targets. Steps are sign steps scaled by a decaying rate
    relative to each parameter's range, robust to the gradients' magnitude.
    Returns the parameter errors, the losses and (timed) fwd+adjoint
    ms/step."""
    import torch
    from fluidsph import scenes as S
    from fluidsph.adjoint import DifferentiableRollout
    from fluidsph.sim import SphBatch3DGrid

    def batch(params):
        b = SphBatch3DGrid([s.particles for s in scenes], params, [s.geom for s in scenes],
                           device=dev)
        for k, s in enumerate(scenes):
            b.update_scene(k, gravity=s.gravity)
        b.set_pcisph_iterations(scenes[0].iterations)
        return b

    def with_(p, **kw):
        q = type(p).from_buffer_copy(p)
        for k, v in kw.items():
            setattr(q, k, v)
        return q

    grids = [S.loss_grid(s, grid_size) for s in scenes]
    hb = batch([with_(s.sph, **h) for s, h in zip(scenes, hidden)])
    hr = DifferentiableRollout(hb, every)
    hr.forward(steps)
    # the targets stay on the device; the losses of all scenes are taken in
    # one call (one grid build of the final state, one read-back)
    targets = [torch.from_numpy(hr.final_splat(grids[k], scenes[k].geom, scene=k)).to(dev)
               for k in range(len(scenes))]
    geoms = [s.geom for s in scenes]
    hr.close()
    hb.close()
    params = [with_(s.sph) for s in scenes]
    b = batch(params)
    r = DifferentiableRollout(b, every, tape_budget_bytes=tape_budget)
    names = ("viscosity", "pcisph_delta", "surface_tension")
    cols = [DifferentiableRollout.PARAM_NAMES.index(n) for n in names]
    init = np.array([[getattr(p, n) for n in names] for p in params], np.float64)
    cur = init.copy()
    truth = np.array([[h[n] for n in names] for h in hidden], np.float64)
    span = np.maximum(np.abs(truth - init).max(axis=0), 1e-3)
    losses, ms = [], []
    for it in range(iters):
        for k, p in enumerate(params):
            p.viscosity, p.pcisph_delta, p.surface_tension = (float(v) for v in cur[k])
            b.update_scene(k, sph_params=p)
        for k, s in enumerate(scenes):
            b.upload_scene_particles(k, s.particles)
        b.sync()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        r.forward(steps)
        loss = sum(r.splat_mse_losses(grids, geoms, targets).tolist())
        r.backward(scenes=len(scenes))
        g = r.param_gradients(scenes=len(scenes))[:, cols]
        torch.cuda.synchronize(dev)
        ms.append((time.perf_counter() - t0) * 1e3 / steps)
        losses.append(loss)
        rate = 0.25 * (0.9 ** it)
        step = np.where(np.isfinite(g) & (g != 0), -np.sign(np.nan_to_num(g)), 0.0) * rate * span
        cur = cur + step
    tape_segments, segment_bytes = r.tape_info()
    r.close()
    b.close()
    err = np.abs(cur - truth) / np.abs(truth)
    err0 = np.abs(init - truth) / np.abs(truth)
    return {"relative_error_initial": {n: float(np.mean(err0[:, i])) for i, n in enumerate(names)},
            "relative_error_final": {n: float(np.mean(err[:, i])) for i, n in enumerate(names)},
            "loss_first": losses[0] if losses else None, "loss_last": losses[-1] if losses else None,
            "gradient_finite": bool(np.isfinite(g).all()) if iters else None,
            "fwd_adjoint_ms_per_step": float(np.median(ms)) if ms else None,
            "tape_segments": tape_segments, "tape_segment_gb": round(segment_bytes / 1e9, 3)}


def run_identify(args, dist: Dist) -> dict | None:
    """Batched adjoint parameter identification (64 scenes, counts in [8192,
    32768], 150 steps, checkpoint every 15): fused batched forward + reverse
    ms/step and the parameter errors after `--gd-iters` iterations; plus the
    same procedure on 64 small rollouts with the reference app's default
    physics, where the loss is smooth and the identification converges."""
    import torch
    from fluidsph import scenes as S
    from fluidsph.sim import SphBatch3DGrid

    dev = dist.local_rank
    torch.cuda.set_device(dev)
    scs, hidden = S.config4()
    total = sum(s.n for s in scs)
    # forward-only ms/step of the same batch (graph-replayed)
    b = SphBatch3DGrid([s.particles for s in scs], [s.sph for s in scs], [s.geom for s in scs],
                       device=dev)
    for k, s in enumerate(scs):
        b.update_scene(k, gravity=s.gravity)
    b.set_pcisph_iterations(scs[0].iterations)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.Stream(device=dev)  # events and steps on one stream
    b.set_stream(stream.cuda_stream)
    # warm-up past the load-batching measurement, then back to the initial state
    b.step(WARMUP_PAST_TUNING)
    for k, s in enumerate(scs):
        b.upload_scene_particles(k, s.particles)
    b.prepare_steps(150)
    torch.cuda.synchronize(dev)
    e0.record(stream)
    b.step(150)
    e1.record(stream)
    torch.cuda.synchronize(dev)
    fwd_ms = e0.elapsed_time(e1) / 150
    b.close()
    spec = _identify(scs, hidden, 150, 15, args.gd_iters, 64, dev)
    budgeted = well = None
    if not getattr(args, "identify_only", False):
        # the same with a tape budget of half the free device memory: the
        # forward records as many checkpoint segments as fit and the backward
        # re-runs only the others (timing only: two iterations)
        free, _ = torch.cuda.mem_get_info(dev)
        budget = int(free * 0.5)
        budgeted = _identify(scs, hidden, 150, 15, 2, 64, dev, tape_budget=budget)
        well = _identify(*S.reference_physics_batch(64, 20), 20, 5, 50, 32, dev)
    if dist.rank != 0:
        return None
    v = spec["fwd_adjoint_ms_per_step"]
    if budgeted is None:
        return {"metric": "batched fwd+adjoint ms/step", "value": round(v, 4), "unit": "ms/step",
                "forward_ms_per_step": round(fwd_ms, 4),
                "fwd_adjoint_over_forward": round(v / fwd_ms, 3),
                "config": {"workload": "batched_identification_64_scenes", "scenes": len(scs),
                           "particles": total, "steps": 150, "checkpoint_every": 15,
                           "tape_budget": 0, "gd_iterations": args.gd_iters,
                           "timing": "median over the iterations of fs_adj_forward(150) + "
                                     "losses + fs_adj_backward, wall clock"},
                "identification": spec}
    return {
        "metric": "batched fwd+adjoint ms/step", "value": round(v, 4), "unit": "ms/step",
        "n_gpus": dist.world, "steps": 150, "warmup": 0, "ms_per_step": round(v, 4),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded scene draws, lattice jitter, hidden parameters)",
        "config": {"workload": "batched_identification_64_scenes", "scenes": len(scs),
                   "particles": total, "steps": 150, "checkpoint_every": 15,
                   "gd_iterations": args.gd_iters},
        "forward_ms_per_step": round(fwd_ms, 4),
        "fwd_adjoint_over_forward": round(v / fwd_ms, 3),
        "identification": spec,
        "with_tape_budget": {
            "tape_budget_gb": round(budget / 1e9, 1),
            "tape_segments": budgeted["tape_segments"],
            "checkpoint_segments": 10,
            "fwd_adjoint_ms_per_step": round(budgeted["fwd_adjoint_ms_per_step"], 4),
            "fwd_adjoint_over_forward": round(budgeted["fwd_adjoint_ms_per_step"] / fwd_ms, 3)},
        "identification_reference_physics": well,
    }


def repo_libraries() -> list[str]:
    """Shared objects of this repository mapped into this process (Linux)."""
    try:
        maps = Path("/proc/self/maps").read_text()
    except OSError:
        return []
    root = str(ROOT)
    found = {ln.split()[-1] for ln in maps.splitlines()
             if ln.split() and ln.split()[-1].startswith(root) and ".so" in ln.split()[-1]}
    return sorted(str(Path(f).relative_to(root)) for f in found)


def run_reference(args, dist: Dist) -> dict | None:
    """The reference arm: the reference step's CPU restatement (the oracle) on
    all host cores. It warms up exactly as this library's arm does
    (max(--warmup, WARMUP_PAST_TUNING) steps from the same seeded scene; the
    oracle's trajectory is the GPU's bit for bit), so both arms time the same
    rollout states from step W+1 on, and it builds its parameter structs with
    the oracle's own restatement of the reference's host builders, so the
    product library is never loaded."""
    if dist.rank != 0:
        return None
    from fluidsph import scenes
    from oracle import host_params, oracle
    if args.config not in (0, 1):
        raise SystemExit("--impl reference runs the plain configurations 0 and 1")
    scene = scenes.CONFIGS[args.config](builders=host_params)
    W, K = max(args.warmup, WARMUP_PAST_TUNING), args.steps
    nthreads = oracle.set_threads(0)
    o = oracle.oracle_for_scene(scene)
    if scene.rigid is not None:
        o.clear_rigid_body_accum()
    k_cpu = min(K, args.cpu_steps)
    o.step(W)
    t0 = time.perf_counter()
    o.step(k_cpu)
    secs = time.perf_counter() - t0
    value = scene.n * k_cpu / secs
    sample = (f"{scene.name}: oracle (FP32 C++ restatement of the step WGSL, OpenMP), "
              f"steps {W + 1}..{W + k_cpu}")
    return {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": METRIC,
            "n_gpus": dist.world, "steps": k_cpu, "warmup": W,
            "ms_per_step": round(secs / k_cpu * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": scene.name, "particles": scene.n,
                       "steps_timed": f"{W + 1}..{W + k_cpu}",
                       "gpu_arm_steps_timed": f"{W + 1}..{W + K}",
                       "same_states": "both arms start timing at step W+1 of the same seeded "
                                      "rollout; this arm times the first "
                                      f"{k_cpu} of the GPU arm's {K} steps"},
            "cpu_baseline": {"value": round(value, 1), "unit": METRIC, "cores": nthreads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": round(value, 1), "unit": METRIC, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "libraries_loaded": repo_libraries()}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--cpu-steps", type=int, default=5)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-forms", action="store_true",
                    help="skip the batched and differentiable forms in the default run")
    ap.add_argument("--stats-steps", type=int, default=1000,
                    help="--config 0: steps of the rollout compared with the FP64 twin's "
                         "flow statistics (0: skip)")
    ap.add_argument("--gd-iters", type=int, default=3,
                    help="gradient-descent iterations of the --config 4 workload")
    ap.add_argument("--loop-steps", type=int, default=20,
                    help="steps per scene of the looped-plain comparison (--config 2)")
    args = ap.parse_args()
    if args.warmup < 3:
        log("warm-up raised to 3 steps")
        args.warmup = 3
    dist = Dist()
    try:
        if args.impl == "reference":
            out = run_reference(args, dist)
        else:
            from fluidsph.build import build_library
            if dist.local_rank == 0:
                build_library()
            dist.barrier()
            if args.config == 2:
                out = run_batch(args, dist)
            elif args.config == 3:
                out = run_adjoint(args, dist)
            elif args.config == 4:
                out = run_identify(args, dist)
            else:
                out = run_ours(args, dist)
        if out is not None:
            print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
