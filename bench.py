#!/usr/bin/env python
"""Benchmark of the GB300 SPH step (one JSON line on stdout).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload dam_break_1M|dam_break_4M|dam_break_10M|dam_break_10k]

A "step" is one SPHEngine::step over the workload's particles.  Protocol: fresh-state
(every step starts from the workload's initial state, restored on the device before the
step and outside its timing): after step 1 the reference's dynamics degenerate (clamped
walls, crowded cells, then inf/NaN), so the initial state is the one the workload
describes.  Between timed steps the L2 cache is flushed (a 512 MiB buffer is written).

  value      particle-steps/s, device time (CUDA events on the library's stream) of the K
             steps with the state already resident in HBM, each step replayed from the CUDA
             graph the library captured (the eager-launch time is in config.launch); summed
             over all ranks' replicas
  e2e        the same through the C ABI with host buffers: every step uploads the initial
             state from pinned host memory, steps, and downloads positions, velocities and
             densities (all inside the step's timed interval; the L2 flush before each step
             is not)
  roofline   the force+integrate kernel (the dominant kernel): algorithmic bytes per launch
             (72 B per particle) over its average CUDA-event duration, against the measured
             HBM copy bandwidth
  roofline_issue  the same kernel against the issue roof (it is instruction-issue bound):
             warp instructions per particle (ncu, profiles/ncu_issue.json) x particles over
             the kernel time, against SMs x 4 issue slots per clock x the sampled SM clock
  cpu_baseline  the oracle port (C restatement of the reference step, OpenMP on all host
             cores) on a bounded sample of the same workload
  extras     e2e_dropin (sph.Simulator step + get_positions + get_densities, host clock),
             batched_256 (the 256-scene mix, batched vs looped plain steps, autotuned, with
             its own trajectory bounded to 30 s and an FP64 density check of 8 scenes in the
             CPU leg), dam_break_1M_precise (the same workload in the precision mode:
             cell + offset storage and the tile sweeps), dam_break_10M (exact and
             precision mode, fresh-state),
             dam_break_10M_trajectory (the 10M configuration's own 50 CFL steps in precision
             mode with per-step FP64 mass / energy drift, bounded to 60 s of device time),
             dam_break_1M_faithful (the 1M workload's own trajectory with per-step cell
             occupancy and non-finite counts, bounded to 30 s of device time)

--impl reference times the reference's CPU implementation of the path (the oracle port:
the reference's own build cannot be compiled on the GPU host) on all host cores, on the
same workload and metric; under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "sph-particle-simulator_gb300" / "python"))
sys.path.insert(0, str(REPO / "oracle"))

import numpy as np  # noqa: E402

import sphx_inputs as I  # noqa: E402

METRIC = "particle-steps/s at 1M and 10M (+% HBM roofline); batched vs plain at stated FP64 error"
UNIT = "particle-steps/s"
FORCE_BYTES_PER_PARTICLE = 72    # read x,v,rho,P,m (36 B); write x,v,a (36 B)
DENSITY_BYTES_PER_PARTICLE = 24  # read x,m (16 B); write rho,P (8 B)
# The passes of each mode: the kernels measured, their algorithmic bytes per particle and
# the keys of their committed ncu summaries.  Precision mode stores a position as an
# integer cell (12 B) plus an FP32 offset (12 B): force reads x (24), v, rho, P, m (24) and
# writes x, v, a (48); density reads x, m (28) and writes rho, P (8).
PASSES = {
    "exact": {"force": "k_force<1,0,0,1,0,0> (force + leapfrog + clamp)",
              "density": "k_density<0,0,1,0>", "force_bytes": FORCE_BYTES_PER_PARTICLE,
              "density_bytes": DENSITY_BYTES_PER_PARTICLE, "issue_force": "k_force",
              "issue_density": "k_density", "traffic": "force"},
    "precise": {"force": "k_force_sweep<1,0,0> (force + leapfrog + clamp, tile sweep)",
                "density": "k_density_sweep<0>", "force_bytes": 96, "density_bytes": 36,
                "issue_force": "k_force_sweep", "issue_density": "k_density_sweep",
                "traffic": "force_sweep"},
}
# published CPU figure for the 1M case: README.md:45, 38 steps/s at 1M particles
PUBLISHED_1M = 38.0 * 1_000_000
L2_FLUSH_BYTES = 512 << 20
FALLBACK_HBM_GBS = 6800.0


def workload(name: str) -> I.Workload:
    return {"dam_break_10k": I.config0, "dam_break_1M": I.config1,
            "dam_break_10M": I.config4,
            # 160^3 = 4.1M: the config-1 lattice large enough that its arrays exceed L2
            # (the case the per-particle DRAM traffic of the passes is measured on)
            "dam_break_4M": lambda: I.scaled_dam_break(160 ** 3, seed=1)}[name]()


SM_COUNT_FALLBACK = 152
ISSUE_PER_SM_PER_CLK = 4  # one warp instruction per clock per sub-partition, 4 per SM


def ncu_issue(kernel: str):
    """Warp instructions per particle of a pass (k_force / k_density) on the 1M dam break,
    from the committed ncu summary; None if absent."""
    p = REPO / "profiles" / "ncu_issue.json"
    if not p.exists():
        return None
    try:
        return float(json.loads(p.read_text())[kernel]["warp_inst_per_particle"])
    except Exception:
        return None


def peaks() -> tuple[float, str]:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(key: str, n: int):
    """Per-launch DRAM bytes of a force kernel ("force": exact mode, "force_sweep":
    precision mode) from the committed ncu summary (measured per particle on the 4.1M
    lattice, whose arrays exceed L2), scaled to this workload's particle count; returns
    (total, hit-mask records part) or (None, None)."""
    p = REPO / "profiles" / "ncu_traffic.json"
    if not p.exists():
        return None, None
    try:
        f = json.loads(p.read_text())[key]
        return (float(f["dram_bytes_per_particle"]) * n,
                float(f.get("hit_mask_bytes_per_particle", 0.0)) * n)
    except Exception:
        return None, None


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(gpu_index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            return None
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(dist, seconds: float, device: str = "cuda") -> float:
    """The slowest rank's time: replicas finish when the last one does (no collective at
    world size 1; NCCL on the GPUs, any backend's tensor device otherwise)."""
    if dist is None:
        return seconds
    import torch

    t = torch.tensor([seconds], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world: int, particles: int, steps: int, max_seconds: float) -> float:
    """Whole-job particle-steps/s of `world` replicas each stepping `particles` `steps`
    times, timed by the slowest."""
    return world * particles * steps / max_seconds


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---------------------------------------------------------------------------------------
# CPU: the oracle port (C restatement of the reference step) on the host cores
# ---------------------------------------------------------------------------------------

def run_cpu(w: I.Workload, steps: int, warmup: int, budget_s: float | None = None) -> dict:
    import sph_oracle as O

    port = O.Port()
    cores = port.threads()
    e = O.Engine(port, w.n)
    e.initialize(w.params)
    e.add(w.pos, w.vel, w.mass)
    times = []
    done = 0
    t_all = time.perf_counter()
    for s in range(warmup + steps):
        e.set_state(w.pos, w.vel)
        t0 = time.perf_counter()
        e.step(w.dt)
        dt = time.perf_counter() - t0
        if s >= warmup:
            times.append(dt)
            done += 1
        if budget_s is not None and time.perf_counter() - t_all > budget_s and done >= 1:
            break
    total = sum(times)
    return {"value": w.n * len(times) / total, "unit": UNIT, "cores": cores, "kind": "port",
            "steps": len(times), "seconds": total,
            "sample": f"{w.name}: {w.n} particles, {len(times)} fresh-state steps"}


def workload_config(w: I.Workload, workload_name: str, world: int, mode: str = "exact") -> dict:
    """The `config` object of both arms' JSON lines: the workload and its protocol."""
    return {
        "workload": workload_name, "particles": w.n,
        "lattice": "x".join(map(str, w.info.get("lattice", ()))), "dt": w.dt,
        "protocol": "fresh-state (initial state restored before each step)",
        "l2": "GPU arm: flushed between timed steps (512 MiB write)", "mode": mode,
        "parallelism": f"replicas x{world}",
    }


def bench_reference(args, world, rank):
    if rank != 0:
        return 0
    w = workload(args.workload)
    # bound the run: a few minutes for warmup + steps on the host cores
    r = run_cpu(w, args.steps, args.warmup, budget_s=180.0)
    line = {
        "impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": r["steps"], "warmup": args.warmup,
        "ms_per_step": 1e3 * r["seconds"] / max(r["steps"], 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": r["value"] / PUBLISHED_1M if args.workload == "dam_break_1M" else None,
        "dtype": "f32", "data": "synthetic",
        "config": workload_config(w, args.workload, world),
        "implementation": "oracle port of the reference step (C, OpenMP on all host cores)",
        "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": r["cores"], "kind": "port",
                         "sample": r["sample"]},
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------------------
# GPU
# ---------------------------------------------------------------------------------------

def timed_steps(torch, ctx, w, steps, flush):
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    for k in range(steps):
        ctx.restore()
        flush.fill_(k & 0xFF)
        ev[k][0].record()
        ctx.step(w.dt)
        ev[k][1].record()
    torch.cuda.synchronize()
    return [a.elapsed_time(b) for a, b in ev]


def ctx_closed(ctx) -> bool:
    return not ctx._h


def bench_batched(torch, stream, flush, steps):
    """The batched fluid-drop mix (256 scenes, log-uniform 2k..200k particles, ~10M total),
    fresh-state steps at dt 5e-4: one batched, graph-captured, autotuned step over all
    scenes, against looping the plain step over the scenes (one context per scene, all on
    the same stream).  Device time of the steps only; restores happen outside it."""
    import sphx

    b = I.batched_fluid_drops()
    ctx = sphx.Context(b.n, graph=True)
    ctx.set_stream(stream.cuda_stream)
    ctx.upload(b.pos, b.vel, b.mass)
    ctx.set_scenes(b.scene_start, b.params)
    wpb, bps, tuned_ms = ctx.autotune(b.dt)
    ctx.snapshot()
    for _ in range(3):
        ctx.restore()
        ctx.step(b.dt)
    ms = timed_steps(torch, ctx, b, steps, flush)
    batched_ms = sum(ms) / steps
    tuned = ctx.tuning()
    # the densities of one batched step from the initial state, for the FP64 check of the
    # CPU leg (sampled scenes)
    ctx.restore()
    ctx.step(b.dt)
    rho_batched = ctx.download(pos=False, vel=False, pressure=False, acc=False)["rho"]
    traj = bench_batched_trajectory(torch, ctx, b)
    ctx.close()
    ctxs = []
    for s in range(len(b.params)):
        pos, vel, mass, prm = b.scene(s)
        c = sphx.Context(pos.shape[0], max_grid_cells=4 * pos.shape[0] + 4096)
        c.set_stream(stream.cuda_stream)
        c.set_params(prm)
        c.upload(pos, vel, mass)
        c.snapshot()
        c.step(b.dt)
        ctxs.append(c)
    torch.cuda.synchronize()
    loop = []
    for _ in range(steps):
        for c in ctxs:
            c.restore()
        flush.fill_(3)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for c in ctxs:
            c.step(b.dt)
        e1.record()
        torch.cuda.synchronize()
        loop.append(e0.elapsed_time(e1))
    for c in ctxs:
        c.close()
    looped_ms = sum(loop) / steps
    return {"scenes": len(b.params), "particles": b.n, "steps": steps,
            "batched_value": b.n / (batched_ms * 1e-3), "batched_ms_per_step": batched_ms,
            "looped_plain_value": b.n / (looped_ms * 1e-3), "looped_ms_per_step": looped_ms,
            "speedup": looped_ms / batched_ms, "unit": UNIT,
            "autotuned": {"warps_per_block": wpb, "blocks_per_sm": bps,
                          "tile_particles": tuned["tile_particles"],
                          "threads_per_tile": 32, "cell_size_multiplier": 1, "ms": tuned_ms},
            "trajectory": traj,
            "protocol": "fresh-state, dt 5e-4, exact mode (every scene bit-identical to "
                        "stepping it alone), batched step captured as a CUDA graph"}, rho_batched


def bench_batched_trajectory(torch, ctx, b, budget_s=30.0):
    """The batched mix's own trajectory: up to its 200 steps at dt 5e-4 from the initial
    state, batched and graph-replayed, each step timed on the device, with the FP64 mass
    and energy summed over the scenes after every step.  Stops after the step crossing
    `budget_s` of device time (the drops' dynamics crowd the cells within a few steps)."""
    ctx.restore()
    torch.cuda.synchronize()
    mass0 = float(b.mass.astype(np.float64).sum())
    log, total = [], 0.0
    for s in range(b.steps):
        e_a, e_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e_a.record()
        ctx.step(b.dt)
        e_b.record()
        torch.cuda.synchronize()
        ms = e_a.elapsed_time(e_b)
        st = ctx.stats()
        mass, energy = 0.0, 0.0
        for k in range(len(b.params)):
            sc = ctx.scene_stats(k)
            mass += sc["sum_mass"]
            energy += sc["kinetic_energy"] + sc["potential_energy"]
        log.append([round(ms, 3), (mass - mass0) / mass0, energy, st["max_cell_occupancy"]])
        total += ms * 1e-3
        if total > budget_s:
            break
    return {"steps_done": len(log), "steps": b.steps, "dt": b.dt, "device_s": total,
            "value": b.n * len(log) / total, "unit": UNIT, "per_step": log,
            "per_step_fields": ["ms", "mass_drift_rel", "fp64_energy_sum",
                                "max_cell_occupancy"],
            "protocol": f"faithful batched trajectory from the initial state, stopped after "
                        f"the step crossing {budget_s:.0f} s of device time"}


def batched_fp64_check(port, rho_batched, nsample=8):
    """Density relative error of the batched step against the oracle's FP64 re-evaluation
    of the same initial state, on a seeded sample of scenes (the CPU leg's checker)."""
    b = I.batched_fluid_drops()
    rng = np.random.default_rng(33)
    worst, means = 0.0, []
    picked = sorted(int(x) for x in rng.choice(len(b.params), nsample, replace=False))
    for s in picked:
        pos, vel, mass, prm = b.scene(s)
        a, e = int(b.scene_start[s]), int(b.scene_start[s + 1])
        rho64, _, _ = port.fields_f64(pos, vel, mass, prm)
        rel = np.abs(rho_batched[a:e].astype(np.float64) - rho64) / np.abs(rho64)
        worst = max(worst, float(rel.max()))
        means.append(float(rel.mean()))
    return {"fp64_rho_rel_max": worst, "fp64_rho_rel_mean": float(np.mean(means)),
            "fp64_scenes_checked": picked}


def bench_10m_trajectory(torch, stream, w10, budget_s=60.0):
    """The 10M dam break as its configuration states it: from the initial state, up to its
    50 steps with step(0) (CFL timestep, FP64 maximum, capped at params.timestep = 2e-4) in
    the precision mode, each step timed on the device, with the FP64 mass, momentum and
    energy (kinetic + gravitational potential) after every step and their drift from the
    initial state's (summed in FP64 on the host from the inputs).  Stops after the step
    that crosses `budget_s` of device time."""
    import sphx

    ctx = sphx.Context(w10.n, mode=sphx.MODE_PRECISE)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_params(w10.params)
    ctx.upload(w10.pos, w10.vel, w10.mass)
    m64 = w10.mass.astype(np.float64)
    g = float(w10.params[6])
    mass0 = float(m64.sum())
    e0 = float((0.5 * m64 * (w10.vel.astype(np.float64) ** 2).sum(1)).sum()
               + (-m64 * g * w10.pos[:, 1].astype(np.float64)).sum())
    torch.cuda.synchronize()
    log, total = [], 0.0
    for s in range(w10.steps):
        e_a, e_b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e_a.record()
        ctx.step(0.0)
        e_b.record()
        torch.cuda.synchronize()
        ms = e_a.elapsed_time(e_b)
        st = ctx.stats()
        t, dt = ctx.time_f64()
        energy = st["kinetic_energy"] + st["potential_energy"]
        log.append([round(ms, 3), dt, t, (st["sum_mass"] - mass0) / mass0,
                    (energy - e0) / abs(e0), st["momentum"][0], st["momentum"][1],
                    st["momentum"][2], st["max_cell_occupancy"], st["nonfinite_particles"]])
        total += ms * 1e-3
        if total > budget_s:
            break
    ctx.close()
    done = len(log)
    return {"value": w10.n * done / total, "unit": UNIT, "steps_done": done,
            "steps": w10.steps, "device_s": total, "mode": "cell + FP32 offset, compensated sums",
            "initial_fp64_mass": mass0, "initial_fp64_energy": e0,
            "max_abs_mass_drift": max(abs(r[3]) for r in log),
            "final_energy_drift": log[-1][4], "per_step": log,
            "per_step_fields": ["ms", "dt_fp64", "time_fp64", "mass_drift_rel",
                                "energy_drift_rel", "momentum_x", "momentum_y", "momentum_z",
                                "max_cell_occupancy", "nonfinite_particles"],
            "protocol": f"faithful trajectory from the initial state, step(0) (CFL, FP64 max, "
                        f"cap 2e-4), stopped after the step crossing {budget_s:.0f} s of "
                        f"device time"}


def bench_dropin(w, steps):
    """The drop-in engine end to end, as a user of the reference's Python API drives it:
    sph.Simulator (the C++ SPHEngine over the C ABI) -- step(dt), then get_positions() and
    get_densities() -- host wall clock per step.  The particle set is restored before
    every step (clear_particles + add_particles_array, outside the timed interval), so
    each step uploads its inputs from the host mirror (x, v, m) inside step() and the
    getters download x, v, rho and P into the mirror and copy them out."""
    lib = REPO / "sph-particle-simulator_gb300" / "lib"
    if str(lib) not in sys.path:
        sys.path.insert(0, str(lib))
    import sph

    prm = w.params
    p = sph.SPHParameters()
    (p.rest_density, p.gas_constant, p.viscosity, p.smoothing_length, p.particle_mass,
     p.timestep, p.gravity, p.damping, p.CFL_factor) = (float(x) for x in prm[:9])
    p.bounds = [float(x) for x in prm[9:15]]
    p.neighbor_search_radius = float(prm[15])
    sim = sph.Simulator(w.n)
    sim.initialize(p)
    times = []
    for k in range(steps + 2):
        sim.clear_particles()
        sim.add_particles_array(w.pos, w.vel, w.mass)
        t0 = time.perf_counter()
        sim.step(w.dt)
        x = sim.get_positions()
        rho = sim.get_densities()
        t1 = time.perf_counter()
        if k >= 2:
            times.append(t1 - t0)
    med = statistics.median(times)
    return {"value": w.n / med, "unit": UNIT, "steps": steps, "ms_per_step_median": 1e3 * med,
            "ms_per_step_min": 1e3 * min(times), "h2d_bytes_per_step": 28 * w.n,
            "d2h_bytes_per_step": 40 * w.n,
            "rho_mean": float(np.mean(rho[: w.n])), "x_mean": float(np.mean(x)),
            "path": "sph.Simulator.step + get_positions + get_densities (pybind11 module over "
                    "the C++ drop-in SPHEngine, libsph_gb300.so -> libsphx.so)"}


def bench_precise(torch, stream, flush, w, steps):
    """A workload's fresh-state step in the precision mode (cell + FP32 offset storage, the
    tile sweeps, compensated sums, FP64 CFL and time): device time of the graph-replayed
    step, with the kernel split from an eager context with phase timers."""
    import sphx

    out = {}
    for graph in (True, False):
        ctx = sphx.Context(w.n, mode=sphx.MODE_PRECISE, graph=graph, profile=not graph)
        ctx.set_stream(stream.cuda_stream)
        ctx.set_params(w.params)
        ctx.upload(w.pos, w.vel, w.mass)
        ctx.snapshot()
        for _ in range(3):
            ctx.restore()
            ctx.step(w.dt)
        torch.cuda.synchronize()
        ctx.reset_stats()
        ms = timed_steps(torch, ctx, w, steps, flush)
        if graph:
            out.update({"value": w.n * steps / (sum(ms) * 1e-3), "unit": UNIT, "steps": steps,
                        "ms_per_step": sum(ms) / steps})
        else:
            st = ctx.stats()
            out.update({"force_kernel_ms": 1e3 * st["force_computation_time"] / steps,
                        "density_kernel_ms": 1e3 * st["density_computation_time"] / steps,
                        "grid_build_ms": 1e3 * st["neighbor_search_time"] / steps})
        ctx.close()
    out.update({"mode": "cell + FP32 offset, tile sweeps, compensated sums",
                "kernels": [PASSES["precise"]["density"], PASSES["precise"]["force"]],
                "protocol": "fresh-state, the workload's dt, captured graph; L2 flushed"})
    return out


def bench_10m_precise(torch, stream, flush, w10, steps):
    """The 10M dam break in the precision mode (cell + FP32 offset storage, compensated
    sums, FP64 CFL maximum and time, FP64 mass / energy sums every step), fresh-state steps
    with the adaptive timestep capped at 2e-4.  (A faithful multi-step trajectory of this
    configuration piles the particles into the walls on the first step -- the reference's
    dynamics -- after which every step is quadratic in the crowded cells' occupancy.)"""
    import sphx

    ctx = sphx.Context(w10.n, mode=sphx.MODE_PRECISE, graph=True)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_params(w10.params)
    ctx.upload(w10.pos, w10.vel, w10.mass)
    ctx.snapshot()
    for _ in range(3):
        ctx.restore()
        ctx.step(0.0)
    ms = timed_steps(torch, ctx, w10, steps, flush)
    st = ctx.stats()
    t, dt = ctx.time_f64()
    ctx.close()
    # the kernel split, from an eager context with phase timers (same state, same steps)
    pc = sphx.Context(w10.n, mode=sphx.MODE_PRECISE, profile=True)
    pc.set_stream(stream.cuda_stream)
    pc.set_params(w10.params)
    pc.upload(w10.pos, w10.vel, w10.mass)
    pc.snapshot()
    pc.restore()
    pc.step(0.0)
    torch.cuda.synchronize()
    pc.reset_stats()
    timed_steps(torch, pc, w10, 3, flush)
    ps = pc.stats()
    pc.close()
    f10 = ps["force_computation_time"] / 3
    return {"value": w10.n * steps / (sum(ms) * 1e-3), "unit": UNIT, "steps": steps,
            "ms_per_step": sum(ms) / steps, "mode": "cell + FP32 offset, compensated sums",
            "last_dt_s": dt, "fp64_sum_mass": st["sum_mass"],
            "fp64_energy": st["kinetic_energy"] + st["potential_energy"],
            "force_kernel_ms": 1e3 * f10,
            "density_kernel_ms": 1e3 * ps["density_computation_time"] / 3,
            "grid_build_ms": 1e3 * ps["neighbor_search_time"] / 3,
            "force_hbm_frac": (PASSES["precise"]["force_bytes"] * w10.n / f10 / 1e9) / peaks()[0],
            "kernels": [PASSES["precise"]["density"], PASSES["precise"]["force"]],
            "protocol": "fresh-state, CFL dt in FP64 (step(0)), captured graph"}


def bench_faithful(torch, stream, w, budget_s=30.0):
    """Faithful trajectory of the workload: its own step count and dt from the initial
    state, each step timed on the device, with the grid's occupancy and the non-finite
    count after every step.  The reference's dynamics pile the particles into the walls
    within the first steps (the lattice starts at 2/3 of the rest density), after which a
    step costs the square of the crowded cells' occupancy; the run stops after the step
    that crosses `budget_s` of device time and reports the steps it did."""
    import sphx

    ctx = sphx.Context(w.n, profile=False)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_params(w.params)
    ctx.upload(w.pos, w.vel, w.mass)
    torch.cuda.synchronize()
    log, total = [], 0.0
    for s in range(w.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        ctx.step(w.dt)
        e1.record()
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        st = ctx.stats()
        occ = max(st["occupied_cells"], 1)
        log.append([round(ms, 3), st["occupied_cells"], st["max_cell_occupancy"],
                    round(w.n / occ, 2), st["nonfinite_particles"]])
        total += ms * 1e-3
        if total > budget_s:
            break
    ctx.close()
    done = len(log)
    return {"value": w.n * done / total, "unit": UNIT, "steps_done": done, "steps": w.steps,
            "dt": w.dt, "device_s": total, "ms_first_step": log[0][0], "ms_last_step": log[-1][0],
            "per_step": log,
            "per_step_fields": ["ms", "occupied_cells", "max_cell_occupancy",
                                "mean_cell_occupancy", "nonfinite_particles"],
            "protocol": f"faithful trajectory from the initial state, stopped after the step "
                        f"crossing {budget_s:.0f} s of device time"}


def bench_ours(args, world, rank, local):
    import torch

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist = dist_mod
    import sphx

    w = workload(args.workload)
    # one dedicated stream carries the library's kernels, the flushes and the timing events
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    # per-phase kernel times: an eager, profiled context (events around each phase)
    mode = sphx.MODE_PRECISE if args.mode == "precise" else sphx.MODE_EXACT
    prof = sphx.Context(w.n, profile=True, mode=mode)
    prof.set_stream(stream.cuda_stream)
    prof.set_params(w.params)
    prof.upload(w.pos, w.vel, w.mass)
    prof.snapshot()
    for _ in range(max(args.warmup, 3)):
        prof.restore()
        prof.step(w.dt)
    torch.cuda.synchronize()
    prof.reset_stats()
    ms_eager = timed_steps(torch, prof, w, args.steps, flush)
    pst = prof.stats()
    prof.close()
    force_s = pst["force_computation_time"] / args.steps
    dens_s = pst["density_computation_time"] / args.steps
    grid_s = pst["neighbor_search_time"] / args.steps

    # the measured path: the step captured once as a CUDA graph and replayed
    ctx = sphx.Context(w.n, graph=True, mode=mode)
    ctx.set_stream(stream.cuda_stream)
    ctx.set_params(w.params)
    ctx.upload(w.pos, w.vel, w.mass)
    ctx.snapshot()

    # warm-up (the first step runs eagerly, the second captures the graph)
    for _ in range(max(args.warmup, 3)):
        ctx.restore()
        ctx.step(w.dt)
    torch.cuda.synchronize()
    ctx.reset_stats()
    launches0 = ctx.stats()["kernel_launches"]

    sampler = ClockSampler(local) if rank == 0 else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_wall = time.perf_counter()
    ms = timed_steps(torch, ctx, w, args.steps, flush)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    if dist:
        dist.barrier()
    clocks = sampler.stop() if sampler else None
    st = ctx.stats()
    launches = st["kernel_launches"] - launches0
    dev_s = max_over_ranks(dist, sum(ms) * 1e-3)
    value = replica_value(world, w.n, args.steps, dev_s)

    # e2e through the C ABI with pinned host buffers
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()
    h_pos, h_vel, h_mass = pin(w.pos), pin(w.vel), pin(w.mass)
    o_pos = torch.empty((w.n, 3), dtype=torch.float32).pin_memory()
    o_vel = torch.empty((w.n, 3), dtype=torch.float32).pin_memory()
    o_rho = torch.empty((w.n,), dtype=torch.float32).pin_memory()

    def e2e_step():
        ctx.upload_ptr(w.n, h_pos.data_ptr(), h_vel.data_ptr(), h_mass.data_ptr())
        ctx.step(w.dt)
        ctx.download_ptr(o_pos.data_ptr(), o_vel.data_ptr(), o_rho.data_ptr(), None, None)

    e2e_step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    # each step timed from its upload to the host's return from the download (the L2
    # flush before it is outside the step's interval)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    for e0, e1 in evs:
        flush.fill_(1)
        e0.record()
        e2e_step()
        e1.record()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(dist, sum(e0.elapsed_time(e1) for e0, e1 in evs) * 1e-3)
    e2e_value = replica_value(world, w.n, args.steps, e2e_s)
    # parity spot-check of the e2e output against the device path (same initial state)
    rho_e2e = o_rho.numpy().copy()

    # secondary workloads (device-timed): the 10M dam break and the batched scene mix
    extra = {}
    rho_batched = None
    if not args.no_dropin:
        ctx.close()
        extra["e2e_dropin"] = bench_dropin(w, max(3, min(args.steps, 10)))
    if args.workload == "dam_break_1M" and not args.no_batch:
        ctx.close()
        extra["batched_256"], rho_batched = bench_batched(torch, stream, flush,
                                                          max(3, min(args.steps, 10)))
    if args.workload == "dam_break_1M" and args.mode == "exact":
        if not ctx_closed(ctx):
            ctx.close()
        extra["dam_break_1M_precise"] = bench_precise(torch, stream, flush, w,
                                                      max(3, min(args.steps, 10)))
    if args.workload == "dam_break_1M" and not args.no_10m:
        w10 = workload("dam_break_10M")
        ctx.close()
        ctx10 = sphx.Context(w10.n, profile=True)
        ctx10.set_stream(stream.cuda_stream)
        ctx10.set_params(w10.params)
        ctx10.upload(w10.pos, w10.vel, w10.mass)
        ctx10.snapshot()
        for _ in range(3):
            ctx10.restore()
            ctx10.step(w10.dt)
        torch.cuda.synchronize()
        ctx10.reset_stats()
        k10 = max(3, min(args.steps, 10))
        ms10 = timed_steps(torch, ctx10, w10, k10, flush)
        st10 = ctx10.stats()
        f10 = st10["force_computation_time"] / k10
        extra["dam_break_10M"] = {
            "value": w10.n * k10 / (sum(ms10) * 1e-3), "unit": UNIT, "steps": k10,
            "ms_per_step": sum(ms10) / k10, "protocol": "fresh-state, CFL dt (step(0)), exact mode",
            "force_kernel_ms": 1e3 * f10,
            "density_kernel_ms": 1e3 * st10["density_computation_time"] / k10,
            "grid_build_ms": 1e3 * st10["neighbor_search_time"] / k10,
            "force_hbm_frac": (FORCE_BYTES_PER_PARTICLE * w10.n / f10 / 1e9) / peaks()[0],
        }
        ctx10.close()
        extra["dam_break_10M_precise"] = bench_10m_precise(torch, stream, flush, w10, k10)
        extra["dam_break_10M_trajectory"] = bench_10m_trajectory(torch, stream, w10)
    elif not ctx_closed(ctx):
        ctx.close()
    if args.workload == "dam_break_1M" and not args.no_faithful:
        if not ctx_closed(ctx):
            ctx.close()
        extra["dam_break_1M_faithful"] = bench_faithful(torch, stream, w)

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0

    peak, peak_kind = peaks()
    ps = PASSES[args.mode]
    achieved = ps["force_bytes"] * w.n / force_s / 1e9
    # the bound that applies: instruction issue (the passes do ~8 FP32 ops per candidate
    # test and ~150 per exact pair term on L1/L2-resident data)
    sm_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(local).multi_processor_count or SM_COUNT_FALLBACK
    issue_peak = sms * ISSUE_PER_SM_PER_CLK * sm_mhz * 1e6
    issue = None
    ipp = ncu_issue(ps["issue_force"])
    if ipp:
        a_issue = ipp * w.n / force_s
        issue = {"bound": "issue", "achieved": a_issue, "peak": issue_peak,
                 "unit": "warp-inst/s", "frac": a_issue / issue_peak,
                 "kernel": ps["force"],
                 "source": "profiles/ncu_issue.json warp instructions per particle x particles "
                           "/ CUDA-event kernel time; peak = SMs x 4 issue slots x median SM clock"}
        ipd = ncu_issue(ps["issue_density"])
        if ipd:
            issue["density_frac"] = ipd * w.n / dens_s / issue_peak
    traffic, traffic_masks = ncu_traffic(ps["traffic"], w.n)
    cpu = None
    if world == 1 and not args.no_cpu:
        cpu = run_cpu(w, steps=8, warmup=0, budget_s=15.0)
        if rho_batched is not None:  # the oracle as the checker of the batched densities
            import sph_oracle as O

            extra["batched_256"].update(batched_fp64_check(O.Port(), rho_batched))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": 1e3 * dev_s / args.steps,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / PUBLISHED_1M if args.workload == "dam_break_1M" else None,
        "dtype": "f32", "data": "synthetic",
        "config": workload_config(w, args.workload, world, args.mode),
        "launch": "step captured as a CUDA graph and replayed (sphx_tuning.graph); "
                  "eager launches: %.4f ms/step" % (sum(ms_eager) / args.steps),
        "vs_baseline_ref": "README.md:45 CPU 1M 38 steps/s = 3.8e7 particle-steps/s",
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 28 * w.n,
                "d2h_bytes_per_step": 28 * w.n,
                "path": "sphx_upload (pinned) + sphx_step + sphx_download (pos, vel, rho)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_hit_masks": traffic_masks,
                     "traffic_note": ("DRAM bytes per launch = the particle data (%.1fx the "
                                      "%d B/particle algorithmic bytes) + the hit-mask records "
                                      "the density pass wrote for this pass (read once)"
                                      % ((traffic - traffic_masks) / (ps["force_bytes"] * w.n),
                                         ps["force_bytes"])) if traffic and traffic_masks else
                                     ("DRAM bytes per launch = %.1fx the %d B/particle "
                                      "algorithmic bytes (no hit-mask records in this mode)"
                                      % (traffic / (ps["force_bytes"] * w.n), ps["force_bytes"])
                                      if traffic else None),
                     "kernel": ps["force"],
                     "peak_source": f"{peak_kind} hbm_gbs"},
        "roofline_issue": issue,
        "kernels_ms": {"grid_build": 1e3 * grid_s, "density": 1e3 * dens_s,
                       "force": 1e3 * force_s, "density_kernel": ps["density"],
                       "density_hbm_frac": (ps["density_bytes"] * w.n / dens_s / 1e9) / peak},
        "gpu_launches": launches,
        "clocks": clocks,
        "cpu_baseline": cpu and {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
        "wall_s_timed_region": t_wall,
        "rho_e2e_mean": float(np.mean(rho_e2e)),
    }
    line.update(extra)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", default="dam_break_1M",
                    choices=("dam_break_10k", "dam_break_1M", "dam_break_4M", "dam_break_10M"))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-10m", action="store_true", help="skip the 10M secondary figures")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched-scene figure")
    ap.add_argument("--no-faithful", action="store_true",
                    help="skip the faithful-trajectory figure")
    ap.add_argument("--mode", choices=("exact", "precise"), default="exact",
                    help="the main workload's mode (precise: cell + offset storage, fast "
                         "pair arithmetic, compensated sums)")
    ap.add_argument("--no-dropin", action="store_true",
                    help="skip the drop-in engine's end-to-end figure")
    args = ap.parse_args()
    world, rank, local = dist_env()
    if args.impl == "reference":
        return bench_reference(args, world, rank)
    return bench_ours(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())
