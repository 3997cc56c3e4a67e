"""Benchmark of the fused collide-and-stream pull step on GB300.

Default workload (the one the headline metric is quoted on): D3Q27 entropic
SRT, FP32 population storage, 512^3 periodic lattice, beta = 0.9995, initial
field = Taylor-Green vortex (U0 = 0.05) + random-phase solenoidal
perturbation of amplitude 1e-3 on the shell 8 <= |k| <= 10 (seed 2). Every
node solves for alpha in FP64 to |F(alpha)| <= 1e-12 (bisection-Newton
fallback). Two arms run on the same GPU from the same state: the learned
alpha guess (the committed MLP) and plain Newton from the previous alpha.
`value` is the learned arm's MLUPS; the Newton arm is reported beside it.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
       [--workload entropic_learned_512|bgk_d3q19_f64_256|bgk_d3q19_f32_256|bgk_d3q19_f16_256]
Under torchrun (N > 1) every rank runs an independent replica of the workload
on its own GPU (the path has no data exchange on one lattice per GPU); the
timed region is bracketed by barriers and the max over ranks is used.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "D3Q27 entropic MLUPS, learned-α vs Newton-α on 1 GB300 at equal H-residual; %HBM"


def metric_for(name: str) -> str:
    """The headline metric for the default workload; the others are named by
    what they run (same unit: million lattice updates per second)."""
    if name == "entropic_learned_512":
        return METRIC
    w = WORKLOADS[name]
    force = w.get("forceT", "None")
    return (f"{w['latticeT']} {w['collisionT']} {w['storage'].upper()} MLUPS, "
            f"{w.get('forcingSchemeT', 'None')} forcing, {force} force")
BETA = 0.9995
TAU = 1.0 / (2.0 * BETA)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ---------------------------------------------------------------------------
# workloads
WORKLOADS = {
    "entropic_learned_512": dict(latticeT="D3Q27", collisionT="ELBM", relaxationTime=TAU,
                                 globalLength=(512, 512, 512), storage="f32",
                                 alphaSolver="residual", newtonTolerance=1e-12,
                                 deviationThreshold=0.0, bytes_per_node=2 * 27 * 4 + 8),
    "bgk_d3q19_f64_256": dict(latticeT="D3Q19", collisionT="BGK", relaxationTime=0.55,
                              forcingSchemeT="Guo", forceT="Kolmogorov",
                              forceAmplitude=(1e-6, 0.0, 0.0), forceWaveLength=(128.0, 1.0, 1.0),
                              kolmogorovAxis=2, globalLength=(256, 256, 256), storage="f64",
                              bytes_per_node=2 * 19 * 8),
    # the same with the fixed-point FP64 collision (exact integer moments and
    # equilibrium on the integer pipe, the update rounded once to FP64)
    "bgk_d3q19_f64_fixed_256": dict(latticeT="D3Q19", collisionT="BGK", relaxationTime=0.55,
                                    forcingSchemeT="Guo", forceT="Kolmogorov",
                                    forceAmplitude=(1e-6, 0.0, 0.0),
                                    forceWaveLength=(128.0, 1.0, 1.0), kolmogorovAxis=2,
                                    globalLength=(256, 256, 256), storage="f64",
                                    fp64Arithmetic="fixed", bytes_per_node=2 * 19 * 8),
    "bgk_d3q19_f32_256": dict(latticeT="D3Q19", collisionT="BGK", relaxationTime=0.55,
                              forcingSchemeT="Guo", forceT="Kolmogorov",
                              forceAmplitude=(1e-6, 0.0, 0.0), forceWaveLength=(128.0, 1.0, 1.0),
                              kolmogorovAxis=2, globalLength=(256, 256, 256), storage="f32",
                              bytes_per_node=2 * 19 * 4),
    "bgk_d3q19_f16_256": dict(latticeT="D3Q19", collisionT="BGK", relaxationTime=0.55,
                              forcingSchemeT="Guo", forceT="Kolmogorov",
                              forceAmplitude=(1e-6, 0.0, 0.0), forceWaveLength=(128.0, 1.0, 1.0),
                              kolmogorovAxis=2, globalLength=(256, 256, 256),
                              storage="f16_shifted", bytes_per_node=2 * 19 * 2),
    # the 3-D production deck's lattice and scheme (Input_prod_3d.in: D3Q27, BGK,
    # exact-difference forcing) with the time-dependent spectral force: the
    # force field from two batched FFTs and a shell filter before every step
    "turbulent_d3q27_f64_256": dict(latticeT="D3Q27", collisionT="BGK", relaxationTime=0.55,
                                    forcingSchemeT="ExactDifferenceMethod", forceT="Turbulent2D",
                                    forceAmplitude=(1e-6, 1e-6, 1e-6), forcekMin=1, forcekMax=2,
                                    removalForceAmplitude=(1e-6, 1e-6, 1e-6), removalForcekMin=1,
                                    removalForcekMax=2, globalLength=(256, 256, 256),
                                    storage="f64", bytes_per_node=2 * 27 * 8 + 3 * 8),
    "turbulent_d3q27_f32_256": dict(latticeT="D3Q27", collisionT="BGK", relaxationTime=0.55,
                                    forcingSchemeT="ExactDifferenceMethod", forceT="Turbulent2D",
                                    forceAmplitude=(1e-6, 1e-6, 1e-6), forcekMin=1, forcekMax=2,
                                    removalForceAmplitude=(1e-6, 1e-6, 1e-6), removalForcekMin=1,
                                    removalForcekMax=2, globalLength=(256, 256, 256),
                                    storage="f32", bytes_per_node=2 * 27 * 4 + 3 * 4),
}

SPECTRAL_FORCES = ("ConstantShell", "EnergyRemoval", "Turbulent2D")


def initial_field(name: str, shape):
    from metalbm_gb300 import fields
    if name.startswith("entropic"):
        rho, u = fields.taylor_green(shape, u0=0.05)
        u = u + fields.solenoidal_shell(shape, 8.0, 10.0, 1e-3, seed=2)
        return rho, u
    return fields.perturbed_rest(shape, 3, 1e-4, seed=1)


def arithmetic_of(name: str) -> str:
    """What the workload computes in, beside its storage type (`dtype`)."""
    w = WORKLOADS[name]
    if w["collisionT"] != "BGK":
        return ("populations stored and updated in FP32; f_neq, B1 and M2 of the entropy "
                "function in double-float FP32, its evaluation and the alpha solve in FP64")
    if w.get("fp64Arithmetic") == "fixed":
        return ("FP64 storage; moments, equilibrium and update in 64-bit fixed point on the "
                "integer pipe, rounded once to FP64")
    return {"f64": "FP64 (the reference's operation order)",
            "f32": "FP32 storage and collision (deviations from the weights)",
            "f16_shifted": "FP16 storage of (f - w) 2^k, FP32 collision"}[w["storage"]]


def deck_for(name: str, **over):
    from metalbm_gb300 import InputDeck
    w = {k: v for k, v in WORKLOADS[name].items() if k != "bytes_per_node"}
    w.update(over)
    return InputDeck(**w)


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self) -> dict:
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The slowest rank's time: the timed region of every replica is
    bracketed by barriers, and the job's time is the max over ranks."""
    if dist is None:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(nodes_per_rank: int, steps: int, world: int, max_ms: float) -> float:
    """Whole-job MLUPS: every rank advances its own replica of `nodes_per_rank`
    nodes by `steps` steps; the job takes the slowest rank's time."""
    return world * nodes_per_rank * steps / (max_ms * 1e-3) / 1e6


def time_steps(lat, steps: int, torch, dist=None, store_each: bool = False):
    """Time one mlbm_step call of `steps` steps with CUDA events on the
    handle's stream (so the solver counters cover exactly the timed steps);
    with store_each, one storing call per step instead. Returns (total ms,
    launches of the library's kernels in the region)."""
    from metalbm_gb300.lattice import kernel_launch_count
    stream = torch.cuda.ExternalStream(lat.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    lat.sync()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    n0 = kernel_launch_count()
    e0.record(stream)
    if store_each:
        for _ in range(steps):
            lat.step(1, store=True)
    else:
        lat.step(steps)
    e1.record(stream)
    lat.sync()
    torch.cuda.synchronize()
    launches = kernel_launch_count() - n0
    if dist is not None:
        dist.barrier()
    return e0.elapsed_time(e1), launches


def time_steps_perfect_guess(lat, steps: int, torch, dist=None):
    """The perfect-guess bound of the alpha solve: before each timed step an
    untimed trial step from the same populations (mlbm_testing_step_in_place)
    leaves every node's solved alpha in the alpha field, so the timed step
    (previous-alpha guess) starts each node from its root. Returns (total ms
    of the timed steps, summed solver counters of the timed steps)."""
    stream = torch.cuda.ExternalStream(lat.stream)
    lib = lat._lib
    lat.sync()
    if dist is not None:
        dist.barrier()
    torch.cuda.synchronize()
    total, sums = 0.0, {}
    for _ in range(steps):
        lat._check(lib.mlbm_testing_step_in_place(lat.handle))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        lat.step(1)
        e1.record(stream)
        d = lat.diagnostics()  # synchronizes
        total += e0.elapsed_time(e1)
        for k in ("solved_nodes", "newton_iterations", "guess_hits", "bisection_nodes",
                  "fallback_nodes", "series_nodes", "learned_nodes"):
            sums[k] = sums.get(k, 0) + d[k]
    torch.cuda.synchronize()
    if dist is not None:
        dist.barrier()
    return total, sums


def solver_stats(d: dict) -> dict:
    """Per-solved-node statistics of the alpha solve over the timed steps."""
    solved = max(d["solved_nodes"], 1)
    return {"newton_iterations_per_solved_node": d["newton_iterations"] / solved,
            "guess_hit_fraction": d["guess_hits"] / solved,
            "fallback_fraction": 1.0 - d["guess_hits"] / solved,
            "bisection_nodes": d["bisection_nodes"], "alpha2_fallback_nodes": d["fallback_nodes"],
            "series_form_fraction": d["series_nodes"] / solved,
            "network_guess_fraction": d.get("learned_nodes", 0) / solved}


def load_or_train_model(deck, torch):
    from metalbm_gb300 import alpha_model, fields
    path = alpha_model.default_model_path(deck.latticeT)
    if path.exists():
        return alpha_model.load_model(path), str(path.relative_to(ROOT))
    # no committed model: train a small one from a plain run (untimed setup)
    shape = (64, 64, 64)
    rho, u = fields.taylor_green(shape, u0=0.05)
    small = deck_for("entropic_learned_512", globalLength=shape, alphaGuess="two")
    X, y = alpha_model.collect_samples(small, rho, u, steps=100, every=25, n_per_log=100000)
    model, _ = alpha_model.fit(X, y, small, epochs=20)
    return model, "trained in bench setup (64^3, 100 steps)"


class PortRun:
    """The oracle port on a sample of a workload. Spectral forces: the force
    field restated with numpy FFTs before every step from the stored fields,
    which stay the initial ones (no step stores, as in the timed GPU steps)."""

    def __init__(self, name: str, shape, threads: int, alpha: str = "workload", fields=None):
        """alpha: "workload" solves alpha as the GPU arm does (the residual
        solver at the workload's tolerance), "reference" with the reference's
        Newton (tolerance 1e-8, alpha = 2 fallback, deviation shortcut 1e-3)."""
        from oracle import ALPHA_REFERENCE, ALPHA_RESIDUAL, OracleConfig, OraclePort
        w = WORKLOADS[name]
        self.w, self.shape = w, shape
        self.spectral = w.get("forceT") in SPECTRAL_FORCES
        self.rho, self.u = fields if fields is not None else initial_field(name, shape)
        solver = {}
        if w["collisionT"] != "BGK" and alpha == "workload":
            solver = dict(alpha_mode=ALPHA_RESIDUAL, newton_tolerance=w["newtonTolerance"],
                          deviation_threshold=w["deviationThreshold"])
        elif w["collisionT"] != "BGK":
            solver = dict(alpha_mode=ALPHA_REFERENCE)
        cfg = OracleConfig(lattice=w["latticeT"],
                           collision="ELBM" if w["collisionT"] != "BGK" else "BGK",
                           forcing=w.get("forcingSchemeT", "None"),
                           force="Field" if self.spectral else w.get("forceT", "None"),
                           tau=w["relaxationTime"], amplitude=w.get("forceAmplitude", (0, 0, 0)),
                           wavelength=w.get("forceWaveLength", (1, 1, 1)),
                           kolmogorov_axis=w.get("kolmogorovAxis", 1), size=shape,
                           threads=threads, **solver)
        self.port = OraclePort(cfg)
        self.port.init_equilibrium(self.rho, self.u)

    def close(self):
        self.port.close()

    def step(self, n: int):
        if not self.spectral:
            self.port.step(n, store_last=False)
            return
        from oracle import spectral_force as sf
        w, D = self.w, 3
        for _ in range(n):
            if w["forceT"] == "ConstantShell":
                F = sf.constant_shell_field(self.shape, D, w["forceAmplitude"], w["forcekMin"],
                                            w["forcekMax"])
            elif w["forceT"] == "EnergyRemoval":  # the force parameters (Algorithm.h:90-91)
                F = sf.energy_removal_field(self.rho, self.u, self.shape, D, w["forceAmplitude"],
                                            w["forcekMin"], w["forcekMax"])
            else:
                F = sf.turbulent_field(self.rho, self.u, self.shape, D, w["forceAmplitude"],
                                       w["forcekMin"], w["forcekMax"],
                                       w["removalForceAmplitude"], w["removalForcekMin"],
                                       w["removalForcekMax"])
            self.port.set_force_field(F)
            self.port.step(1, store_last=False)


# The reference CPU path's grid per workload: the workload's own, except the
# 512^3 entropic one, whose 25 steps at the CPU path's ~5-10 MLUPS on 16 host
# cores would take ~10 minutes; it runs the same construction on 256^3.
REFERENCE_GRID = {"entropic_learned_512": (256, 256, 256)}


def reference_shape(name: str, grid: int = 0):
    if grid:
        return (grid,) * 3
    return REFERENCE_GRID.get(name, tuple(WORKLOADS[name]["globalLength"]))


def reference_differences(name: str, shape) -> list[str]:
    """Why the reference arm's configuration is not the GPU arm's (empty when
    it is)."""
    w = WORKLOADS[name]
    out = []
    if tuple(shape) != tuple(w["globalLength"]):
        out.append(f"grid {'x'.join(map(str, shape))} instead of "
                   f"{'x'.join(map(str, w['globalLength']))} (the CPU path's time)")
    if w["storage"] != "f64":
        out.append(f"FP64 populations (the reference has no {w['storage']} storage)")
    return out


def solver_words(name: str, alpha: str = "workload") -> str:
    w = WORKLOADS[name]
    if w["collisionT"] == "BGK":
        return "BGK"
    if alpha == "workload":
        return (f"entropic, residual alpha solver |F| <= {w['newtonTolerance']:g} (the GPU arm's "
                "solver)")
    return "entropic, reference alpha solver (Newton to 1e-8, alpha = 2 fallback)"


def cpu_baseline_port(name: str, shape, threads: int, fields=None,
                      seconds_budget: float = 20.0) -> dict:
    """The oracle port (C restatement of the reference path) on the host
    cores, on the workload's own grid and initial field with the GPU arm's
    alpha solver: one warm-up step, then steps until about `seconds_budget`
    seconds (a bounded sample of the workload)."""
    w = WORKLOADS[name]
    run = PortRun(name, shape, threads, fields=fields)
    run.step(1)
    steps, t0 = 0, time.perf_counter()
    while True:
        run.step(1)
        steps += 1
        dt = time.perf_counter() - t0
        if dt > seconds_budget or steps >= 50:
            break
    run.close()
    V = int(np.prod(shape))
    extra = ", force field by numpy FFTs each step (1 thread)" if run.spectral else ""
    return {"value": V * steps / dt / 1e6, "unit": "MLUPS", "cores": threads, "kind": "port",
            "sample": f"{w['latticeT']} FP64 {solver_words(name)}, the workload's "
                      f"{'x'.join(map(str, shape))} grid and initial field, {steps} steps after "
                      f"1 warm-up, {threads} threads{extra}"}


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    import torch.distributed as dist_mod
    from metalbm_gb300 import Lattice, build
    from metalbm_gb300.lattice import kernel_launch_count

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        torch.cuda.set_device(local)
        dist_mod.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist = dist_mod
    if rank == 0:
        build.build()
    if dist is not None:
        dist.barrier()
    name = args.workload
    w = WORKLOADS[name]
    grid_over = {"globalLength": (args.grid,) * 3} if args.grid else {}
    deck = deck_for(name, device=local, **grid_over)
    shape = deck.shape
    V = int(np.prod(shape))
    rho, u = initial_field(name, shape)
    entropic = w["collisionT"] != "BGK"
    extra = {}

    # --- arm 1: the learned guess (or the only arm for BGK workloads)
    if entropic:
        model, model_src = load_or_train_model(deck, torch)
        deck_l = deck_for(name, device=local, alphaGuess="learned", **grid_over)
    else:
        deck_l = deck
    lat = Lattice(deck_l)
    if entropic:
        lat.set_alpha_model(model)
    lat.init_equilibrium(rho, u)
    lat.step(args.warmup)
    # time-dependent spectral forces: fields stored every step, so the force
    # is recomputed from them before every step (the reference's isStored
    # path on every iteration)
    store_each = w.get("forceT") in ("EnergyRemoval", "Turbulent2D")
    with ClockSampler(local) as clk:
        total_ms, launches = time_steps(lat, args.steps, torch, dist, store_each)
    dl = lat.diagnostics()
    lat.close()
    total_ms = max_over_ranks(total_ms, dist, f"cuda:{local}")

    # --- the other arms, same initial state, same residual tolerance, same
    # GPU: plain Newton from the previous step's alpha (the reference's guess,
    # Algorithm.h:103-106) and from alpha = 2, the network at every node, and
    # the perfect-guess bound (every node starts from its root)
    if entropic:
        value_l = job_value(V, args.steps, world, total_ms)
        arms = {}
        for guess in ("previous", "two", "learned_everywhere"):
            lat = Lattice(deck_for(name, device=local, alphaGuess=guess, **grid_over))
            if guess.startswith("learned"):
                lat.set_alpha_model(model)
            lat.init_equilibrium(rho, u)
            lat.step(args.warmup)
            ms, _ = time_steps(lat, args.steps, torch, dist)
            d = lat.diagnostics()
            lat.close()
            ms = max_over_ranks(ms, dist, f"cuda:{local}")
            arms[guess] = {"value": job_value(V, args.steps, world, ms), "unit": "MLUPS",
                           "ms_per_step": ms / args.steps, **solver_stats(d)}
        lat = Lattice(deck_for(name, device=local, alphaGuess="previous", **grid_over))
        lat.init_equilibrium(rho, u)
        lat.step(args.warmup)
        ms, sums = time_steps_perfect_guess(lat, args.steps, torch, dist)
        lat.close()
        ms = max_over_ranks(ms, dist, f"cuda:{local}")
        arms["perfect"] = {"value": job_value(V, args.steps, world, ms), "unit": "MLUPS",
                           "ms_per_step": ms / args.steps, **solver_stats(sums),
                           "what": "every timed step preceded by an untimed trial step from "
                                   "the same populations (mlbm_testing_step_in_place), so each "
                                   "node's guess is its solved alpha (to the FP32 alpha field's "
                                   "precision, alpha - 2 in float)"}
        # the first step from the initial state (alpha = 2 stored everywhere):
        # the network guess against the constant 2 the reference starts from
        cold = {}
        for guess in ("learned", "two"):
            lat = Lattice(deck_for(name, device=local, alphaGuess=guess, **grid_over))
            if guess == "learned":
                lat.set_alpha_model(model)
            lat.init_equilibrium(rho, u)
            lat.step(1)
            cold[guess] = solver_stats(lat.diagnostics())
            lat.close()
        sl = solver_stats(dl)
        extra = {
            "newton_alpha": arms["previous"],
            "newton_alpha_from_2": arms["two"],
            "learned_alpha": {**sl, "model": model_src,
                              "guess": "the network where a node has no solved alpha from the "
                                       "previous step (stored alpha exactly 2), the previous "
                                       "alpha elsewhere"},
            "learned_alpha_everywhere": {**arms["learned_everywhere"],
                                         "guess": "the network at every solved node"},
            "perfect_guess": arms["perfect"],
            "speedup_learned_vs_newton": value_l / arms["previous"]["value"],
            "speedup_learned_vs_newton_from_2": value_l / arms["two"]["value"],
            "speedup_learned_everywhere_vs_newton":
                arms["learned_everywhere"]["value"] / arms["previous"]["value"],
            "speedup_perfect_guess_vs_newton": arms["perfect"]["value"] / arms["previous"]["value"],
            "first_step_from_initial_state": {
                "learned": cold["learned"], "alpha_2": cold["two"],
                "what": "one step after mlbm_init_equilibrium (alpha = 2 stored everywhere): "
                        "the network guess at every node against the reference's constant 2"},
            "newton_iterations_saved_per_solved_node": {
                "vs_previous_alpha": arms["previous"]["newton_iterations_per_solved_node"]
                - sl["newton_iterations_per_solved_node"],
                "vs_alpha_2": arms["two"]["newton_iterations_per_solved_node"]
                - sl["newton_iterations_per_solved_node"]},
            "residual_tolerance": deck.newtonTolerance,
            "solver_stats_over": f"the {args.steps} timed steps",
        }

    # --- spectral workloads: the same step kernel with the time-independent
    # ConstantShell field (no per-step transforms) times the kernel alone;
    # the difference is the per-step force update (momentum, D2Z, filter, Z2D)
    kernel_ms = total_ms
    if w.get("forceT") in SPECTRAL_FORCES and w["forceT"] != "ConstantShell":
        lat = Lattice(deck_for(name, device=local, forceT="ConstantShell", **grid_over))
        lat.init_equilibrium(rho, u)
        lat.step(args.warmup)
        kernel_ms, _ = time_steps(lat, args.steps, torch, dist, store_each)
        lat.close()
        kernel_ms = max_over_ranks(kernel_ms, dist, f"cuda:{local}")
        extra["spectral_force"] = {
            "force": w["forceT"],
            "step_kernel_ms": kernel_ms / args.steps,
            "force_update_ms": (total_ms - kernel_ms) / args.steps,
            "what": "fields stored every step, so the force is recomputed before every "
                    "step; step_kernel_ms: the same storing steps with the time-independent "
                    "ConstantShell field; force_update_ms = ms_per_step - step_kernel_ms "
                    "(separable partial transforms of the removal shell, 6 kernels)"}

    value = job_value(V, args.steps, world, total_ms)
    pop_gb = V * {"D2Q9": 9, "D3Q19": 19, "D3Q27": 27}[deck.latticeT] * \
        {"f64": 8, "f32": 4, "f16_shifted": 2}[deck.storage] * 2 / 1e9
    peaks, peak_src = measured_peaks()
    bpn = w["bytes_per_node"]
    avg_launch_ms = kernel_ms / args.steps
    achieved = bpn * V / (avg_launch_ms * 1e-3) / 1e9
    # ncu figures of the dominant kernel (profiles/roofline_inputs.json, each
    # entry naming the profile summary it comes from): DRAM bytes per node of
    # one launch and, for the FP64-bound kernels, FP64 instructions per node
    prof = {}
    pfile = ROOT / "profiles" / "roofline_inputs.json"
    if pfile.exists():
        prof = json.loads(pfile.read_text()).get(name, {})
    traffic = prof["dram_bytes_per_node"] * V if "dram_bytes_per_node" in prof else None
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs, burst copy)"
                if peak_src == "measured" else "fallback 6.8 TB/s",
                "bytes_per_node": bpn, "kernel": "elbm_lowp_kernel" if entropic else
                (("bgk_f64x_kernel" if w.get("fp64Arithmetic") == "fixed" else "bgk_f64_kernel")
                 if w["storage"] == "f64" else
                 ("bgk_f16_pair_kernel" if w["storage"].startswith("f16") and deck_l.shape[2] % 2 == 0
                  else "bgk_lowp_kernel")),
                "traffic_source": prof.get("source")}
    if "fp64_inst_per_node" in prof:
        # the kernel's binding roof: GB300's FP64 pipe (no FP64 figure in
        # MEASURED_PEAKS.json; the peak is the DFMA rate of a throughput
        # probe on a GB300, profiles/fp64_throughput_gb300.md)
        gops = prof["fp64_inst_per_node"] * V / (avg_launch_ms * 1e-3) / 1e9
        roofline["fp64_pipe"] = {"achieved": gops, "peak": prof["fp64_peak_gops"],
                                 "unit": "G FP64 instr/s", "frac": gops / prof["fp64_peak_gops"],
                                 "instructions_per_node": prof["fp64_inst_per_node"],
                                 "peak_source": "measured DFMA throughput (profiles/fp64_throughput_gb300.md)"}
    if "limiter" in prof:
        roofline["limiter"] = prof["limiter"]
    if "fp64_pipe_busy_pct" in prof:
        # ncu's FP64-pipe occupancy also counts the compares, conversions
        # and reciprocal seeds that run on the pipe besides the arithmetic
        roofline.setdefault("fp64_pipe", {})["pipe_busy_ncu"] = prof["fp64_pipe_busy_pct"] / 100.0

    # --- end to end through the C ABI with host buffers (rank 0 reports)
    e2e = run_e2e(name, deck_l, rho, u, model if entropic else None, args.steps, args.warmup, torch,
                  dist, world)

    # the BGK kernels of the other workloads, device-timed in the same run
    # (their own lines come from --workload NAME)
    others = {}
    if name == "entropic_learned_512" and not args.grid and not args.no_others:
        for oname in ("bgk_d3q19_f64_256", "bgk_d3q19_f64_fixed_256", "bgk_d3q19_f32_256",
                      "bgk_d3q19_f16_256"):
            others[oname] = quick_workload(oname, local, torch, dist, world, peaks)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        # the reference arm's sample: its grid, initial field and alpha solver
        rshape = reference_shape(name, args.grid)
        cpu = cpu_baseline_port(name, rshape, os.cpu_count() or 1,
                                fields=(rho, u) if tuple(rshape) == tuple(shape) else None)

    if rank == 0:
        line = {
            "metric": metric_for(name), "value": value, "unit": "MLUPS", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"f64": "f64", "f32": "f32", "f16_shifted": "f16"}[w["storage"]],
            "data": "synthetic (Taylor-Green + seeded solenoidal perturbation)" if entropic
                    else "synthetic (seeded uniform velocity perturbation)",
            "config": {"workload": name, "lattice": deck.latticeT, "collision": deck.collisionT,
                       "storage": deck.storage, "arithmetic": arithmetic_of(name),
                       "grid": list(shape), "beta": 1 / (2 * deck.relaxationTime),
                       "alpha_solver": deck.alphaSolver if entropic else None,
                       "parallelism": f"replicas x{world}",
                       "l2": f"populations {pop_gb:.1f} GB read and written per step > 129 MB L2, "
                             "no flush needed"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clk.summary(), **extra,
        }
        if others:
            line["other_workloads"] = others
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def quick_workload(name, local, torch, dist, world, peaks, steps=10, warmup=3):
    """A BGK workload device-timed as in its own run (warm-up, then `steps`
    steps of one mlbm_step call between CUDA events), for the default line."""
    from metalbm_gb300 import Lattice
    w = WORKLOADS[name]
    deck = deck_for(name, device=local)
    V = int(np.prod(deck.shape))
    rho, u = initial_field(name, deck.shape)
    with Lattice(deck) as lat:
        lat.init_equilibrium(rho, u)
        lat.step(warmup)
        ms, _ = time_steps(lat, steps, torch, dist)
    ms = max_over_ranks(ms, dist, f"cuda:{local}")
    value = job_value(V, steps, world, ms)
    gbs = w["bytes_per_node"] * V * steps / (ms * 1e-3) / 1e9  # one GPU's lattice
    return {"value": value, "unit": "MLUPS", "ms_per_step": ms / steps, "steps": steps,
            "warmup": warmup, "arithmetic": arithmetic_of(name),
            "hbm": {"achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": gbs / peaks["hbm_gbs"], "bytes_per_node": w["bytes_per_node"]}}


def run_e2e(name, deck, rho, u, model, steps, warmup, torch, dist, world):
    """Whole job through the public C ABI from page-locked host memory
    (metalbm_gb300.hostbuf). `e2e`: the initial rho/u uploaded from the host
    (mlbm_init_equilibrium, H2D), then per step mlbm_step(DIAGNOSTICS) and
    mlbm_get_diagnostics (D2H: the step's energy, mass, max Mach, alpha range
    and solver counters), and the final fields rho, u read back
    (mlbm_get_fields, D2H). `fields_every_step`: the same with the fields read
    back after every step (the reference's isStored path on every step). Each
    sequence runs once untimed first, as an application's first pass over
    freshly registered buffers would."""
    from metalbm_gb300 import Lattice
    from metalbm_gb300.hostbuf import pinned_array as pin
    V = rho.size
    D = u.shape[0]
    h_rho, h_u = pin((V,)), pin((D, V))
    h_rho[:] = rho
    h_u[:] = u
    o_rho, o_u = pin((V,)), pin((D, V))
    lat = Lattice(deck)
    if model is not None:
        lat.set_alpha_model(model)

    def read_fields():
        lat._check(lat._lib.mlbm_get_fields(lat.handle, o_rho.ctypes.data_as(_dp()),
                                            o_u.ctypes.data_as(_dp()), None, None, 0))

    def job(n, fields_each_step):
        lat.init_equilibrium(h_rho, h_u)
        for i in range(n):
            last = i == n - 1
            lat.step(1, store=fields_each_step or last, diagnostics=True)
            lat.diagnostics()
            if fields_each_step or last:
                read_fields()
        lat.sync()

    out = {}
    for key, each in (("e2e", False), ("fields_every_step", True)):
        job(warmup, each)
        if dist is not None:
            dist.barrier()
        t0 = time.perf_counter()
        job(steps, each)
        dt = time.perf_counter() - t0
        dt = max_over_ranks(dt, dist, torch.device("cuda", torch.cuda.current_device()))
        out[key] = (world * V * steps / dt / 1e6, dt)
    lat.close()
    h2d = (1 + D) * V * 8
    fields = (1 + D) * V * 8
    diag = 160
    value, _ = out["e2e"]
    return {"value": value, "unit": "MLUPS",
            "h2d_bytes_per_step": h2d // steps,
            "d2h_bytes_per_step": (fields + diag * steps) // steps,
            "what": "mlbm_init_equilibrium from page-locked host rho/u, then per step "
                    "mlbm_step(DIAGNOSTICS) + mlbm_get_diagnostics, and mlbm_get_fields(rho, u) "
                    "after the last step; the same sequence once untimed before",
            "fields_every_step": {"value": out["fields_every_step"][0], "unit": "MLUPS",
                                  "d2h_bytes_per_step": fields + diag,
                                  "what": "as e2e with mlbm_step(STORE_FIELDS|DIAGNOSTICS) + "
                                          "mlbm_get_fields(rho, u) after every step"}}


def _dp():
    import ctypes
    return ctypes.POINTER(ctypes.c_double)


# ---------------------------------------------------------------------------
def run_reference(args):
    """The reference's CPU implementation of the path (the oracle port of
    metaLBM's serial Algorithm loop, all host threads over x slabs) on the
    GPU arm's workload: same grid, initial field, metric and alpha solver,
    W warm-up and K timed steps; entropic workloads add one step with the
    reference's own alpha solver. Rank 0 only."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    name = args.workload
    w = WORKLOADS[name]
    threads = os.cpu_count() or 1
    shape = reference_shape(name, args.grid)
    V = int(np.prod(shape))
    fields = initial_field(name, shape)
    differences = reference_differences(name, shape)
    run = PortRun(name, shape, threads, fields=fields)
    run.step(args.warmup)
    t0 = time.perf_counter()
    run.step(args.steps)
    dt = time.perf_counter() - t0
    run.close()
    value = V * args.steps / dt / 1e6
    sample = (f"{w['latticeT']} FP64 {solver_words(name)}, the workload's "
              f"{'x'.join(map(str, shape))} grid and initial field, {args.warmup} warm-up + "
              f"{args.steps} timed steps, {threads} threads (x slabs)")
    line = {
        "impl": "reference", "metric": metric_for(name), "value": value, "unit": "MLUPS",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": name, "grid": list(shape), "same_config": not differences,
                   "differences": differences, "alpha_solver": solver_words(name)},
        "cpu_baseline": {"value": value, "unit": "MLUPS", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": value, "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    if w["collisionT"] != "BGK":
        ref = PortRun(name, shape, threads, alpha="reference", fields=fields)
        t0 = time.perf_counter()
        ref.step(1)
        dtr = time.perf_counter() - t0
        ref.close()
        line["reference_alpha_solver"] = {
            "value": V / dtr / 1e6, "unit": "MLUPS",
            "sample": f"one step of the same run with {solver_words(name, 'reference')}"}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="entropic_learned_512", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline leg")
    ap.add_argument("--no-others", action="store_true",
                    help="skip the other workloads' device timings in the default line")
    ap.add_argument("--grid", type=int, default=0,
                    help="cubic grid side overriding the workload's (profiling captures of a "
                         "smaller case; not a bench configuration)")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
