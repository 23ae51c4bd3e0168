"""Benchmark of the MLS-MPM time step on GB300: particle-steps/s.

Workload (default): 3D jelly, 128^3 grid, 4 jittered cubes of 64^3 lattice particles
(1,048,576 particles) with centres uniform in [0.25, 0.75]^3, jitter +-0.25 cell, per-cube
velocity N(0, 0.5^2) per axis, dt = 1e-4, E = 1e4, nu = 0.2, gravity = -100, the
reference's physics (MaterialModel::kJelly).  Seeded synthetic input.

A step is one advance() over all particles.  Lines printed (rank 0, one JSON line):
  value     particle-steps/s with the state resident in HBM: K steps of advance() on the
            simulation's stream, CUDA events around them, max over ranks;
  e2e       the same metric through the C ABI with host buffers: every step uploads the
            particle state from pinned host memory (nclr_set_particles), advances one step and
            reads the state back (nclr_get_particles);
  roofline  the dominant kernel's algorithmic bytes per launch / its average launch time,
            measured with CUDA events on the simulation's stream inside the timed region;
  cpu_baseline  the CPU oracle (a restatement of the reference's step, built -Ofast like the
            reference) on one host core, on a bounded sample of the same workload;
  error_vs_fp64  one GPU step at the timed size from the state the timed region ended in,
            against the FP64 oracle on all host cores (normwise per field and for the grid).
Further forms (objects on the same line; `--only FORM` runs one alone): batched (256 2D
scenes), adjoint (fwd + backward rollout), mixed (4.19M liquid + snow), snow, corrected (the
headline geometry in jelly and snow under the corrected physics), readme, models.  Each carries
its own roofline and error_vs_fp64.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

N > 1 (under torchrun): every rank runs its own replica of the scene on its own GPU (the
step has no cross-scene exchange), value = all ranks' particle-steps / the slowest rank's
time ("scaling": "weak").
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("particle-steps/s 1×GB300 (plain, batched, fwd+adjoint) vs CPU ref; "
          "%HBM roofline")
UNIT = "particle-steps/s"
WORKLOAD = {"workload": "3D jelly (MaterialModel::kJelly), 4 cubes of 64^3 lattice particles",
            "particles": 1_048_576, "grid": "128^3 (129^3 nodes)", "dim": 3, "dt": 1e-4,
            "E": 1e4, "nu": 0.2, "gravity": -100.0, "physics": "reference", "seed": 0,
            "l2": "inputs larger than L2 (particle state ~190 MB in HBM)"}

# Per-launch DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) of the dominant kernel
# from one ncu capture of this workload: the sixth launch of g2p2g_kernel<3, 1, 0, 0, 1> (a
# step, reference physics, the material fixed to jelly).
NCU_TRAFFIC = {"g2p2g": 68.49408e6 + 5.248e6}
# Warp-instructions of one launch of that kernel (smsp__inst_executed.sum, same capture): the
# kernel is bound by issue and latency rather than HBM, so the line also reports how close one
# launch comes to its issue floor (4 schedulers per SM, one warp-instruction per cycle each).
NCU_INSTRUCTIONS = {"g2p2g": 63.485103e6}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def algorithmic_bytes(dim: int, n: int, active: int) -> dict:
    """Bytes the fused step kernel must move per launch (every input read once, every output
    written once, FP32).  g2p2g reads x, F, Jp, mass, volume (60 B in 3D) and writes x, F, Jp
    (52 B); it reads one updated node (16 B) and adds one accumulated node (16 B) per active
    node; v and C (48 B) are written only by the last step of an advance() call and are not
    counted.  The grid sweep reads G and writes V and the cleared G: 48 B per node."""
    d2 = dim * dim
    g2p2g = n * ((dim + d2 + 3) + (dim + d2 + 1)) * 4 + active * 32
    return {"g2p2g": g2p2g}


FIELDS = ("x", "v", "F", "C", "Jp")
# Floors of the normwise error, in each field's units (the measure of the parity tests).
FLOORS = {"x": 1.0, "v": 1e-2, "F": 1.0, "C": 1.0, "Jp": 1.0, "grid_v": 1e-2, "grid_m": 1e-3}


def field_err(a, b, name: str) -> float:
    """max|a - b| / max(max|b|, floor): the normwise relative error of one field."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    if a.size == 0:
        return 0.0
    return float(np.abs(a - b).max() / max(float(np.abs(b).max()), FLOORS.get(name, 0.0), 1e-30))


def roofline_of(kernel: str, alg_bytes: float, avg_ms: float, traffic=None, **extra) -> dict:
    """HBM roofline of one kernel: algorithmic bytes per launch / its CUDA-event launch time."""
    hbm, kind = peaks()
    achieved = alg_bytes / (avg_ms / 1e3) / 1e9
    out = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": hbm, "unit": "GB/s",
           "frac": achieved / hbm, "peak_source": kind, "traffic": traffic,
           "algorithmic_bytes": alg_bytes, "avg_launch_ms": avg_ms}
    out.update(extra)
    return out


def state_of(sim, scene: dict) -> dict:
    """The particles of a simulation as an oracle state (caller order)."""
    p = sim.particles()
    return {"x": p.x, "v": p.v, "F": p.F, "C": p.C, "Jp": p.Jp, "mass": scene["mass"],
            "volume": scene["volume"]}


def error_vs_fp64(state: dict, *, dim: int, model: int, res: int, device: int, what: str,
                  material=None, physics: int = 0, dt: float = 1e-4, E: float = 1e4,
                  nu: float = 0.2, gravity: float = -100.0, stress: int = 0, E_p=None,
                  nu_p=None) -> dict:
    """The error of one GPU step at the timed size against the FP64 oracle (the reference's step
    restated in double precision, on all host cores) from the same state: a fresh simulation
    created from `state` advances one step; every field and the grid are compared normwise."""
    from oracle import pyoracle as po
    from nuclearmpm_gb300 import MPMSimulation
    sim = MPMSimulation(dict(state), model, res=res, dt=dt, E=E, nu=nu, gravity=gravity,
                        material=material, physics=physics, stress_model=stress, device=device)
    if E_p is not None:
        sim.set_moduli(E_p, nu_p)
    sim.advance(1)
    p = sim.particles()
    g = sim.grid()
    sim.close()
    threads = os.cpu_count() or 1
    kw = dict(dim=dim, model=model, res=res, dt=dt, E=E, nu=nu, gravity=gravity, steps=1,
              physics=physics, material=material, threads=threads, stress=stress,
              E_particles=E_p, nu_particles=nu_p)
    o, og, st, _ = po.advance(state, fp64=True, **kw)
    o32, og32, _, _ = po.advance(state, **kw)  # the FP32 restatement: its own distance
    gpu = {f: getattr(p, f) for f in FIELDS}
    gpu.update(grid_v=g.velocity, grid_m=g.mass)
    o.update(grid_v=og[0], grid_m=og[1])
    o32.update(grid_v=og32[0], grid_m=og32[1])
    fields = {f: field_err(gpu[f], o[f], f) for f in gpu}
    own = {f: field_err(o32[f], o[f], f) for f in gpu}
    # particles whose F row is further than 1e-5 from FP64 (each F entry is of order 1)
    rows = lambda a: np.abs(np.asarray(a, np.float64) - o["F"]).reshape(len(o["F"]), -1).max(1)  # noqa: E731
    return {"max": max(fields.values()), "fields": fields, "state": what,
            "fp32_oracle_vs_fp64": own,
            "F_rows_over_1e-5": {"gpu": int((rows(p.F) > 1e-5).sum()),
                                 "fp32_oracle": int((rows(o32["F"]) > 1e-5).sum()),
                                 "particles": int(len(o["F"]))},
            "measure": "max|gpu - fp64| / max(max|fp64|, floor) per field",
            "oracle": f"FP64 oracle, one step, {threads} host threads", "oracle_status": st}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for _, _, r in rows for i, v in enumerate(r) if v == "Active"})
        top = max(r[0] for r in rows)
        loaded = [r[0] for r in rows if r[0] >= 0.5 * top] or [r[0] for r in rows]
        return {"sm_mhz": statistics.median(loaded), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


def host_cpu() -> dict:
    """The host the CPU legs run on: online cores and the CPU model (Arm machines report no
    "model name"; their implementer/part codes and /proc/device-tree model stand in)."""
    model = None
    try:
        with open("/proc/cpuinfo") as f:
            info = f.read()
        for key in ("model name", "Model", "CPU part"):
            for line in info.splitlines():
                if line.split(":")[0].strip() == key:
                    model = line.split(":", 1)[1].strip()
                    break
            if model:
                break
    except OSError:
        pass
    try:
        with open("/proc/device-tree/model") as f:
            model = (model + " / " if model else "") + f.read().strip("\x00\n ")
    except OSError:
        pass
    import platform
    arm_parts = {"0xd4f": "Arm Neoverse-V2 (Grace)", "0xd40": "Arm Neoverse-V1",
                 "0xd0c": "Arm Neoverse-N1", "0xd8e": "Arm Neoverse-N3"}
    if model in arm_parts:
        model = arm_parts[model]
    return {"nproc": os.cpu_count(), "cpu": model or platform.processor() or platform.machine(),
            "arch": platform.machine()}


def tune_plain(state: dict, model: int, res: int, device: int, physics: int = 0,
               material=None) -> dict:
    """The project's autotuner (nuclearmpm_gb300.autotune) on this workload: re-sort interval
    and thin-block threshold, from short timed runs of the simulation itself."""
    from nuclearmpm_gb300 import MPMSimulation, autotune
    # 256-step runs, best of three (about 42 ms each at 1M particles): the candidates differ by
    # a few percent (re-sorting every 8 steps against 16 trades sort time against a faster
    # fused kernel, 2% apart on the 1M jelly scene), which 128-step runs timed on the host
    # resolved differently from run to run; the pick is then confirmed against the defaults
    # in two alternating rounds
    return autotune.tune(lambda **o: MPMSimulation(dict(state), model, res=res, device=device,
                                                   physics=physics, material=material, **o),
                         key=None, candidates=autotune.PLAIN_CANDIDATES, steps=256, repeats=3,
                         cache_path=None, confirm=2)


def make_scene():
    from nuclearmpm_gb300 import scenes
    return scenes.jelly_cubes_3d(seed=0, res=128)


def cpu_reference_run(scene: dict, steps: int, warmup: int, budget_s: float, threads: int = 1,
                      model: int = 1, res: int = 128, material=None):
    """The CPU oracle (-Ofast build; one thread, or `threads` for the multi-threaded port of
    oracle/nclr_oracle_mt.h) on the workload: `warmup` untimed steps, then `steps` timed
    steps, on the full scene if that fits `budget_s`, else on the first particles of the scene
    (same per-particle work) so that it does."""
    from oracle import pyoracle as po
    n = len(scene["x"])
    kw = dict(dim=3, model=model, res=res, fast=True, want_grid=False, threads=threads)
    t0 = time.perf_counter()
    state, _, st, _ = po.advance(scene, steps=1, material=material, **kw)
    one = time.perf_counter() - t0
    total = max(1, steps + max(warmup - 1, 0))
    frac = min(1.0, budget_s / max(one * total, 1e-9))
    m = n if frac >= 1.0 else max(4096, int(n * frac) // 4096 * 4096)
    sample = {k: (np.asarray(v)[:m] if k in ("x", "v", "F", "C", "Jp", "mass", "volume") else v)
              for k, v in state.items()}
    mat = None if material is None else np.asarray(material)[:m]
    if warmup > 1:
        sample, _, st, _ = po.advance(sample, steps=warmup - 1, material=mat, **kw)
    t0 = time.perf_counter()
    _, _, st, _ = po.advance(sample, steps=steps, material=mat, **kw)
    dt = time.perf_counter() - t0
    if st != 0:
        raise RuntimeError("CPU oracle reported an out-of-range stencil")
    desc = (f"{m:,} of {n:,} particles (the scene's first) x {steps} steps, {res}^3 grid"
            if m < n else f"all {n:,} particles x {steps} steps, {res}^3 grid")
    return m * steps / dt, desc


def run_batched(device: int, steps: int = 100, sequential: bool = True, repeats: int = 3) -> dict:
    """The batched form on 256 independent 2D scenes (particle counts log-uniform in
    [1,000, 65,536], grids of 64/128/256, mixed materials and moduli; seeded): one
    BatchSimulation advancing `steps` steps in one CUDA graph, against the same scenes stepped
    one after another as plain simulations (each `steps` steps with its own graphs, on its
    automatically chosen path).  Both timed the same way: CUDA events on the simulations'
    streams after a warm-up call, the best of `repeats` calls (one call is a few ms for the
    batch and tens of µs for a small scene, where single timings vary by ~10%)."""
    import torch

    from nuclearmpm_gb300 import BatchSimulation, MPMSimulation, autotune, scenes
    scs = scenes.batched_scenes_2d(seed=0)
    total = sum(len(sc["x"]) for sc in scs)
    # tuned on runs as long as the timed one, best of three each, and the pick confirmed
    # against the defaults in two alternating rounds: the candidates' times differ by a few
    # percent, and one noisy measurement can pick a set slower than the defaults
    tuned = autotune.tune(lambda **o: BatchSimulation(scs, device=device, **o), key=None,
                          candidates=autotune.BATCH_CANDIDATES, steps=steps, repeats=3,
                          graph_steps=steps, cache_path=None, confirm=2)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def best_of(sim) -> float:
        sim.advance(steps)  # warm-up: sort, first P2G, graph capture
        st = torch.cuda.ExternalStream(sim.stream)
        best = float("inf")
        for _ in range(repeats):
            a.record(st)
            sim.advance(steps)
            b.record(st)
            b.synchronize()
            best = min(best, a.elapsed_time(b) / 1e3)
        return best

    batch = BatchSimulation(scs, device=device, **tuned)  # tuned includes graph_steps = steps
    t_batch = best_of(batch)
    launches = batch.stats()[0]
    batch.close()
    # the fused kernel's roofline: the same batch with per-kernel CUDA events (direct launches)
    pb = BatchSimulation(scs, device=device, profile=True,
                         **{k: v for k, v in tuned.items() if k != "graph_steps"})
    pb.advance(steps)
    pb.profile_reset()
    pb.advance(steps)
    prof = pb.profile()
    active = pb.active_nodes()
    pb.close()
    g_ms = prof["g2p2g"][0] / max(prof["g2p2g"][1], 1)
    alg = algorithmic_bytes(2, total, active)["g2p2g"]
    roof = roofline_of("g2p2g", alg, g_ms, active_nodes=active,
                       kernels={k: {"total_ms": v[0], "launches": v[1], "avg_ms": v[0] / max(v[1], 1)}
                                for k, v in prof.items() if v[1] > 0},
                       timing="a separate run of the same batch with per-kernel CUDA events")
    err = batched_error_vs_fp64(scs, device)
    t_seq = 0.0
    for sc in (scs if sequential else []):
        sim = MPMSimulation({k: sc[k] for k in ("x", "v", "F", "C", "Jp", "mass", "volume")},
                            sc["model"], res=sc["res"], dt=sc["dt"], E=sc["E"], nu=sc["nu"],
                            gravity=sc["gravity"], device=device)
        t_seq += best_of(sim)
        sim.close()
    return {"value": total * steps / t_batch, "unit": UNIT, "scenes": len(scs),
            "particles": total, "steps": steps, "ms_per_step": t_batch / steps * 1e3,
            "gpu_launches": launches, "tuned": tuned, "roofline": roof, "error_vs_fp64": err,
            "sequential_value": total * steps / t_seq if sequential else None,
            "speedup_vs_sequential": t_seq / t_batch if sequential else None,
            "config": "256 2D scenes, n log-uniform [1e3, 65536], res {64,128,256}, "
                      "materials uniform, E log-uniform [1e3,1e5], nu uniform [0.1,0.4], "
                      "dt 1e-4, one CUDA graph per 100 steps; sequential = the same scenes as "
                      "plain simulations one after another; best of 3 calls on both sides"}


def batched_error_vs_fp64(scs: list, device: int) -> dict:
    """One step of all 256 scenes as one batch against the FP64 oracle of each scene: the
    largest normwise error over the scenes, per field and for the grid."""
    from oracle import pyoracle as po
    from nuclearmpm_gb300 import BatchSimulation
    b = BatchSimulation(scs, device=device)
    b.advance(1)
    threads = os.cpu_count() or 1
    worst = {}
    for i, sc in enumerate(scs):
        got = b.particles(i)
        g = b.grid(i)
        state = {k: sc[k] for k in ("x", "v", "F", "C", "Jp", "mass", "volume")}
        o, og, st, _ = po.advance(state, dim=2, model=sc["model"], res=sc["res"], dt=sc["dt"],
                                  E=sc["E"], nu=sc["nu"], gravity=sc["gravity"], steps=1,
                                  fp64=True, threads=threads)
        errs = {f: field_err(got[f], o[f], f) for f in FIELDS}
        errs["grid_v"] = field_err(g.velocity, og[0], "grid_v")
        errs["grid_m"] = field_err(g.mass, og[1], "grid_m")
        for f, e in errs.items():
            worst[f] = max(worst.get(f, 0.0), e)
    b.close()
    return {"max": max(worst.values()), "fields": worst,
            "state": f"the {len(scs)} scenes as built, one batched step",
            "measure": "max over scenes of max|gpu - fp64| / max(max|fp64|, floor) per field",
            "oracle": f"FP64 oracle per scene, one step, {threads} host threads"}


def adjoint_error_vs_fp64(device: int, sc: dict, v0: np.ndarray, target: np.ndarray,
                          steps: int = 1) -> dict:
    """The gradients of the timed rollout's loss through `steps` steps at the timed size
    (131,072 particles) against the FP64 adjoint of the reference step on the host: the
    initial-velocity gradients normwise, E and nu relative."""
    import torch

    from oracle import pyoracle as po
    from nuclearmpm_gb300.autograd import Rollout
    n = len(sc["x"])
    dev = torch.device("cuda", device)
    roll = Rollout(sc["x"], res=64, steps=steps, checkpoint_every=1, device=device)
    x0 = torch.tensor(sc["x"], device=dev)
    v = torch.tensor(v0, device=dev, requires_grad=True)
    E = torch.tensor(1e4, dtype=torch.float64, requires_grad=True)
    nu = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    tgt = torch.tensor(target, device=dev)
    xT, _ = roll(x0, v, E, nu)
    loss = ((xT.mean(0) - tgt) ** 2).sum()
    loss.backward()
    roll.close()
    # the loss's adjoint of the final positions, evaluated at the GPU's final state
    seed_x = np.broadcast_to((2.0 * (xT.mean(0) - tgt) / n).detach().cpu().numpy().astype(np.float64),
                             (n, 3)).copy()
    state = dict(sc, v=v0)
    _, g = po.adjoint(state, dim=3, res=64, steps=steps, seed={"x": seed_x})
    gv = v.grad.detach().cpu().numpy().astype(np.float64)
    e_v = float(np.abs(gv - g["v"]).max() / max(np.abs(g["v"]).max(), 1e-300))
    e_E = abs(float(E.grad) - g["E"]) / max(abs(g["E"]), 1e-300)
    e_nu = abs(float(nu.grad) - g["nu"]) / max(abs(g["nu"]), 1e-300)
    return {"max": max(e_v, e_E, e_nu), "fields": {"grad_v0": e_v, "grad_E": e_E, "grad_nu": e_nu},
            "state": f"the timed rollout's scene, initial velocities and loss, {steps} step",
            "measure": "grad_v0: max|gpu - fp64| / max|fp64|; grad_E, grad_nu: relative",
            "oracle": "FP64 adjoint of the reference step (oracle/nclr_adjoint.h), one thread"}


def run_adjoint_snow(device: int, sc: dict, v0, target, x0, steps: int = 500,
                     every: int = 50) -> dict:
    """The same scene, velocities and loss as a snow rollout (the plastic adjoint: the clamp's
    singular-value backward, the Jp update and the Jp-dependent hardening) under the corrected
    physics, `steps` steps with a checkpoint every `every`: device times of the forward and of
    the backward."""
    import torch

    from nuclearmpm_gb300 import scenes
    from nuclearmpm_gb300.autograd import Rollout
    n = len(sc["x"])
    roll = Rollout(sc["x"], res=64, steps=steps, checkpoint_every=every, device=device,
                   physics=scenes.CORRECTED, model=scenes.SNOW)
    v = v0.clone().requires_grad_(True)
    E = torch.tensor(1e4, dtype=torch.float64, requires_grad=True)
    nu = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    for _ in range(2):  # the second iteration is the measured one (F0 = I, C0 = 0)
        v.grad = None
        xT, _ = roll(x0, v, E, nu)
        ((xT.mean(0) - target) ** 2).sum().backward()
    fwd_ms, bwd_ms = roll.timing()
    roll.close()
    return {"value": n * steps / ((fwd_ms + bwd_ms) / 1e3), "unit": UNIT, "particles": n,
            "steps": steps, "checkpoint_every": every, "forward_ms": fwd_ms,
            "backward_ms": bwd_ms, "backward_over_forward": bwd_ms / fwd_ms,
            "grad_norms": {"v0": float(v.grad.norm()), "E": float(E.grad), "nu": float(nu.grad)},
            "config": "3D snow rollout, the adjoint form's scene and loss, corrected physics"}


def run_adjoint(device: int, steps: int = 2000, every: int = 50) -> dict:
    """The differentiable form: 3D jelly, 64^3 grid, one 64x64x32 jittered lattice (131,072
    particles, seeded), `steps` steps with a checkpoint every `every`; loss = squared distance
    of the final centre of mass from a seeded target; gradients with respect to the initial
    velocities, Young's modulus and Poisson ratio through nuclearmpm_gb300.autograd.  Device
    times of the forward and of the backward (which recomputes every segment) from CUDA
    events on the rollout's stream."""
    import torch

    from nuclearmpm_gb300 import scenes
    from nuclearmpm_gb300.autograd import Rollout
    sc = scenes.jelly_block_3d(seed=0, res=64, shape=(64, 64, 32))
    n = len(sc["x"])
    rng = np.random.default_rng(0)
    dev = torch.device("cuda", device)
    roll = Rollout(sc["x"], res=64, steps=steps, checkpoint_every=every, device=device)
    x0 = torch.tensor(sc["x"], device=dev)
    v0 = torch.tensor(rng.normal(0, 0.5, size=(n, 3)).astype(np.float32), device=dev,
                      requires_grad=True)
    E = torch.tensor(1e4, dtype=torch.float64, requires_grad=True)
    nu = torch.tensor(0.2, dtype=torch.float64, requires_grad=True)
    target = torch.tensor(rng.uniform(0.3, 0.7, size=3).astype(np.float32), device=dev)
    for _ in range(2):  # the second iteration is the measured one
        v0.grad = None
        E.grad = None
        nu.grad = None
        xT, vT = roll(x0, v0, E, nu)
        loss = ((xT.mean(0) - target) ** 2).sum()
        loss.backward()
    fwd_ms, bwd_ms = roll.timing()
    roll.close()
    # per-kernel CUDA events: a second rollout of the same scene with profiling (direct launches)
    proll = Rollout(sc["x"], res=64, steps=steps, checkpoint_every=every, device=device,
                    profile=True)
    v0.grad = None
    xT, _ = proll(x0, v0, E, nu)
    ((xT.mean(0) - target) ** 2).sum().backward()
    prof = proll.profile()
    proll.close()
    nodes = 65 ** 3
    per_particle = {"adj_g2p": 228, "adj_p2g": 248}  # bytes per particle: see bytes_note below
    roofs = {}
    for k in ("adj_g2p", "adj_grid", "adj_p2g", "g2p2g"):
        if prof[k][1] == 0:
            continue
        avg = prof[k][0] / prof[k][1]
        if k == "adj_grid":
            alg = 64 * nodes
        elif k == "g2p2g":
            alg = algorithmic_bytes(3, n, 0)["g2p2g"]
        else:
            alg = per_particle[k] * n
        roofs[k] = roofline_of(k, alg, avg, launches=prof[k][1])
    dom = max(("adj_g2p", "adj_grid", "adj_p2g"), key=lambda k: prof[k][0])
    err = adjoint_error_vs_fp64(device, sc, v0.detach().cpu().numpy(), target.cpu().numpy())
    snow = run_adjoint_snow(device, sc, v0.detach(), target, x0)
    return {"value": n * steps / ((fwd_ms + bwd_ms) / 1e3), "unit": UNIT, "snow": snow,
            "roofline": dict(roofs[dom], kernels=roofs,
                             bytes_note="algorithmic bytes per launch: adj_g2p reads x, F, C', "
                             "gF', gC', gx', gv' and writes gx, gF (228 B per particle); adj_p2g "
                             "reads x, v, F, C, m, vol, gx, gF and writes gx, gv, gF, gC (248 B); "
                             "adj_grid reads V, VB and writes GB and the cleared VB over all 65^3 "
                             "nodes (64 B per node); the particle kernels' node gathers and "
                             "reductions (about 23k touched nodes) are not counted; g2p2g counts "
                             "the plain step's 112 B per particle (the recorded rows are extra)"),
            "error_vs_fp64": err,
            "metric": "fwd+adjoint particle-steps/s", "particles": n, "steps": steps,
            "checkpoint_every": every, "forward_ms": fwd_ms, "backward_ms": bwd_ms,
            "backward_over_forward": bwd_ms / fwd_ms,
            "forward_value": n * steps / (fwd_ms / 1e3),
            "grad_norms": {"v0": float(v0.grad.norm()), "E": float(E.grad), "nu": float(nu.grad)},
            "config": "3D jelly, 64^3 grid, 64x64x32 jittered lattice, dt 1e-4, loss |COM - "
                      "target|^2, gradients w.r.t. v0, E, nu"}


def run_plain_form(scene: dict, model: int, res: int, device: int, steps: int, *, physics: int,
                   material=None, label: str, tune: bool = True) -> dict:
    """One single-simulation form: the autotuned simulation (the library's defaults otherwise:
    CUDA graphs, overlapped launches) advances `steps` steps after a 10-step warm-up, timed
    with CUDA events on its stream; the same steps on a profiled handle (direct launches with
    CUDA events around every kernel) give the fused kernel's roofline; then the error of one
    step from the state the timed region ended in, against the FP64 oracle."""
    import torch

    from nuclearmpm_gb300 import MPMSimulation
    n = len(scene["x"])
    tuned = tune_plain(scene, model, res, device, physics, material) if tune else {}
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(profile: bool):
        sim = MPMSimulation(dict(scene), model, res=res, material=material, physics=physics,
                            profile=profile, device=device, **tuned)
        sim.advance(10)
        sim.profile_reset()
        st = torch.cuda.ExternalStream(sim.stream)
        a.record(st)
        sim.advance(steps)
        b.record(st)
        b.synchronize()
        return sim, a.elapsed_time(b) / 1e3

    sim, t = timed(False)
    launches = sim.stats()[0]
    end_state = state_of(sim, scene)
    sim.close()
    psim, pt = timed(True)
    prof = psim.profile()
    active = psim.active_nodes()
    psim.close()
    g_ms = prof["g2p2g"][0] / max(prof["g2p2g"][1], 1)
    alg = algorithmic_bytes(3, n, active)["g2p2g"] + (n if material is not None else 0)
    kernels = {k: {"total_ms": v[0], "launches": v[1], "avg_ms": v[0] / max(v[1], 1),
                   "share": v[0] / max(pt * 1e3, 1e-9)} for k, v in prof.items() if v[1] > 0}
    err = error_vs_fp64(end_state, dim=3, model=model, res=res, device=device, material=material,
                        physics=physics, what=f"the state after the {10 + steps} steps run")
    return {"value": n * steps / t, "unit": UNIT, "particles": n, "steps": steps,
            "ms_per_step": t / steps * 1e3, "gpu_launches": launches,
            "physics": "reference" if physics == 0 else "corrected", "tuned": tuned,
            "roofline": dict(roofline_of("g2p2g", alg, g_ms, kernels=kernels, active_nodes=active),
                             timing="CUDA events around every kernel, the same steps on a "
                                    "profiled handle (direct launches: "
                                    f"{pt / steps * 1e3:.4f} ms per step there)"),
            "error_vs_fp64": err, "config": label}


def run_mixed(device: int, steps: int = 100) -> dict:
    """The mixed-material workload: 3D, 256^3 grid, 4,194,304 particles in 16 seeded boxes in
    the upper half of the domain, half liquid and half snow (one material per particle, an
    extension of the reference), falling under gravity; `steps` steps timed with CUDA events
    on the simulation's stream after warm-up; the CPU oracle (one thread, -Ofast) on a sample
    of the same scene beside it."""
    from nuclearmpm_gb300 import scenes
    sc, mat = scenes.liquid_snow_boxes_3d(seed=0, res=256)
    out = run_plain_form(sc, scenes.SNOW, 256, device, steps, physics=scenes.REFERENCE,
                         material=mat, tune=False,
                         label="3D liquid + snow, 256^3 grid, 16 boxes (sides U[0.05,0.2]), "
                               "per-particle material, dt 1e-4, reference physics")
    if int(os.environ.get("RANK", "0")) == 0:
        v, desc = cpu_reference_run(sc, steps=2, warmup=1, budget_s=12.0, model=scenes.SNOW,
                                    res=256, material=mat)
        out["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": desc + "; the reference's step restated in C++ "
                               "(oracle/, -Ofast like the reference build), one thread"}
    return out


def run_snow(device: int, steps: int = 100) -> dict:
    """3D snow on the headline geometry: the four jittered 64^3 lattices of the 1M-particle
    jelly scene (128^3 grid, same seed) with MaterialModel::kSnow, reference physics; `steps`
    steps timed with CUDA events on the simulation's stream after warm-up, with the fused
    kernel's per-launch device time and its fraction of the HBM roofline.  Under the
    reference's diag(1,1,0) this scene flies apart (see run_corrected for the same scene under
    the corrected physics)."""
    from nuclearmpm_gb300 import scenes
    out = run_plain_form(make_scene(), scenes.SNOW, 128, device, steps, physics=scenes.REFERENCE,
                         label="3D snow (MaterialModel::kSnow), the 1M-particle scene above, "
                               "128^3 grid, dt 1e-4, reference physics")
    # the keys of earlier lines
    out["g2p2g_avg_ms"] = out["roofline"]["avg_launch_ms"]
    out["g2p2g_frac"] = out["roofline"]["frac"]
    return out


def run_corrected(device: int, steps: int = 100) -> dict:
    """The headline geometry (four jittered 64^3 lattices, 1,048,576 particles, 128^3 grid)
    under the corrected physics (the true identity, where the reference has diag(1,1,0)), where
    the step's physics is meaningful: jelly and snow, each timed, with its roofline and its
    one-step error against the FP64 oracle."""
    from nuclearmpm_gb300 import scenes
    sc = scenes.jelly_cubes_3d(seed=0, res=128, physics=scenes.CORRECTED)
    out = {}
    for name, model in (("jelly", scenes.JELLY), ("snow", scenes.SNOW)):
        out[name] = run_plain_form(sc, model, 128, device, steps, physics=scenes.CORRECTED,
                                   label=f"3D {name}, the 1M-particle scene of the headline, "
                                         "128^3 grid, dt 1e-4, corrected physics")
    return out


def run_readme(device: int, steps: int = 4000, cpu_steps: int = 400) -> dict:
    """The README scene (2D snow, two cube<2>(50, 0.4, 0.6) lattices, 5,000 particles, res 64,
    dt 1e-4): `steps` steps timed with CUDA events on the simulation's stream (CUDA graphs),
    and the CPU oracle (-Ofast, one thread) timed on `cpu_steps` steps of the same scene."""
    import torch

    from oracle import pyoracle as po
    from nuclearmpm_gb300 import MPMSimulation, autotune, scenes
    sc = scenes.readme_scene()
    n = len(sc["x"])
    tuned = autotune.tune(lambda **o: MPMSimulation(dict(sc), scenes.SNOW, res=64, device=device, **o),
                          key=None, candidates=autotune.SMALL_CANDIDATES, steps=200, repeats=2,
                          cache_path=None, confirm=2)
    sim = MPMSimulation(dict(sc), scenes.SNOW, res=64, graph_steps=200, device=device, **tuned)
    sim.advance(200)
    st = torch.cuda.ExternalStream(sim.stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    sim.advance(steps)
    b.record(st)
    b.synchronize()
    t = a.elapsed_time(b) / 1e3
    launches = sim.stats()[0]
    end_state = state_of(sim, sc)
    sim.close()
    t0 = time.perf_counter()
    po.advance(sc, dim=2, model=scenes.SNOW, res=64, steps=cpu_steps, fast=True, want_grid=False)
    tc = time.perf_counter() - t0
    err = error_vs_fp64(end_state, dim=2, model=scenes.SNOW, res=64, device=device,
                        what=f"the state after the {200 + steps} steps run")
    return {"value": n * steps / t, "unit": UNIT, "particles": n, "steps": steps,
            "ms_per_step": t / steps * 1e3, "gpu_launches": launches,
            "cpu_value": n * cpu_steps / tc, "cpu_sample": f"{cpu_steps} steps of the same scene, "
            "oracle -Ofast, one thread", "speedup_vs_cpu": (n * steps / t) / (n * cpu_steps / tc),
            "tuned": tuned, "error_vs_fp64": err,
            "config": "README scene: 2D snow, 5,000 particles, res 64, dt 1e-4, reference "
                      "physics, CUDA graphs of 200 steps"}


def run_models(device: int, steps: int = 100) -> dict:
    """The model extensions on the headline geometry: the four jittered 64^3 jelly lattices,
    128^3 grid, under the corrected physics (det F > 0, which the neo-Hookean stress needs).
    Three runs: the reference's fixed-corotated stress; the neo-Hookean stress; and the
    corotated stress with every particle's own E (log-uniform in [1e3, 1e4]) and nu (uniform
    in [0.1, 0.4]). Each is `steps` steps, timed with CUDA events on the simulation's stream
    after warm-up, with the library's defaults (CUDA graphs, overlapped launches); the same
    steps on a profiled handle give the fused kernel's time."""
    import torch

    from nuclearmpm_gb300 import MPMSimulation, capi, scenes
    sc = scenes.jelly_cubes_3d(seed=0, res=128, physics=scenes.CORRECTED)
    n = len(sc["x"])
    rng = np.random.default_rng(0)
    E = np.exp(rng.uniform(np.log(1e3), np.log(1e4), size=n)).astype(np.float32)
    nu = rng.uniform(0.1, 0.4, size=n).astype(np.float32)
    out = {"unit": UNIT, "particles": n, "steps": steps}
    for name, stress, own in (("corotated", capi.STRESS_COROTATED, False),
                              ("neohookean", capi.STRESS_NEOHOOKEAN, False),
                              ("per_particle_moduli", capi.STRESS_COROTATED, True)):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

        def timed(profile: bool):
            sim = MPMSimulation(dict(sc), scenes.JELLY, res=128, physics=scenes.CORRECTED,
                                stress_model=stress, device=device, profile=profile)
            if own:
                sim.set_moduli(E, nu)
            sim.advance(10)
            sim.profile_reset()
            st = torch.cuda.ExternalStream(sim.stream)
            a.record(st)
            sim.advance(steps)
            b.record(st)
            b.synchronize()
            return sim, a.elapsed_time(b) / 1e3

        sim, t = timed(False)
        launches = sim.stats()[0]
        end_state = state_of(sim, sc)
        sim.close()
        psim, pt = timed(True)
        prof = psim.profile()
        active = psim.active_nodes()
        psim.close()
        g_ms = prof["g2p2g"][0] / max(prof["g2p2g"][1], 1)
        alg = algorithmic_bytes(3, n, active)["g2p2g"] + (8 * n if own else 0)
        out[name] = {"value": n * steps / t, "ms_per_step": t / steps * 1e3,
                     "gpu_launches": launches,
                     "roofline": dict(roofline_of("g2p2g", alg, g_ms, active_nodes=active),
                                      timing="the same steps on a profiled handle (direct "
                                             f"launches: {pt / steps * 1e3:.4f} ms per step)")}
        out[name]["error_vs_fp64"] = error_vs_fp64(
            end_state, dim=3, model=scenes.JELLY, res=128, device=device,
            physics=scenes.CORRECTED, stress=stress, E_p=E if own else None,
            nu_p=nu if own else None, what=f"the state after the {10 + steps} steps run")
    out["config"] = ("3D jelly, the 1M-particle scene of the headline built under the corrected "
                     "physics, 128^3 grid, dt 1e-4; corotated / neo-Hookean stress / corotated "
                     "with per-particle E in [1e3, 1e4] and nu in [0.1, 0.4]")
    return out


FORMS = {"batched": run_batched, "adjoint": run_adjoint, "mixed": run_mixed, "snow": run_snow,
         "readme": run_readme, "models": run_models, "corrected": run_corrected}


def run_form(args):
    """One form alone (for profiling): its JSON object on one line, `--form-steps` steps."""
    import torch
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    kw = {} if args.form_steps is None else {"steps": args.form_steps}
    if args.only == "batched" and args.no_sequential:
        kw["sequential"] = False
    out = FORMS[args.only](local, **kw)
    print(json.dumps({"form": args.only, **out}), flush=True)
    return 0


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    scene = make_scene()
    value, desc = cpu_reference_run(scene, args.steps, args.warmup, budget_s=150.0)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)", "config": dict(WORKLOAD), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": 1, "kind": "port",
                             "host": host_cpu(),
                             "sample": desc + "; the reference's step restated in C++ "
                             "(oracle/, -Ofast like the reference build), single thread as "
                             "the reference runs (its OpenMP pragmas are inert)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


class Replicas:
    """The ranks of a run: one independent replica of the workload per rank (one simulation
    does not shard; there is no data-path collective), with a barrier around the timed region
    and the max over ranks of its duration.  NCCL between GPUs; gloo on the host (tests)."""

    def __init__(self, backend: str = "nccl"):
        import torch
        import torch.distributed as dist
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.cuda = backend == "nccl"
        self._dist = dist
        if self.cuda:
            torch.cuda.set_device(self.local)
        if self.world > 1:
            kw = {"device_id": torch.device("cuda", self.local)} if self.cuda else {}
            dist.init_process_group(backend, **kw)

    def barrier(self) -> None:
        import torch
        if self.world > 1:
            self._dist.barrier()
        if self.cuda:
            torch.cuda.synchronize()

    def max(self, x: float) -> float:
        import torch
        if self.world == 1:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda" if self.cuda else "cpu")
        self._dist.all_reduce(t, op=self._dist.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.world > 1:
            self._dist.destroy_process_group()


def replica_value(world: int, particles: int, steps: int, ms_max: float) -> float:
    """Whole-job particle-steps/s: every rank steps its own replica, timed by the slowest."""
    return world * particles * steps / (ms_max / 1e3)


def run_ours(args):
    import torch

    from nuclearmpm_gb300 import MPMSimulation, scenes

    ranks = Replicas("nccl")
    world, rank, local = ranks.world, ranks.rank, ranks.local
    barrier, max_over_ranks = ranks.barrier, ranks.max

    scene = make_scene()
    n = len(scene["x"])
    tuned = tune_plain(scene, scenes.JELLY, 128, local)

    # ---- device-resident throughput: a handle with the library's defaults (CUDA graphs,
    # overlapped launches), as a caller's advance() runs ------------------------------------
    gsim = MPMSimulation(dict(scene), scenes.JELLY, res=128, device=local, **tuned)
    gstream = torch.cuda.ExternalStream(gsim.stream, device=torch.device("cuda", local))
    gsim.advance(args.warmup)
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches_total = 0
    with ClockSampler(local) as clocks:
        barrier()
        start.record(gstream)
        gsim.advance(args.steps)
        stop.record(gstream)
        stop.synchronize()
        barrier()
    launches_total += gsim.stats()[0]
    headline_end_state = state_of(gsim, scene)
    ms = start.elapsed_time(stop)
    ms_max = max_over_ranks(ms)
    clk = clocks.summary()
    value = replica_value(world, n, args.steps, ms_max)

    # ---- per-kernel times for the roofline: the same steps on a profiled handle (direct
    # launches with CUDA events around every kernel on its stream), timed the same way ------
    sim = MPMSimulation(dict(scene), scenes.JELLY, res=128, device=local, profile=True, **tuned)
    stream = torch.cuda.ExternalStream(sim.stream, device=torch.device("cuda", local))
    sim.advance(args.warmup)
    sim.profile_reset()
    pstart, pstop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    pstart.record(stream)
    sim.advance(args.steps)
    pstop.record(stream)
    pstop.synchronize()
    barrier()
    prof_ms = pstart.elapsed_time(pstop)
    prof = sim.profile()
    active = sim.active_nodes()
    sim.close()

    # ---- roofline of the dominant kernel ------------------------------------------------
    hbm_peak, peak_kind = peaks()
    alg = algorithmic_bytes(3, n, active)
    per_launch = {k: prof[k][0] / max(prof[k][1], 1) for k in prof if prof[k][1] > 0}
    dom = "g2p2g"
    achieved = alg[dom] / (per_launch[dom] / 1e3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm_peak,
                "unit": "GB/s", "frac": achieved / hbm_peak, "peak_source": peak_kind,
                "traffic": NCU_TRAFFIC.get(dom), "algorithmic_bytes": alg[dom],
                "avg_launch_ms": per_launch[dom],
                "kernels": {k: {"total_ms": prof[k][0], "launches": prof[k][1],
                                "avg_ms": prof[k][0] / max(prof[k][1], 1),
                                "share": prof[k][0] / max(prof_ms, 1e-9)} for k in prof},
                "active_nodes": active,
                "timing": "CUDA events around every kernel on the handle's stream, over the "
                          "same number of steps right after the headline's timed region, on a "
                          "handle created with nclr_options.profile (direct launches: "
                          f"{prof_ms / args.steps:.4f} ms per step there)"}
    inst = NCU_INSTRUCTIONS.get(dom)
    mhz = clk.get("sm_mhz") or clk.get("sm_max_mhz")
    if inst and mhz:
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        floor_ms = inst / (sms * 4 * mhz * 1e6) * 1e3
        roofline["issue"] = {"warp_instructions": inst, "sms": sms, "sm_mhz": mhz,
                             "floor_ms": floor_ms, "frac": floor_ms / per_launch[dom],
                             "source": "ncu smsp__inst_executed.sum of one launch"}

    # ---- end to end through the C ABI with host buffers ----------------------------------
    pin = lambda shape: torch.empty(shape, dtype=torch.float32, pin_memory=True).numpy()  # noqa: E731
    hx, hv, hF, hC, hJ = pin((n, 3)), pin((n, 3)), pin((n, 3, 3)), pin((n, 3, 3)), pin((n,))
    hx[:] = scene["x"]; hv[:] = scene["v"]; hF[:] = scene["F"]; hC[:] = scene["C"]; hJ[:] = scene["Jp"]
    ox, ov, oF, oC, oJ = pin((n, 3)), pin((n, 3)), pin((n, 3, 3)), pin((n, 3, 3)), pin((n,))
    from nuclearmpm_gb300 import capi
    from nuclearmpm_gb300.simulation import _ptr
    L = capi.lib()
    h = gsim._h  # the headline's handle: the library's defaults, as a caller's

    def e2e_step():
        capi.check(L.nclr_set_particles(h, _ptr(hx), _ptr(hv), _ptr(hF), _ptr(hC), _ptr(hJ)), h)
        capi.check(L.nclr_advance(h, 1), h)
        launches = gsim.stats()[0]
        capi.check(L.nclr_get_particles(h, _ptr(ox), _ptr(ov), _ptr(oF), _ptr(oC), _ptr(oJ)), h)
        return launches

    e2e = None
    if not args.no_e2e:
        for _ in range(max(args.warmup, 1)):
            e2e_step()
        barrier()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            launches_total += e2e_step() + 2  # + the import/prepare and export kernels
        torch.cuda.synchronize()
        e2e_s = max_over_ranks(time.perf_counter() - t0)
        barrier()
        row = 4 * (2 * 3 + 2 * 9 + 1)
        e2e = {"value": replica_value(world, n, args.steps, e2e_s * 1e3), "unit": UNIT,
               "h2d_bytes_per_step": n * row, "d2h_bytes_per_step": n * row,
               "path": "nclr_set_particles (pinned host) + nclr_advance(1) + nclr_get_particles"}

    batched = None
    if not args.no_batched:
        batched = run_batched(local)
    adjoint = None
    if not args.no_adjoint:
        adjoint = run_adjoint(local)
    mixed = None
    if not args.no_mixed:
        mixed = run_mixed(local)
    snow = None
    if not args.no_snow:
        snow = run_snow(local)
    readme = None
    if not args.no_readme and rank == 0:
        readme = run_readme(local)
    models = None
    if not args.no_models:
        models = run_models(local)
    corrected = None
    if not args.no_corrected:
        corrected = run_corrected(local)
    # one step at the headline's size from the state its timed region ended in, against the
    # FP64 oracle (the handle's state after the end-to-end leg is the uploaded scene stepped)
    err = error_vs_fp64(headline_end_state, dim=3, model=scenes.JELLY, res=128, device=local,
                        what=f"the state after the {args.warmup + args.steps} device-resident steps")

    cpu = cpu_mt = None
    if rank == 0 and not args.no_cpu_baseline:
        v, desc = cpu_reference_run(scene, steps=args.cpu_steps, warmup=1, budget_s=20.0)
        cpu = {"value": v, "unit": UNIT, "cores": 1, "kind": "port", "host": host_cpu(),
               "sample": desc + "; the reference's step restated in C++ (oracle/, -Ofast like "
                                "the reference build), one thread"}
        nt = os.cpu_count() or 1
        v, desc = cpu_reference_run(scene, steps=args.cpu_steps, warmup=1, budget_s=15.0,
                                    threads=nt)
        cpu_mt = {"value": v, "unit": UNIT, "cores": nt, "kind": "port",
                  "sample": desc + f"; the same port on {nt} threads, race-free (P2G over two "
                                   "colours of x-slabs, oracle/nclr_oracle_mt.h); the "
                                   "reference itself runs on one thread"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_max / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded scene with the workload's shapes and distributions)",
                "config": dict(WORKLOAD), "parallelism": f"replicas x{world}", "tuned": tuned,
                "roofline": roofline, "error_vs_fp64": err, "cpu_baseline": cpu,
                "cpu_baseline_mt": cpu_mt, "e2e": e2e, "batched": batched,
                "adjoint": adjoint, "mixed": mixed, "snow": snow, "corrected": corrected,
                "readme": readme, "models": models, "gpu_launches": launches_total,
                "clocks": clk}
        print(json.dumps(line), flush=True)
    gsim.close()
    ranks.close()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-steps", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-mixed", action="store_true")
    ap.add_argument("--no-snow", action="store_true")
    ap.add_argument("--no-readme", action="store_true")
    ap.add_argument("--no-models", action="store_true")
    ap.add_argument("--no-corrected", action="store_true")
    ap.add_argument("--no-e2e", action="store_true",
                    help="skip the end-to-end (host buffers) measurement, e.g. for a launch list "
                         "of the device-resident steps alone")
    ap.add_argument("--only", choices=sorted(FORMS), default=None,
                    help="run one of the other forms alone and print its object")
    ap.add_argument("--form-steps", type=int, default=None)
    ap.add_argument("--no-sequential", action="store_true",
                    help="with --only batched: skip stepping the scenes one by one")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    if args.only is not None:
        return run_form(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
