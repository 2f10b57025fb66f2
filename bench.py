#!/usr/bin/env python3
"""Benchmark of the GB300 patchy-Langevin step: particle-steps/s on the batched-replica workload.

Workload (default): 512 independent replicas, N_r log-uniform in [1,024, 32,768] (5,158,422 particles with seed 0),
4 tetrahedral patches, phi 0.15, kT_r ~ U[0.8, 1.2], depth_r ~ U[6, 10], range 1.2, cos 0.90, dt 0.005,
FP32 state with FP64 reductions, cell list rebuilt every step, one CUDA-graph launch per step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mtcode|reference]

One JSON line on rank 0.  ``value``: particle-steps/s of the device-resident step (all ranks);
``e2e``: the same metric through the C ABI with host buffers (state upload, every step's temperature
read back to pinned host memory as Condensate::run measures it every step, final state download) inside the
timed region; ``e2e.per_step_sync`` repeats it with a synchronous read after each step.  ``roofline``: the
dominant kernel's algorithmic bytes / its CUDA-event time against the measured HBM copy bandwidth.
``cpu_baseline``: the oracle (CPU restatement of the reference step) on a bounded sample, all host cores.
Multi-GPU: replicas only -- each rank runs its own full replica set (weak scaling), no collective on the
data path; the barrier and the max-over-ranks time use torch.distributed.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s on 1 GB300, batched FP32 vs plain FP64, force rel err <=1e-5"
UNIT = "particle-steps/s"
# algorithmic bytes per particle (FP32 rows of 48 B): what a pass must read and write once per particle
BYTES_FORCE = 48 + 24 + 4 + 48 + 8 + 4          # own x,Q + p,L + id; write p,L,F~,T~ + bin + histogram
BYTES_SCATTER = 8 + 4 + 48 + 48 + 4 + 24 + 48 + 24 + 4 + 24  # bin,start,row,row,id,disp -> row,p+L,id,disp
BYTES_SCAN_PER_CELL = 16
# the epilogue kernel alone: the force pass's own-particle traffic plus the read and clear of the 64-bit
# fixed-point force/torque sums the pair kernels accumulate (48 + 48 B)
BYTES_EPILOGUE = BYTES_FORCE + 96
# measured DRAM bytes per particle and launch (ncu dram__bytes_read + dram__bytes_write, one kernel per
# capture, 160 replicas aged 2,000 steps, state larger than L2; profiles/step_dram_traffic_c4x160_aged.md),
# scaled by the particle count.  Force pass: fused pair finding 113.6 + patch pairs 113.0 + epilogue 227.0 (the
# pair-force kernel has no pairs to take).  Scatter: 235.2.
TRAFFIC_PER_PARTICLE = {"force": 453.6, "scatter": 235.2}
# the end-to-end leg: a fixed number of steps, whatever --steps is
E2E_STEPS = 1000   # Condensate::run uploads once per run of 10^4 steps; a tenth of that per e2e leg
# CPU legs (reference arm and cpu_baseline): the same replica sample, processed largest first, one replica
# per host thread at a time
CPU_SAMPLE_REPLICAS = 128


def metric_of(args) -> str:
    if args.single_bond:
        return "particle-steps/s on 1 GB300, single-bond-per-patch step (run_singlebond), batched FP32"
    return METRIC


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
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
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return rank, world, local


def dist_barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def dist_max(world, value: float) -> float:
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_replicas(n_replicas: int, rank: int, world: int) -> list:
    """Replica indices a rank owns when a fixed set is split (contiguous blocks)."""
    per = n_replicas // world
    extra = n_replicas % world
    start = rank * per + min(rank, extra)
    return list(range(start, start + per + (1 if rank < extra else 0)))


def make_workload(args, rank: int, gen=None):
    """The bench workload; ``gen`` (the oracle's generators for the CPU legs) supplies the seeded inputs."""
    from mtcode_gb300 import workloads
    if args.workload == "c4":
        return workloads.patchy_c4(seed=args.seed + rank, n_replicas=args.replicas, gen=gen)
    return workloads.WORKLOADS[args.workload](seed=args.seed + rank, gen=gen)


# ---------------------------------------------------------------- CPU side (oracle port)
def cpu_info() -> dict:
    """Host facts the CPU figures depend on: logical cores, CPU model, and the long double format (the
    reference's angular factors run in long double; on aarch64 that is IEEE binary128 in software)."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.split(":")[0].strip() == "Model name":
                model = (model + " / " if model else "") + ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    if not model:
        try:
            for ln in Path("/proc/cpuinfo").read_text().splitlines():
                if ln.lower().startswith(("model name", "cpu part")):
                    model = ln.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    nm = np.finfo(np.longdouble).nmant
    ld = {112: "IEEE binary128 (software arithmetic)", 63: "x87 80-bit extended (hardware)",
          52: "same as double"}.get(nm, f"{nm}-bit mantissa")
    return {"nproc": os.cpu_count(), "cpu_model": model, "machine": os.uname().machine, "long_double": ld}


def cpu_sample_rate(W, n_reps: int, steps: int, threads: int, single_bond=None) -> dict:
    """Oracle port of the reference step on a bounded sample: the first n_reps replicas, `steps` steps
    each, one replica per host thread (the reference's own scale-out is one process per system), largest
    replica first.  With single_bond = (on, off): the run_singlebond loop with BindingModelSingle(on, off)."""
    from oracle import pyoracle as po
    po.orc()
    reps = W.replicas[:n_reps]
    offs = np.concatenate([[0], np.cumsum([r.n for r in W.replicas])])

    def one(r):
        spec = reps[r]
        sysm = po.System(spec)
        a, b = offs[r], offs[r + 1]
        st = dict(x=np.ascontiguousarray(W.x[a:b]), p=np.zeros((spec.n, 3)), Lb=np.zeros((spec.n, 3)),
                  Q=np.ascontiguousarray(W.Q[a:b]))
        if single_bond:
            npatch = sysm.total_patches()
            st.update(Ft=np.zeros((spec.n, 3)), Tt=np.zeros((spec.n, 3)),
                      boundto=np.zeros(npatch, dtype=np.intc), isbound=np.zeros(npatch, dtype=np.uint8))
            bind = po.binding_single(*single_bond)
            sysm.run_singlebond(st, bind, 0, sysm.default_max_ang(), init=True, noise_mode=2, seed=spec.seed,
                                replica=r, init_draw=0)
            t0 = time.perf_counter()
            sysm.run_singlebond(st, bind, steps, sysm.default_max_ang(), noise_mode=2, seed=spec.seed, replica=r,
                                draw0=1)
            return spec.n * steps, time.perf_counter() - t0
        st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"])
        t0 = time.perf_counter()
        sysm.run(st, steps, noise_mode=2, seed=spec.seed, replica=r, draw0=1, check_skin=False)
        return spec.n * steps, time.perf_counter() - t0

    order = sorted(range(len(reps)), key=lambda r: -reps[r].n)   # longest first: balanced threads
    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        res = list(ex.map(one, order))
    wall = time.perf_counter() - t0
    ps = sum(r[0] for r in res)
    cpu_s = sum(r[1] for r in res)
    return {"value": ps / wall, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{len(reps)} of {len(W.replicas)} replicas ({ps // steps} particles) x {steps} steps from the "
                      f"seeded start, one replica per thread (largest first), {cpu_s:.1f} s of CPU work"
                      + (" (run_singlebond loop)" if single_bond else "")}


def cpu_baseline_line(W, steps: int, single_bond=None) -> dict:
    """cpu_baseline: the sample on every host thread, plus a 1-thread figure on its first 4 replicas."""
    threads = os.cpu_count() or 1
    cb = cpu_sample_rate(W, min(len(W.replicas), CPU_SAMPLE_REPLICAS), steps, threads, single_bond)
    one = cpu_sample_rate(W, min(len(W.replicas), 16), 3, 1, single_bond)
    cb["one_thread"] = {"value": one["value"], "sample": one["sample"]}
    cb.update(cpu_info())
    cb["note"] = ("oracle port of the reference step (FP64, long double angular factors like the reference), "
                  "timed instead of the reference's own build, whose sources do not travel to the GPU host")
    return cb


def run_reference(args, rank, world):
    """Reference arm: the oracle port of the reference's CPU step (the reference's own build cannot travel
    to the GPU host), all host threads, on the same replica sample as the cpu_baseline leg.  The workload is
    built with the oracle's generators: nothing of the product library is loaded."""
    if rank != 0:
        return
    from oracle import pyoracle as po
    W = make_workload(args, 0, gen=po.Generators)
    threads = os.cpu_count() or 1
    cpu_sample_rate(W, min(len(W.replicas), threads), max(1, args.warmup), threads, args.single_bond)  # warm-up
    steps = max(1, args.steps)
    t0 = time.perf_counter()
    cb = cpu_baseline_line(W, steps, args.single_bond)
    elapsed = time.perf_counter() - t0
    value = cb["value"]
    line = {"metric": metric_of(args), "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": f"{args.workload}: {len(W.replicas)} patchy replicas, {W.n_total} particles",
                       "sample": cb["sample"], "state_age_steps": 0},
            "cpu_baseline": cb,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- GPU side
def run_gpu(args, rank, world, local):
    import torch
    from mtcode_gb300 import LangevinNVTRGPU

    torch.cuda.set_device(local)
    W = make_workload(args, rank)
    n = W.n_total
    z = np.zeros((n, 3))
    s = LangevinNVTRGPU(W.replicas, precision=args.precision, device=local)
    if args.single_bond:
        from mtcode_gb300.system import binding_single
        s.set_single_bond(binding_single(*args.single_bond))
    s.initialize(W.x, z, z, W.Q)
    s.init_forces()
    # untimed equilibration: the timed steps see the bonded steady state, not the random start
    s.step(args.equilibrate)
    # launch shapes of the pair pipeline: the autotuner (or this device's cached choice for this workload)
    from mtcode_gb300 import tuning
    tune = tuning.tuned(s, f"{args.workload}|single_bond={args.single_bond}", device=local) if args.tune else None
    s.step(max(args.warmup, 3))
    s.sync()
    stream = torch.cuda.ExternalStream(s.stream, device=torch.device("cuda", local))
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)

    # ---- device-resident timed region
    dist_barrier(world)
    torch.cuda.synchronize()
    l0 = s.launches
    with ClockSampler(local) as clk:
        ev0.record(stream)
        s.step(args.steps)
        ev1.record(stream)
        ev1.synchronize()
        torch.cuda.synchronize()
    dist_barrier(world)
    launches = s.launches - l0
    ms = ev0.elapsed_time(ev1)
    ms = dist_max(world, ms)
    s.sync()
    value = world * n * args.steps / (ms / 1e3)

    # ---- per-kernel device times (instrumented steps, same stream) -> roofline of the dominant kernel
    prof_steps = max(5, min(50, args.steps // 4))
    prof = s.step_profile(prof_steps)
    # slots of the step's passes; the pipeline's per-kernel slots split the force pass
    passes = ["scan_reduce", "scan_top", "scan_down", "scatter", "force"]
    if args.single_bond:
        passes += ["bind_begin", "bind_decide"]
    sub = {k: prof[k] / prof_steps for k in ("pairfind", "pairforce", "patch_pairs", "epilogue") if prof.get(k, 0) > 0}
    prof = {k: prof[k] for k in passes}
    total_prof = sum(prof.values())
    per_launch = {k: v / prof_steps for k, v in prof.items()}
    dominant = max(per_launch, key=per_launch.get)
    bytes_per = {"force": BYTES_FORCE * n, "scatter": BYTES_SCATTER * n}
    pk = peaks()
    alg = bytes_per.get(dominant)
    achieved = alg / (per_launch[dominant] / 1e3) / 1e9 if alg else None
    traffic = TRAFFIC_PER_PARTICLE.get(dominant) if not args.single_bond else None
    roofline = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                "frac": (achieved / pk["hbm_gbs"]) if achieved else None,
                "traffic": traffic * n if traffic else None,
                "traffic_source": "ncu DRAM bytes per particle at 160 replicas (bonded state), scaled" if traffic else None,
                "peak_source": pk["source"],
                "kernel_ms_per_step": {k: round(v, 5) for k, v in per_launch.items()},
                "share": {k: round(v / total_prof, 4) for k, v in prof.items()},
                "algorithmic_bytes_per_particle": {"force": BYTES_FORCE, "scatter": BYTES_SCATTER}}
    if sub:
        roofline["force_kernels_ms_per_step"] = {k: round(v, 5) for k, v in sub.items()}
    if "scatter" in per_launch:
        a2 = BYTES_SCATTER * n / (per_launch["scatter"] / 1e3) / 1e9
        roofline["scatter_gbs"] = a2
        roofline["scatter_frac"] = a2 / pk["hbm_gbs"]
    if "epilogue" in sub:
        a3 = BYTES_EPILOGUE * n / (sub["epilogue"] / 1e3) / 1e9
        roofline["epilogue_gbs"] = a3
        roofline["epilogue_frac"] = a3 / pk["hbm_gbs"]
        roofline["epilogue_bytes_per_particle"] = BYTES_EPILOGUE

    # ---- end to end through the C ABI with host buffers
    # three repetitions, the median reported (the one-time host copies of ~1 GB each way vary with the shared
    # host's load: 5-6 ms each when it is quiet, several times that at times); all three are in the line
    reps = sorted((run_e2e(s, W, args, stream, ev0, ev1) for _ in range(3)), key=lambda e: e["value"])
    e2e = dict(reps[1])
    e2e["repetitions"] = [{k: r[k] for k in ("value", "upload_ms", "steps_ms_per_step", "download_ms")} for r in reps]
    e2e["value"] = dist_max(world, -e2e["value"]) * -1 if world > 1 else e2e["value"]
    # the same with a synchronous temperature read after every step, for comparison
    sync = run_e2e(s, W, args, stream, ev0, ev1, batched=False)
    e2e["per_step_sync"] = {k: sync[k] for k in ("value", "upload_ms", "steps_ms_per_step", "download_ms", "what")}

    # ---- plain FP64 single-system path on a sample of the same replicas
    plain = run_plain_fp64(args, local) if args.plain_fp64 and rank == 0 else None

    cpu = None
    s_launch = s.launch_config
    s.close()
    if rank == 0 and world == 1 and args.cpu_baseline:
        cpu = cpu_baseline_line(W, args.cpu_steps, args.single_bond)

    if rank == 0:
        line = {"metric": metric_of(args), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "fp32" if args.precision == "fp32" else "f64",
                "data": "synthetic (seeded)",
                "config": {"workload": f"{args.workload}: {len(W.replicas)} patchy replicas, {n} particles per GPU",
                           "replicas": len(W.replicas), "particles_per_gpu": n, "precision": args.precision,
                           "l2": "inputs larger than L2 (state ~%d MB per GPU)" % (n * 250 // 2 ** 20),
                           "parallelism": f"replicas x{world}",
                           "state_age_steps": args.equilibrate + max(args.warmup, 3),
                           "single_bond": (f"run_singlebond force pass, BindingModelSingle{tuple(args.single_bond)}"
                                           if args.single_bond else None)},
                "launch_config": s_launch, "tuning": ({k: v for k, v in tune.items() if k != "launch_config"}
                                                        if tune else "defaults (--no-tune)"),
                "gpu_launches": launches, "clocks": clk.summary(), "roofline": roofline, "e2e": e2e,
                "cpu_baseline": cpu, "plain_fp64": plain}
        print(json.dumps(line), flush=True)


def run_e2e(s, W, args, stream, ev0, ev1, batched: bool = True) -> dict:
    """The metric through the C ABI with host buffers: the FP64 state uploaded from pinned memory, a fixed number
    of steps each followed by its temperature read back to the host (Condensate::run measures it every step), the
    state downloaded into pinned memory.  batched: mtg_step_temperatures (every step's sums reach pinned host
    memory as that step completes, one synchronisation at the end); else mtg_step(1) + mtg_temperature per step
    (a synchronisation after every step)."""
    import torch
    n = W.n_total
    R = len(W.replicas)
    state = s.get_state()
    pinned = {k: torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy() for k, v in state.items()}
    for k in pinned:
        pinned[k][...] = state[k]
    out = {k: torch.empty(v.shape, dtype=torch.float64, pin_memory=True).numpy() for k, v in state.items()}
    k_e2e = E2E_STEPS
    ev_up, ev_down = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ev0.record(stream)
    s.initialize(pinned["x"], pinned["p"], pinned["Lb"], pinned["Q"], pinned["Ft"], pinned["Tt"])
    ev_up.record(stream)
    if batched:
        temps = s.step_temperatures(k_e2e)
    else:
        temps = np.empty((k_e2e, R, 6))
        for i in range(k_e2e):
            s.step(1)
            temps[i] = s.measured_temperature()
    ev_down.record(stream)
    st = s.get_state(out)
    ev1.record(stream)
    ev1.synchronize()
    wall = time.perf_counter() - t0
    if temps.shape != (k_e2e, R, 6) or not np.isfinite(temps).all() or not np.isfinite(st["x"]).all():
        raise RuntimeError("e2e: non-finite temperatures or state")
    h2d = n * (3 + 3 + 3 + 9 + 3 + 3) * 8
    d2h_state = n * (3 + 3 + 3 + 9 + 3 + 3) * 8
    what = ("mtg_set_state (host FP64 state) + mtg_step_temperatures (each step's temperatures summed on the "
            "device and read back to pinned host memory) + mtg_get_state at the end" if batched else
            "mtg_set_state (host FP64 state) + per step: mtg_step(1) + mtg_temperature (synchronous read-back) "
            "+ mtg_get_state at the end")
    return {"value": n * k_e2e / wall, "unit": UNIT, "h2d_bytes_per_step": h2d / k_e2e,
            "d2h_bytes_per_step": R * 6 * 8 + d2h_state / k_e2e, "steps": k_e2e,
            "upload_ms": ev0.elapsed_time(ev_up), "download_ms": ev_down.elapsed_time(ev1),
            "steps_ms_per_step": ev_up.elapsed_time(ev_down) / k_e2e, "wall_ms": 1e3 * wall, "what": what}


def run_plain_fp64(args, device) -> dict:
    """The plain FP64 single-system path: one system per FP64 handle (the pair pipeline in FP64), at the
    single-system configurations' sizes -- 4,096 tetrahedral particles at phi 0.10 and the 1,048,576-particle
    crowded condensate at phi 0.25 -- each from its seeded start, `plain_steps` steps after 3 untimed ones."""
    from mtcode_gb300 import LangevinNVTRGPU, workloads
    import torch
    out = {}
    for name, build in (("c1", workloads.patchy_c1), ("c3", workloads.patchy_c3)):
        W = build(seed=args.seed)
        spec = W.replicas[0]
        steps = args.plain_steps
        with LangevinNVTRGPU([spec], precision="fp64", device=device, track_displacement=False) as s:
            if args.single_bond:
                from mtcode_gb300.system import binding_single
                s.set_single_bond(binding_single(*args.single_bond))
            z = np.zeros((spec.n, 3))
            s.initialize(W.x, z, z, W.Q)
            s.init_forces()
            s.step(3)
            s.sync()
            stream = torch.cuda.ExternalStream(s.stream)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.step(steps)
            e1.record(stream)
            e1.synchronize()
            sec = e0.elapsed_time(e1) / 1e3
        out[name] = {"value": spec.n * steps / sec, "unit": UNIT, "dtype": "f64", "particles": spec.n,
                     "ms_per_step": 1e3 * sec / steps}
    out["sample"] = (f"single systems, each alone in its own FP64 handle (pair pipeline in FP64), {args.plain_steps} "
                     "steps from the seeded start: c1 = 4,096 tetrahedral patchy particles at phi 0.10, c3 = "
                     "1,048,576 particles (1:3 patchy:crowder) at phi 0.25")
    out["value"] = max(out["c1"]["value"], out["c3"]["value"])
    out["unit"] = UNIT
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["mtcode", "reference"], default="mtcode")
    ap.add_argument("--workload", default="c4", choices=["c1", "c2", "c3", "c4"])
    ap.add_argument("--replicas", type=int, default=512)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--cpu-steps", type=int, default=10)
    ap.add_argument("--no-tune", dest="tune", action="store_false",
                    help="keep the default launch shapes instead of the autotuner's")
    ap.add_argument("--equilibrate", type=int, default=2000,
                    help="untimed steps before the timed region (the bonded steady state)")
    ap.add_argument("--no-plain-fp64", dest="plain_fp64", action="store_false")
    ap.add_argument("--plain-steps", type=int, default=20)
    ap.add_argument("--single-bond", nargs=2, type=float, metavar=("ON", "OFF"), default=None,
                    help="time the single-bond-per-patch step (Condensate::run_singlebond's force pass) with "
                         "BindingModelSingle(ON, OFF) instead of the full Kern-Frenkel step")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, world, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_gpu(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
