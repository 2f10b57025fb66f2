"""Run a seeded workload for a number of steps and report the time per step.

    python -m mtcode_gb300.run --workload c4 --replicas 48 --steps 4 [--precision fp32] [--profile]

Used for quick timing and as the target of profiler captures (it launches the same kernels as the
benchmark, on a workload of the chosen size).  ``--save-state F`` writes the state after the timed steps to F
(.npz; in single-bond mode with the bond state) and ``--load-state F`` starts from it instead of the seeded
start, so a capture of a few launches can see an aged (bonded) state without running the steps that aged it.
"""
from __future__ import annotations

import argparse
import time

import numpy as np

from . import LangevinNVTRGPU, workloads


def main() -> None:
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--workload", default="c4", choices=sorted(workloads.WORKLOADS))
    ap.add_argument("--replicas", type=int, default=512, help="replicas of the c4 / c5 workloads (c5: 64 by default)")
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--precision", choices=["fp32", "fp64"], default="fp32")
    ap.add_argument("--kernel", choices=["pairs", "tiled", "per_particle"], default="pairs")
    ap.add_argument("--profile", action="store_true", help="also print per-kernel device times")
    ap.add_argument("--skin", type=float, default=0.0, help="neighbour skin (sigma); 0 rebuilds cells every step")
    ap.add_argument("--single-bond", nargs=2, type=float, metavar=("ON", "OFF"), default=None,
                    help="single-bond-per-patch mode (run_singlebond) with BindingModelSingle(ON, OFF)")
    ap.add_argument("--launch", default=None,
                    help="pair-pipeline launch shapes as pairfind_threads,pairforce_blocks_per_sm,"
                         "patch_blocks_per_sm,epilogue_threads,fused_pairs (default: the library's)")
    ap.add_argument("--tune", action="store_true", help="run the launch-shape autotuner before timing")
    ap.add_argument("--save-state", default=None, help="write the final state (x, p, Lb, Q, Ft, Tt) to this .npz")
    ap.add_argument("--load-state", default=None, help="start from a state written by --save-state")
    args = ap.parse_args()
    if args.workload == "c4":
        W = workloads.patchy_c4(seed=args.seed, n_replicas=args.replicas)
    elif args.workload == "c5":
        W = workloads.polymer_c5(seed=args.seed, n_replicas=min(args.replicas, 64))
    else:
        W = workloads.WORKLOADS[args.workload](seed=args.seed)
    n = W.n_total
    z = np.zeros((n, 3))
    with LangevinNVTRGPU(W.replicas, precision=args.precision, force_kernel=args.kernel, neighbor_skin=args.skin) as s:
        if args.load_state:
            st = np.load(args.load_state)
            s.initialize(st["x"], st["p"], st["Lb"], st["Q"], st["Ft"], st["Tt"])
        else:
            s.initialize(W.x, z, z, W.Q)
        if W.bonds is not None:
            s.set_bonds(W.bonds, W.bond_k, W.bond_r0)
        if args.single_bond:
            from .system import binding_single
            s.set_single_bond(binding_single(*args.single_bond))
            if args.load_state and "boundto" in st:
                s.set_bind_state(st["boundto"], st["isbound"])
        if args.launch:
            keys = ("pairfind_threads", "pairforce_blocks_per_sm", "patch_blocks_per_sm", "epilogue_threads",
                    "fused_pairs")
            s.launch_config = dict(zip(keys, (int(v) for v in args.launch.split(","))))
        s.init_forces()
        if args.tune:
            cfg, ms = s.autotune(5)
            print(f"autotune: {cfg} at {ms:.3f} ms/step", flush=True)
        s.sync()
        t0 = time.perf_counter()
        s.step(args.steps)
        s.sync()
        dt = time.perf_counter() - t0
        line = f"{W.name}: {len(W.replicas)} replicas, {n} particles, {args.steps} steps, {1e3 * dt / args.steps:.3f} ms/step, " \
               f"{n * args.steps / dt:.3e} particle-steps/s"
        if args.skin > 0:
            line += f", {s.rebuilds} list builds"
        if args.single_bond:
            line += f", {int(s.get_bind_state()[1].sum())} bound patches"
        if args.profile:
            prof = s.step_profile(max(1, args.steps))
            line += " | " + " ".join(f"{k}={v / max(1, args.steps):.3f}ms" for k, v in prof.items())
        print(line, flush=True)
        if args.save_state:
            state = s.get_state()
            if args.single_bond:   # the bond state too
                state["boundto"], state["isbound"] = s.get_bind_state()
            np.savez(args.save_state, **state)


if __name__ == "__main__":
    main()
