"""GPU tests of the batched path: many uneven replicas in one handle.

  forces of every replica of a batch vs the oracle (the three FP32 force kernels, and both FP64 ones);
  a replica advanced inside a batch equals the same replica advanced alone (noise off);
  FP32 steps are bit-for-bit reproducible run to run (fixed-point force sums + counter-based noise);
  at the full batched size, Newton's third law holds exactly (the fixed-point pair sums cancel).
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU
from mtcode_gb300 import workloads
from oracle import pyoracle as po
from tests._util import force_errors

pytestmark = pytest.mark.gpu


def small_batch(seed=3, n_replicas=12, phi=0.15, kT=None):
    W = workloads.patchy_c4(seed=seed, n_replicas=n_replicas, n_min=200, n_max=6000, phi=phi)
    if kT is not None:
        for r in W.replicas:
            r.kT = kT
    W.x = W.x.astype(np.float32).astype(np.float64)
    W.Q = W.Q.astype(np.float32).astype(np.float64)
    return W


def offsets(W):
    return np.concatenate([[0], np.cumsum([r.n for r in W.replicas])])


@pytest.mark.parametrize("precision,kernel", [("fp32", "tiled"), ("fp32", "per_particle"), ("fp32", "pairs"),
                                              ("fp64", "pairs"), ("fp64", "per_particle")])
def test_batched_forces_vs_oracle(precision, kernel):
    W = small_batch(phi=0.3)
    z = W.zeros3()
    with LangevinNVTRGPU(W.replicas, precision=precision, force_kernel=kernel) as s:
        s.initialize(W.x, z, z, W.Q)
        F, T = s.calculate_forces_and_torques3D()
    off = offsets(W)
    for r, spec in enumerate(W.replicas):
        a, b = off[r], off[r + 1]
        Fo, To = po.System(spec).forces(W.x[a:b], W.Q[a:b])
        rms_tol = 1e-12 if precision == "fp64" else 1e-5
        assert force_errors(F[a:b], Fo)["rms"] <= rms_tol, r
        assert force_errors(T[a:b], To)["rms"] <= rms_tol, r


def test_tiled_and_per_particle_kernels_agree():
    W = small_batch(seed=5, phi=0.25)
    z = W.zeros3()
    out = {}
    for kernel in ("tiled", "per_particle", "pairs"):
        with LangevinNVTRGPU(W.replicas, force_kernel=kernel) as s:
            s.initialize(W.x, z, z, W.Q)
            out[kernel] = s.calculate_forces_and_torques3D()
    # each kernel is within 1e-5 of the FP64 oracle (test_gpu_parity); two FP32 kernels that round
    # their pair terms differently agree to a few 1e-6
    for other in ("per_particle", "pairs"):
        assert force_errors(out["tiled"][0], out[other][0])["rms"] <= 5e-6
        assert force_errors(out["tiled"][1], out[other][1])["rms"] <= 5e-6


@pytest.mark.parametrize("kernel", ["tiled", "per_particle", "pairs"])
def test_replica_in_batch_equals_replica_alone(kernel):
    W = small_batch(seed=7, n_replicas=6, kT=0.0)
    z = W.zeros3()
    with LangevinNVTRGPU(W.replicas, force_kernel=kernel) as s:
        s.initialize(W.x, z, z, W.Q)
        s.init_forces()
        s.step(25)
        batch = s.get_state()
    off = offsets(W)
    for r in (0, 3, 5):
        a, b = off[r], off[r + 1]
        zz = np.zeros((b - a, 3))
        with LangevinNVTRGPU([W.replicas[r]], force_kernel=kernel) as s1:
            s1.initialize(W.x[a:b], zz, zz, W.Q[a:b])
            s1.init_forces()
            s1.step(25)
            alone = s1.get_state()
        for key in ("x", "p", "Lb", "Q"):
            assert np.array_equal(batch[key][a:b], alone[key]), (r, key)


@pytest.mark.parametrize("kernel", ["tiled", "pairs"])
def test_fp32_steps_are_bitwise_reproducible(kernel):
    W = small_batch(seed=11, n_replicas=8)
    z = W.zeros3()
    finals = []
    for _ in range(2):
        with LangevinNVTRGPU(W.replicas, force_kernel=kernel) as s:
            s.initialize(W.x, z, z, W.Q)
            s.init_forces()
            s.step(40)
            finals.append(s.get_state())
    for key in finals[0]:
        assert np.array_equal(finals[0][key], finals[1][key]), key


@pytest.mark.parametrize("kernel", ["tiled", "pairs"])
def test_full_size_batch_newton_third_law_and_finiteness(kernel):
    """The benchmark workload (512 replicas, ~5 M particles): per replica the fixed-point pair sums
    cancel exactly, so the total force is zero to the fixed-point resolution after the float round."""
    W = workloads.patchy_c4(seed=0)
    z = W.zeros3()
    with LangevinNVTRGPU(W.replicas, force_kernel=kernel) as s:
        s.initialize(W.x, z, z, W.Q)
        F, T = s.calculate_forces_and_torques3D()
        s.init_forces()
        s.step(20)
        st = s.get_state()
        assert s.flags & 1 == 0
    off = offsets(W)
    sums = np.array([F[off[r]:off[r + 1]].sum(0) for r in range(len(W.replicas))])
    # each particle's force is one float rounding of an exact integer sum: |sum| <= n * ulp(|F|max)
    for r in range(len(W.replicas)):
        Fr = F[off[r]:off[r + 1]]
        bound = len(Fr) * np.spacing(np.float32(np.abs(Fr).max())) + 1e-6
        assert np.abs(sums[r]).max() <= bound, r
    assert np.isfinite(st["x"]).all() and np.isfinite(st["p"]).all() and np.isfinite(st["Lb"]).all()
    for r, spec in enumerate(W.replicas):
        xr = st["x"][off[r]:off[r + 1]]
        assert (xr >= 0).all() and (xr <= spec.box).all()


@pytest.mark.parametrize("kernel,single_bond,per_step", [("pairs", False, 9), ("tiled", False, 5),
                                                         ("per_particle", False, 5), ("pairs", True, 15)])
def test_launch_count_per_step(kernel, single_bond, per_step):
    """mtg_launches counts every kernel a step replays: scans (3) + scatter + the force pass (pair pipeline:
    reset, pairfind, pairforce, patch pairs, epilogue; single-bond mode: bind begin, the edge pass, its FP64
    recheck, the three decision kernels and the bound-pair pass instead of the patch pairs), plus one launch
    per mtg_step call
    that sets the device's noise-draw counter."""
    from mtcode_gb300.system import binding_single
    W = small_batch(seed=6, n_replicas=4)
    z = W.zeros3()
    with LangevinNVTRGPU(W.replicas, force_kernel=kernel) as s:
        s.initialize(W.x, z, z, W.Q)
        if single_bond:
            s.set_single_bond(binding_single(1.0, 0.1))
        s.init_forces()
        s.step(2)
        s.sync()
        l0 = s.launches
        s.step(5)
        s.sync()
        assert s.launches - l0 == 5 * per_step + 1
        assert s.flags == 0


def test_identical_replicas_in_batch_equal_each_alone():
    """A batch whose replicas share every pair constant (same size, box, model) takes the pair kernels'
    uniform form (no per-pair replica search); each replica still equals the same replica run alone."""
    from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
    n = 900
    box = workloads.box_for(n, 0.15)
    model = PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9))
    reps = [ReplicaSpec(n=n, box=box, model=model, kT=0.0, seed=40 + r) for r in range(3)]
    xs = [random_positions(n, box, True, 0.95, 50 + r) for r in range(3)]
    Qs = [random_rotations(n, 60 + r) for r in range(3)]
    x, Q = np.concatenate(xs), np.concatenate(Qs)
    z = np.zeros((3 * n, 3))
    with LangevinNVTRGPU(reps, force_kernel="pairs") as s:
        s.initialize(x, z, z, Q)
        s.init_forces()
        s.step(25)
        batch = s.get_state()
        assert s.flags == 0
    for r in range(3):
        zz = np.zeros((n, 3))
        with LangevinNVTRGPU([reps[r]], force_kernel="pairs") as s1:
            s1.initialize(xs[r], zz, zz, Qs[r])
            s1.init_forces()
            s1.step(25)
            alone = s1.get_state()
        for key in ("x", "p", "Lb", "Q"):
            assert np.array_equal(batch[key][r * n:(r + 1) * n], alone[key]), (r, key)


def test_more_replicas_than_the_slot_table_holds():
    """65,537 replicas: past the 2-byte per-slot replica table (65,536 replicas), every kernel finds a slot's
    replica by binary search over the replica offsets; forces of sampled replicas against the oracle, then steps."""
    from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
    from mtcode_gb300.workloads import box_for
    n_rep, n = 65537, 4
    box = box_for(n, 0.1)
    model = PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9))
    reps = [ReplicaSpec(n=n, box=box, model=model, kT=1.0, seed=r) for r in range(n_rep)]
    x = np.concatenate([random_positions(n, box, True, 0.9, 10 + r) for r in range(n_rep)])
    x = x.astype(np.float32).astype(np.float64)
    Q = random_rotations(n * n_rep, 3).astype(np.float32).astype(np.float64)
    z = np.zeros((n * n_rep, 3))
    with LangevinNVTRGPU(reps, precision="fp32") as s:
        s.initialize(x, z, z, Q)
        F, T = s.calculate_forces_and_torques3D()
        for r in (0, 1, 32768, 65535, 65536):
            a, b = r * n, (r + 1) * n
            Fo, To = po.System(reps[r]).forces(x[a:b], Q[a:b])
            assert np.abs(F[a:b] - Fo).max() <= 1e-5 * max(1.0, np.abs(Fo).max()), r
            assert np.abs(T[a:b] - To).max() <= 1e-5 * max(1.0, np.abs(To).max()), r
        s.init_forces()
        s.step(5)
        st = s.get_state()
        assert np.isfinite(st["x"]).all() and s.flags == 0
