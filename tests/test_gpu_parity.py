"""GPU parity: the CUDA path, called through the C ABI, against the oracle / reference fixtures.

Tolerances (stated once, used below):
  pair sets          bit-exact (FP64 inclusion test on identical coordinates) -- FP32 and FP64 builds
  forces, torques    relative RMS error ||F - F_ref|| / ||F_ref|| over all particles:
                       FP64 build <= 1e-12, FP32 build <= 1e-5 (the stated force-error target);
                     worst particle |F_i - F_ref,i| / rms|F_ref|: FP64 <= 1e-11, FP32 <= 1e-4
  trajectories       FP64 build, 100 steps: 1e-9 relative to the state's scale
                     FP32 build, 100 steps: 2e-4 absolute on positions and 1e-3 on the carried state
                     (single-precision rounding, ~6e-8, amplified by 100 steps of the stiff WCA core)
  noise-free relaxations (kT = 0) in FP32: "FP32 shadow" bound.  A step moves a particle by ~1e-3
                     sigma while float spacing at x ~ 5-50 is 5e-7-4e-6, so every drift increment is
                     rounded at 1e-4-1e-3 relative and the stiff WCA core feeds that back.  The oracle is
                     rerun with one-ulp (2^-23) random errors added to its state and float32 storage after
                     every step (four seeds); the GPU's FP32 error must stay within 20x the largest
                     deviation of those FP32-quality runs (or the FP32 floor above): a four-run
                     ensemble underestimates the worst case, measured ratios are 1-10.
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU
from oracle import pyoracle as po
from tests._util import force_errors, load, sorted_pairs, spec_from

pytestmark = pytest.mark.gpu
# fp32 / fp64: the default pair pipeline in each precision; fp32-tiled: the tile kernel; fp64-pp: the FP64
# one-thread-per-particle kernel
PRECISIONS = ["fp32", "fp64", "fp32-tiled", "fp64-pp"]


def make(spec, x, Q, precision, p=None, Lb=None, Ft=None, Tt=None):
    n = spec.n
    if precision == "fp32-tiled":
        s = LangevinNVTRGPU([spec], precision="fp32", force_kernel="tiled")
    elif precision == "fp64-pp":
        s = LangevinNVTRGPU([spec], precision="fp64", force_kernel="per_particle")
    else:
        s = LangevinNVTRGPU([spec], precision=precision)
    z = np.zeros((n, 3))
    s.initialize(x, z if p is None else p, z if Lb is None else Lb, Q, Ft, Tt)
    return s


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", range(7))
def test_pair_sets_bit_exact(k, precision):
    d = load(f"pairs_{k}.npz")
    spec = spec_from(d)
    with make(spec, d["x"], np.tile(np.eye(3).ravel(), (spec.n, 1)), precision) as s:
        got = sorted_pairs(s.calculatepairs_parallel(float(d["rc"])))
    assert np.array_equal(got, d["pairs"])


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", range(5))
def test_forces_and_torques(k, precision):
    d = load(f"forces_{k}.npz")
    spec = spec_from(d)
    with make(spec, d["x"], d["Q"], precision) as s:
        F, T = s.calculate_forces_and_torques3D()
    check_errors(F, d["F"], precision)
    check_errors(T, d["T"], precision)


def check_errors(a, b, precision, flipped_ok=0.0):
    e = force_errors(a, b)
    rms_tol, max_tol = (1e-12, 1e-11) if precision.startswith("fp64") else (1e-5, 1e-4)
    assert e["rms"] <= rms_tol, e
    if flipped_ok == 0.0:
        assert e["max"] <= max_tol, e


@pytest.mark.parametrize("precision", PRECISIONS)
def test_forces_fresh_inputs_vs_oracle(precision):
    """Larger random systems (not in the fixtures), each model, against the oracle."""
    from mtcode_gb300.system import random_positions, random_rotations
    from mtcode_gb300.workloads import box_for, crowded_model, tubulin_model
    from mtcode_gb300.system import PatchModelSpec, ReplicaSpec
    for n, model in ((4000, PatchModelSpec.tetrahedral(4000, 8.0, 1.2, math.acos(0.9))),
                     (4000, tubulin_model(4000)), (4000, crowded_model(1000, 4000))):
        spec = ReplicaSpec(n=n, box=box_for(n, 0.3), model=model)
        x = random_positions(n, spec.box, True, 0.95, 11).astype(np.float32).astype(np.float64)
        Q = random_rotations(n, 12).astype(np.float32).astype(np.float64)
        Fo, To = po.System(spec).forces(x, Q)
        with make(spec, x, Q, precision) as s:
            F, T = s.calculate_forces_and_torques3D()
        check_errors(F, Fo, precision)
        check_errors(T, To, precision)


def _run_gpu(d, precision, nsteps=None):
    spec = spec_from(d)
    n = spec.n
    nsteps = int(d["nsteps"]) if nsteps is None else nsteps
    s = make(spec, d["x0"], d["Q0"], precision)
    mode = str(d["noise_mode"]) if "noise_mode" in d else "off"
    if mode == "shared":
        noise = po.philox_noise(n * (nsteps + 1), int(d["noise_seed"]), 0, 0).reshape(nsteps + 1, n, 6)
        s.init_forces(np.ascontiguousarray(noise[0]))
        s.step(nsteps, np.ascontiguousarray(noise[1:]))
    else:
        s.init_forces()
        if spec.kT == 0:
            s.step(nsteps)
        else:
            raise AssertionError("unexpected fixture")
    st = s.get_state()
    s.close()
    return st


def fp32_shadow_error(d, nsteps, rc, seeds=(1, 2, 3, 4)) -> dict:
    """Largest deviation from the FP64 reference trajectory among oracle runs of FP32 quality: after
    every step each state value gets a random relative error of up to one float32 ulp (2^-23) and is
    stored as float32.  This is the spread that single precision alone produces on this trajectory."""
    spec = spec_from(d)
    n = spec.n
    sysm = po.System(spec)
    worst = {}
    for sd in seeds:
        rng = np.random.default_rng(sd)
        st = dict(x=d["x0"].copy(), p=np.zeros((n, 3)), Lb=np.zeros((n, 3)), Q=d["Q0"].copy())
        st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"], None, rc)
        for _ in range(nsteps):
            for k in st:
                noisy = st[k] * (1 + 2.0 ** -23 * rng.uniform(-1, 1, st[k].shape))
                st[k][...] = noisy.astype(np.float32)
            sysm.run(st, 1, noise_mode=0, rc=rc)
        for k in st:
            worst[k] = max(worst.get(k, 0.0), float(np.abs(st[k] - d["final_" + k]).max()))
    return worst


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", range(4))
def test_trajectories_100_steps(k, precision):
    d = load(f"traj_{k}.npz")
    st = _run_gpu(d, precision)
    noise_free = str(d["noise_mode"]) == "off"
    spread = fp32_shadow_error(d, int(d["nsteps"]), float(d["rc"])) if (noise_free and not precision.startswith("fp64")) else None
    for key in ("x", "p", "Lb", "Q", "Ft", "Tt"):
        ref = d["final_" + key]
        scale = max(1.0, float(np.abs(ref).max()))
        err = float(np.abs(st[key] - ref).max())
        if precision.startswith("fp64"):
            assert err <= 1e-9 * scale, (key, err)
        else:
            tol = 2e-4 if key == "x" else 1e-3 * scale
            if spread is not None:
                tol = max(tol, 20 * spread[key])
            assert err <= tol, (key, err, tol)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", range(6))
def test_two_particle_torque_cases(k, precision):
    d = load(f"torque_{k}.npz")
    spec = spec_from(d)
    with make(spec, d["x0"], d["Q0"], precision) as s:
        s.init_forces()
        s.step(int(d["nsteps"]))
        st = s.get_state()
    spread = fp32_shadow_error(d, int(d["nsteps"]), float(d["rc"])) if not precision.startswith("fp64") else None
    for key in ("x", "Q", "p", "Lb"):
        ref = d["final_" + key]
        err = float(np.abs(st[key] - ref).max())
        if precision.startswith("fp64"):
            assert err <= 1e-10 * max(1.0, float(np.abs(ref).max())), (key, err)
        else:
            tol = max(2e-5, 20 * spread[key])
            assert err <= tol, (key, err, tol)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_philox_noise_matches_oracle(precision):
    """Isolated particles (no forces): F~ = Q^T (Rt xi), T~ = Rr xi_r with p = L = 0 exposes the draw."""
    n = 64
    from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_rotations
    spec = ReplicaSpec(n=n, box=200.0, model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9)), kT=1.3,
                       seed=0xDEADBEEF12345)
    g = np.stack(np.meshgrid(np.arange(4), np.arange(4), np.arange(4), indexing="ij"), -1).reshape(-1, 3)
    x = 10.0 + 40.0 * g.astype(float)
    Q = random_rotations(n, 3).astype(np.float32).astype(np.float64)
    with make(spec, x, Q, precision) as s:
        s.draw = 5
        s.init_forces()
        st = s.get_state()
        assert s.draw == 6
    xi = po.philox_noise(n, spec.seed, 0, 5)
    Rt = math.sqrt(2 * spec.gamma * spec.kT / spec.dt)
    Rr = math.sqrt(2 * spec.gammar * spec.kT / spec.dt)
    Qm = Q.reshape(n, 3, 3)
    # F~ = Q^T (Rt xi): solve instead of multiplying by Q (the rounded Q is not exactly orthogonal)
    xi_t = np.linalg.solve(np.transpose(Qm, (0, 2, 1)), st["Ft"][..., None])[..., 0] / Rt
    xi_r = st["Tt"] / Rr
    tol = 1e-12 if precision.startswith("fp64") else 2e-6
    assert np.abs(xi_t - xi[:, :3]).max() <= tol
    assert np.abs(xi_r - xi[:, 3:]).max() <= tol
