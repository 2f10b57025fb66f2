"""GPU parity: the CUDA path, called through the C ABI, against the oracle / reference fixtures.

Tolerances (stated once, used below):
  pair sets          bit-exact (FP64 inclusion test on identical coordinates) -- FP32 and FP64 builds
  forces, torques    FP64 build: per-particle relative error <= 1e-12 (floor |F| = 1 eps/sigma)
                     FP32 build: per-particle relative error <= 1e-5  (floor |F| = 1 eps/sigma)
  trajectories       FP64 build, 100 steps: 1e-9 relative to the state's scale
                     FP32 build, 100 steps: 2e-4 absolute on positions and 1e-3 on the carried state
                     (single-precision rounding, ~6e-8, amplified by 100 steps of the stiff WCA core)
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU
from oracle import pyoracle as po
from tests._util import load, rel_err, sorted_pairs, spec_from

pytestmark = pytest.mark.gpu
PRECISIONS = ["fp32", "fp64"]


def make(spec, x, Q, precision, p=None, Lb=None, Ft=None, Tt=None):
    n = spec.n
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
    tol = 1e-12 if precision == "fp64" else 1e-5
    assert rel_err(F, d["F"], floor=1.0) <= tol
    assert rel_err(T, d["T"], floor=1.0) <= tol


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
        tol = 1e-12 if precision == "fp64" else 1e-5
        # borderline pairs (within 1e-6 of a cone edge) may flip in FP32: allow at most 0.1% such particles
        bad = np.linalg.norm(F - Fo, axis=1) / np.maximum(np.linalg.norm(Fo, axis=1), 1.0) > tol
        assert bad.mean() <= (0.0 if precision == "fp64" else 1e-3), (precision, bad.sum())


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


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", range(4))
def test_trajectories_100_steps(k, precision):
    d = load(f"traj_{k}.npz")
    st = _run_gpu(d, precision)
    for key in ("x", "p", "Lb", "Q", "Ft", "Tt"):
        ref = d["final_" + key]
        scale = max(1.0, float(np.abs(ref).max()))
        err = float(np.abs(st[key] - ref).max())
        if precision == "fp64":
            assert err <= 1e-9 * scale, (key, err)
        else:
            tol = 2e-4 if key == "x" else 1e-3 * scale
            assert err <= tol, (key, err)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", range(6))
def test_two_particle_torque_cases(k, precision):
    d = load(f"torque_{k}.npz")
    spec = spec_from(d)
    with make(spec, d["x0"], d["Q0"], precision) as s:
        s.init_forces()
        s.step(int(d["nsteps"]))
        st = s.get_state()
    tol = 1e-10 if precision == "fp64" else 2e-5
    for key in ("x", "Q"):
        assert np.abs(st[key] - d["final_" + key]).max() <= tol, key
    for key in ("p", "Lb"):
        ref = d["final_" + key]
        assert np.abs(st[key] - ref).max() <= tol * max(1.0, np.abs(ref).max() * 1e3), key


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
    xi_t = np.einsum("nab,nb->na", Qm, st["Ft"]) / Rt
    xi_r = st["Tt"] / Rr
    tol = 1e-12 if precision == "fp64" else 2e-6
    assert np.abs(xi_t - xi[:, :3]).max() <= tol
    assert np.abs(xi_r - xi[:, 3:]).max() <= tol
