"""The loop body of Condensate::run one method at a time (the per-phase entry points and the C++ adapter's
reference-signature methods), against the oracle's restatement of the same methods.

  calculateforces                   MD::calculateforces(pairs, HSPotential)            (MD.cpp:1684-1764)
  calculate_forces_and_torques3D    adds patch forces and lab torques                  (LangevinR.cpp:911-1047)
  create_forces_and_torques_sphere  friction + noise, T to the body frame              (LangevinR.cpp:474-592)
  advancemom_halfstep               p += dt/2 F, L += dt/2 T                           (LangevinR.cpp:327-347)
  advance_pos                       x += dt/m p, wrap / reflect                        (Langevin.cpp:205-222)
  rotate                            free-rotor propagator                              (LangevinR.cpp:594-695)

Tolerances: FP64 builds 1e-12 relative (forces as relative RMS, the rest against the array's scale); FP32
builds 1e-5 relative RMS for forces and 2e-6 of the scale for the single-precision elementwise phases.  The
per-phase loop equals the fused step (mtg_step) to 1e-10 in FP64 after 20 steps with the same Philox draws, and
the adapter's loop (C++, reference signatures, patch model converted from a GeneralPatch-shaped object) follows
the oracle's loop with shared noise to 1e-9.
"""
import math
import subprocess

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU, _lib
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
from mtcode_gb300.workloads import box_for
from oracle import pyoracle as po
from tests._util import force_errors
from tests.test_adapter import BUILD, compile_driver

pytestmark = pytest.mark.gpu

KINDS = ["fp64", "fp32", "fp64-pp", "fp32-tiled"]


def handle(spec, kind):
    prec = "fp64" if kind.startswith("fp64") else "fp32"
    kernel = {"fp64-pp": "per_particle", "fp32-tiled": "tiled"}.get(kind, "pairs")
    return LangevinNVTRGPU([spec], precision=prec, force_kernel=kernel)


def system(n=1500, phi=0.3, seed=3):
    spec = ReplicaSpec(n=n, box=box_for(n, phi), model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9)),
                       kT=1.0, seed=seed)
    x = random_positions(n, spec.box, True, 0.95, seed + 1).astype(np.float32).astype(np.float64)
    Q = random_rotations(n, seed + 2).astype(np.float32).astype(np.float64)
    rng = np.random.default_rng(seed)
    p = rng.normal(size=(n, 3)).astype(np.float32).astype(np.float64)
    L = (0.3 * rng.normal(size=(n, 3))).astype(np.float32).astype(np.float64)
    return spec, x, Q, p, L


def close(a, b, kind, what, box=None):
    tol = 1e-12 if kind.startswith("fp64") else 2e-6
    scale = max(1.0, float(np.abs(b).max()))
    d = np.asarray(a) - b
    if box is not None:   # positions: a wrap decided differently at a face is one box length, not an error
        d -= box * np.round(d / box)
    assert float(np.abs(d).max()) <= tol * scale, (what, float(np.abs(d).max()))


@pytest.mark.parametrize("kind", KINDS)
def test_each_phase_against_the_oracle(kind):
    spec, x, Q, p, L = system()
    n = spec.n
    sysm = po.System(spec)
    with handle(spec, kind) as s:
        s.initialize(x, p, L, Q)
        # the force routines
        F = s.calculateforces()
        Fo = sysm.central_forces(x)
        rms = 1e-12 if kind.startswith("fp64") else 1e-5
        assert force_errors(F, Fo)["rms"] <= rms
        T = np.zeros((n, 3))
        s.add_patch_forces_and_torques(F, T)
        Fp, Tp = np.zeros((n, 3)), np.zeros((n, 3))
        sysm.patch_forces(x, Q, Fp, Tp)
        assert force_errors(F, Fo + Fp)["rms"] <= rms
        assert force_errors(T, Tp)["rms"] <= rms
        # friction and noise with a caller's R
        R = po.philox_noise(n, 99, 0, 5)
        Fo_t, To_t = Fo + Fp, Tp.copy()
        s.create_forces_and_torques_sphere(F, T, R)
        sysm.langevin_forces(p, L, Q, R, Fo_t, To_t)
        assert force_errors(F, Fo_t)["rms"] <= rms and force_errors(T, To_t)["rms"] <= rms
        st = s.get_state()
        assert force_errors(st["Ft"], Fo_t)["rms"] <= rms   # carried as the handle's F~, T~
        # the integrator phases, each from the handle's own state
        s.advancemom_halfstep(Fo_t, To_t)
        po_, Lo = p.copy(), L.copy()
        sysm.halfkick(po_, Lo, Fo_t, To_t)
        st = s.get_state()
        close(st["p"], po_, kind, "p after the half-kick")
        close(st["Lb"], Lo, kind, "L after the half-kick")
        xo, pm = st["x"].copy(), st["p"].copy()
        s.advance_pos()
        sysm.drift(xo, pm)
        st = s.get_state()
        close(st["x"], xo, kind, "x after advance_pos", box=spec.box)
        close(st["p"], pm, kind, "p after advance_pos")
        Lr, Qr = st["Lb"].copy(), st["Q"].copy()
        s.rotate()
        sysm.rotate(Lr, Qr)
        st = s.get_state()
        close(st["Lb"], Lr, kind, "L after rotate")
        close(st["Q"], Qr, kind, "Q after rotate")
        # the forces at the moved state (the cell list follows the move)
        F2 = s.calculateforces()
        assert force_errors(F2, sysm.central_forces(st["x"]))["rms"] <= rms
        assert s.flags == 0


@pytest.mark.parametrize("kind", ["fp64", "fp64-pp"])
def test_per_phase_loop_equals_the_fused_step(kind):
    spec, x, Q, _, _ = system(n=1200, phi=0.25, seed=7)
    n, steps = spec.n, 20
    z = np.zeros((n, 3))
    with handle(spec, kind) as s:
        s.initialize(x, z, z, Q)
        s.init_forces()
        s.step(steps)
        fused = s.get_state()
    with handle(spec, kind) as s:
        s.initialize(x, z, z, Q)
        s.init_forces()
        st = s.get_state()
        F, T = st["Ft"].copy(), st["Tt"].copy()
        for _ in range(steps):   # Condensate.cpp:335-378, the same Philox draws as mtg_step
            s.advancemom_halfstep(F, T)
            s.advance_pos()
            s.rotate()
            F = s.calculateforces()
            T = np.zeros((n, 3))
            s.add_patch_forces_and_torques(F, T)
            s.create_forces_and_torques_sphere(F, T)
            s.advancemom_halfstep(F, T)
        phased = s.get_state()
    for key in ("x", "p", "Lb", "Q"):
        d = phased[key] - fused[key]
        if key == "x":
            d -= spec.box * np.round(d / spec.box)
        assert np.abs(d).max() <= 1e-10 * max(1.0, np.abs(fused[key]).max()), key


def test_adapter_loop_with_reference_signatures_matches_oracle(tmp_path):
    exe = compile_driver("phases_gpu.cpp", BUILD / "phases_gpu")
    n, steps = 400, 30
    spec = ReplicaSpec(n=n, box=box_for(n, 0.3), model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9)),
                       kT=1.0)
    x = random_positions(n, spec.box, True, 0.95, 41)
    Q = random_rotations(n, 42)
    noise = po.philox_noise(n * (steps + 1), 77, 0, 0).reshape(steps + 1, n, 6)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([n, _lib.MTG_FP64, steps], dtype=np.int32).tofile(f)
        np.array([spec.box, spec.kT, spec.dt], dtype=np.float64).tofile(f)
        x.tofile(f)
        Q.tofile(f)
        noise.tofile(f)
    out = tmp_path / "out.bin"
    proc = subprocess.run([str(exe), str(inp), str(out)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stdout
    raw = out.read_bytes()
    npairs = int(np.frombuffer(raw[:8], dtype=np.int64)[0])
    vals = np.frombuffer(raw[8:], dtype=np.float64)
    F0, T0, xf, pf, Qf, Lf = (vals[a:b].reshape(n, -1) for a, b in
                              ((0, 3 * n), (3 * n, 6 * n), (6 * n, 9 * n), (9 * n, 12 * n), (12 * n, 21 * n),
                               (21 * n, 24 * n)))
    sysm = po.System(spec)
    assert npairs == len(sysm.pairs(x, 3.5))
    z = np.zeros((n, 3))
    st = dict(x=x.copy(), p=z.copy(), Lb=z.copy(), Q=Q.copy())
    st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"], noise=np.ascontiguousarray(noise[0]))
    assert force_errors(F0, st["Ft"])["rms"] <= 1e-12 and force_errors(T0, st["Tt"])["rms"] <= 1e-12
    assert sysm.run(st, steps, noise_mode=1, noise=np.ascontiguousarray(noise[1:]), check_skin=False) == 0
    for got, key in ((xf, "x"), (pf, "p"), (Qf, "Q"), (Lf, "Lb")):
        assert np.abs(got - st[key]).max() <= 1e-9 * max(1.0, np.abs(st[key]).max()), key
