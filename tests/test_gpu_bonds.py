"""GPU parity of the bonded term (harmonic bonds, HarmonicPotential over a fixed bond list) through the C ABI.

Tolerances are those of test_gpu_parity.py: forces and torques as relative RMS error over all particles,
FP64 build <= 1e-12 (worst particle <= 1e-11 of the RMS force), FP32 build <= 1e-5 (worst particle
<= 1e-4); FP64 trajectories 1e-9 relative to the state's scale after 50 steps.
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU, MtgError
from mtcode_gb300.system import ReplicaSpec, random_rotations
from mtcode_gb300.workloads import bead_model, box_for, chain_replica
from oracle import pyoracle as po
from tests._util import force_errors, load, spec_from

pytestmark = pytest.mark.gpu
PRECISIONS = ["fp32", "fp64"]


def check(a, b, precision):
    e = force_errors(a, b)
    rms_tol, max_tol = (1e-12, 1e-11) if precision == "fp64" else (1e-5, 1e-4)
    assert e["rms"] <= rms_tol, e
    assert e["max"] <= max_tol, e


def bonded_system(n_ch, beads, phi, every, seed, periodic=True, jitter=0.06):
    n = n_ch * beads
    box = box_for(n, phi)
    x, bonds, n_patchy = chain_replica(n_ch, beads, box, every, seed, periodic)
    x = x + np.random.default_rng(seed).uniform(-jitter, jitter, x.shape)
    x = np.mod(x, box) if periodic else np.clip(x, 0.0, np.nextafter(box, 0))
    x = x.astype(np.float32).astype(np.float64)
    Q = random_rotations(n, seed + 1).astype(np.float32).astype(np.float64)
    spec = ReplicaSpec(n=n, box=box, model=bead_model(n_patchy, n), periodic=periodic, dt=0.002, seed=seed)
    return spec, x, Q, bonds


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", range(2))
def test_bonded_forces_vs_reference_fixture(k, precision):
    d = load(f"bonded_{k}.npz")
    spec = spec_from(d)
    z = np.zeros((spec.n, 3))
    with LangevinNVTRGPU([spec], precision=precision) as s:
        s.initialize(d["x"], z, z, d["Q"])
        s.set_bonds(d["bonds"], float(d["bond_k"]), float(d["bond_r0"]))
        F, T = s.calculate_forces_and_torques3D()
        check(F, d["F"], precision)
        check(T, d["T"], precision)
        # removing the bonds leaves the pair forces alone
        s.set_bonds([], 0.0, 0.0)
        F0, _ = s.calculate_forces_and_torques3D()
    check(F0, d["F"] - d["F_bond"], precision)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_bonds_set_before_state_and_after_steps(precision):
    """The id -> slot map follows the particles: bonds given before the state, and forces after steps
    that re-sorted the particles, still agree with the oracle."""
    spec, x, Q, bonds = bonded_system(40, 50, 0.25, 5, 21)
    sysm = po.System(spec)
    sysm.set_bonds(bonds, 100.0, 1.0)
    z = np.zeros((spec.n, 3))
    with LangevinNVTRGPU([spec], precision=precision) as s:
        s.set_bonds(bonds, 100.0, 1.0)
        s.initialize(x, z, z, Q)
        F, T = s.calculate_forces_and_torques3D()
        Fo, To = sysm.forces(x, Q)
        check(F, Fo, precision)
        check(T, To, precision)
        s.init_forces()
        s.step(7)
        st = s.get_state()
        F, T = s.calculate_forces_and_torques3D()
    Fo, To = sysm.forces(st["x"], st["Q"])
    check(F, Fo, precision)
    check(T, To, precision)


def test_bonded_trajectory_fp64_vs_oracle():
    """50 noise-free steps (kT = 0) of a bonded chain system, FP64 build against the oracle's loop."""
    spec, x, Q, bonds = bonded_system(30, 40, 0.25, 4, 31)
    spec.kT = 0.0
    n = spec.n
    z = np.zeros((n, 3))
    with LangevinNVTRGPU([spec], precision="fp64") as s:
        s.initialize(x, z, z, Q)
        s.set_bonds(bonds, 100.0, 1.0)
        s.init_forces()
        s.step(50)
        got = s.get_state()
    sysm = po.System(spec)
    sysm.set_bonds(bonds, 100.0, 1.0)
    st = dict(x=x.copy(), p=z.copy(), Lb=z.copy(), Q=Q.copy())
    st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"])
    assert sysm.run(st, 50, noise_mode=0) == 0
    for key in ("x", "p", "Lb", "Q"):
        scale = max(1.0, np.abs(st[key]).max())
        assert np.abs(got[key] - st[key]).max() <= 1e-9 * scale, key


def test_batched_bonded_replicas_fp32():
    """Three bonded replicas of different sizes in one FP32 handle (tile kernel): bond indices are
    global, each replica's forces match its own oracle."""
    systems = [bonded_system(30, 40, 0.25, 4, 41), bonded_system(50, 30, 0.3, 3, 42),
               bonded_system(20, 60, 0.2, 10, 43)]
    specs = [sp for sp, _, _, _ in systems]
    offs = np.cumsum([0] + [sp.n for sp in specs])
    x = np.concatenate([xx for _, xx, _, _ in systems])
    Q = np.concatenate([qq for _, _, qq, _ in systems])
    bonds = np.concatenate([b + offs[r] for r, (_, _, _, b) in enumerate(systems)])
    z = np.zeros((len(x), 3))
    with LangevinNVTRGPU(specs, precision="fp32") as s:
        s.initialize(x, z, z, Q)
        s.set_bonds(bonds, 100.0, 1.0)
        F, T = s.calculate_forces_and_torques3D()
    for r, (sp, xx, qq, b) in enumerate(systems):
        sysm = po.System(sp)
        sysm.set_bonds(b, 100.0, 1.0)
        Fo, To = sysm.forces(xx, qq)
        check(F[offs[r]:offs[r + 1]], Fo, "fp32")
        check(T[offs[r]:offs[r + 1]], To, "fp32")


def test_bond_list_is_checked():
    spec_a, xa, Qa, ba = bonded_system(5, 20, 0.2, 5, 51)
    spec_b, xb, Qb, bb = bonded_system(5, 20, 0.2, 5, 52)
    x = np.concatenate([xa, xb])
    Q = np.concatenate([Qa, Qb])
    z = np.zeros((len(x), 3))
    with LangevinNVTRGPU([spec_a, spec_b], precision="fp32") as s:
        s.initialize(x, z, z, Q)
        for bad in ([[0, 150]], [[3, 3]], [[0, 200]], [[-1, 2]]):  # two replicas, self bond, out of range
            with pytest.raises(MtgError) as err:
                s.set_bonds(bad, 100.0, 1.0)
            assert err.value.status == 1
        with pytest.raises(MtgError):
            s.set_bonds([[0, 1]], math.nan, 1.0)
        # the handle stays usable after rejected lists
        s.set_bonds(np.concatenate([ba, bb + spec_a.n]), 100.0, 1.0)
        F, _ = s.calculate_forces_and_torques3D()
    assert np.isfinite(F).all()
