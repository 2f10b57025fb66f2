"""Verlet-skin neighbour lists (mtg_config.neighbor_skin > 0) through the C ABI.

The skin only changes how the pair set is found, not the pair set: every pair within the force range
is in the lists while no particle has moved more than half the skin since they were built, and the
step rebuilds them before that can happen.  With fixed-point force sums and the same first-half-step
arithmetic, FP32 trajectories with a skin are therefore BIT-IDENTICAL to those that rebuild the cells
every step; FP64 ones (plain sums in candidate order) agree to 1e-12 relative.
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
from mtcode_gb300.workloads import bead_model, box_for, chain_replica, crowded_model, patchy_c4
from oracle import pyoracle as po
from tests._util import force_errors

pytestmark = pytest.mark.gpu


def tetra(n, phi, **kw):
    return ReplicaSpec(n=n, box=box_for(n, phi), model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9)), **kw)


def run(specs, x, Q, steps, precision="fp32", skin=0.0, chunks=1, bonds=None, observe=False, kernel="tiled"):
    n = len(x)
    z = np.zeros((n, 3))
    out = []
    with LangevinNVTRGPU(specs, precision=precision, neighbor_skin=skin, force_kernel=kernel) as s:
        s.initialize(x, z, z, Q)
        if bonds is not None:
            s.set_bonds(bonds, 100.0, 1.0)
        s.init_forces()
        for c in range(chunks):
            s.step(steps)
            if observe and c == 0:
                s.observables()  # re-sorts the state by another grid: the next step must rebuild
            out.append(s.get_state())
        rebuilds = s.rebuilds
    return out, rebuilds


@pytest.mark.parametrize("kernel", ["tiled", "pairs"])
@pytest.mark.parametrize("skin", [0.3, 0.6])
def test_fp32_trajectory_is_bit_identical_with_a_skin(skin, kernel):
    W = patchy_c4(seed=3, n_replicas=6)
    exact, _ = run(W.replicas, W.x, W.Q, 40, chunks=3, kernel=kernel)
    listed, rebuilds = run(W.replicas, W.x, W.Q, 40, skin=skin, chunks=3, kernel=kernel)
    for a, b in zip(exact, listed):
        for key in ("x", "p", "Lb", "Q", "Ft", "Tt"):
            assert np.array_equal(a[key], b[key]), key
    assert 1 < rebuilds < 121, rebuilds  # lists were reused, and rebuilt


@pytest.mark.parametrize("kernel", ["tiled", "pairs"])
def test_fp32_bonded_crowded_and_walled_systems_with_a_skin(kernel):
    sp1, x1, Q1, b1 = None, None, None, None
    n = 40 * 30
    box = box_for(n, 0.25)
    xc, bonds, n_patchy = chain_replica(40, 30, box, 3, 17)
    sp1 = ReplicaSpec(n=n, box=box, model=bead_model(n_patchy, n), dt=0.002, seed=1)
    sp2 = ReplicaSpec(n=2000, box=box_for(2000, 0.3), model=crowded_model(500, 2000), seed=2)
    sp3 = tetra(1500, 0.2, periodic=False, seed=3)
    x = np.concatenate([xc, random_positions(2000, sp2.box, True, 0.95, 18),
                        random_positions(1500, sp3.box, False, 0.95, 19)])
    Q = random_rotations(len(x), 20)
    specs = [sp1, sp2, sp3]
    exact, _ = run(specs, x, Q, 60, chunks=2, bonds=bonds, observe=True, kernel=kernel)
    listed, rebuilds = run(specs, x, Q, 60, skin=0.4, chunks=2, bonds=bonds, observe=True, kernel=kernel)
    for a, b in zip(exact, listed):
        for key in ("x", "p", "Lb", "Q", "Ft", "Tt"):
            assert np.array_equal(a[key], b[key]), key
    assert rebuilds > 1


@pytest.mark.parametrize("kernel", ["pairs", "per_particle"])
def test_fp64_trajectory_with_a_skin(kernel):
    """FP64 sums a particle's pair terms in the order the pairs are found (double atomics in the pair pipeline),
    which the lists change: the two runs agree to rounding, amplified over 50 steps."""
    spec = tetra(1500, 0.25, seed=5)
    x = random_positions(spec.n, spec.box, True, 0.95, 6)
    Q = random_rotations(spec.n, 7)
    exact, _ = run([spec], x, Q, 50, precision="fp64", kernel=kernel)
    listed, rebuilds = run([spec], x, Q, 50, precision="fp64", skin=0.4, kernel=kernel)
    for key in ("x", "p", "Lb", "Q"):
        scale = max(1.0, np.abs(exact[0][key]).max())
        assert np.abs(listed[0][key] - exact[0][key]).max() <= 1e-10 * scale, key
    assert rebuilds >= 1


@pytest.mark.parametrize("kernel", ["tiled", "pairs"])
def test_forces_with_a_skin_match_the_oracle_between_rebuilds(kernel):
    spec = tetra(3000, 0.3, seed=8)
    x = random_positions(spec.n, spec.box, True, 0.95, 9)
    Q = random_rotations(spec.n, 10)
    z = np.zeros((spec.n, 3))
    sysm = po.System(spec)
    with LangevinNVTRGPU([spec], precision="fp32", neighbor_skin=0.5, force_kernel=kernel) as s:
        s.initialize(x, z, z, Q)
        s.init_forces()
        for _ in range(4):
            s.step(7)
            st = s.get_state()
            F, T = s.calculate_forces_and_torques3D()  # from the stored lists when they are still valid
            Fo, To = sysm.forces(st["x"], st["Q"])
            e = force_errors(F, Fo)
            assert e["rms"] <= 1e-5 and e["max"] <= 1e-4, e
            e = force_errors(T, To)
            assert e["rms"] <= 1e-5 and e["max"] <= 1e-4, e
