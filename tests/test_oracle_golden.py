"""Pins the oracle (oracle/oracle.c, the FP64 CPU restatement) to the reference.

Golden fixtures were produced by the reference's own routines (tests/golden/make_golden.py over
oracle/_ref).  On x86-64 the oracle reproduces them bit for bit; on other hosts (aarch64: long double
is binary128, so the angular factors round differently) to 1e-12 relative.  Where the reference
shim is present (only in the build container) the oracle is also compared live on fresh inputs.
"""
import math
import platform

import numpy as np
import pytest

from oracle import pyoracle as po
from tests._util import load, sorted_pairs, spec_from

EXACT = platform.machine() in ("x86_64", "AMD64")


def close(a, b, rtol=1e-12):
    if EXACT:
        return np.array_equal(a, b)
    return np.allclose(a, b, rtol=rtol, atol=rtol * max(1.0, np.abs(b).max()))


@pytest.mark.parametrize("k", range(7))
def test_pairs_match_reference(k):
    d = load(f"pairs_{k}.npz")
    sysm = po.System(spec_from(d))
    got = sorted_pairs(sysm.pairs(d["x"], float(d["rc"]), int(d["ncell"])))
    assert np.array_equal(got, d["pairs"])


@pytest.mark.parametrize("k", range(5))
def test_forces_match_reference(k):
    d = load(f"forces_{k}.npz")
    sysm = po.System(spec_from(d))
    F, T = sysm.forces(d["x"], d["Q"], float(d["rc"]))
    assert close(F, d["F"])
    assert close(T, d["T"])


@pytest.mark.parametrize("k", range(4))
def test_trajectories_match_reference(k):
    d = load(f"traj_{k}.npz")
    spec = spec_from(d)
    sysm = po.System(spec)
    n, nsteps = spec.n, int(d["nsteps"])
    st = dict(x=d["x0"].copy(), p=np.zeros((n, 3)), Lb=np.zeros((n, 3)), Q=d["Q0"].copy())
    rc = float(d["rc"])
    if str(d["noise_mode"]) == "shared":
        noise = po.philox_noise(n * (nsteps + 1), int(d["noise_seed"]), 0, 0).reshape(nsteps + 1, n, 6)
        st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"], np.ascontiguousarray(noise[0]), rc)
        status = sysm.run(st, nsteps, noise_mode=1, noise=np.ascontiguousarray(noise[1:]), rc=rc)
    else:
        st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"], None, rc)
        status = sysm.run(st, nsteps, noise_mode=0, rc=rc)
    assert status == 0
    for key in ("x", "p", "Lb", "Q", "Ft", "Tt"):
        assert close(st[key], d["final_" + key], rtol=1e-10), key


@pytest.mark.parametrize("k", range(6))
def test_two_particle_torque_cases(k):
    d = load(f"torque_{k}.npz")
    spec = spec_from(d)
    sysm = po.System(spec)
    st = dict(x=d["x0"].copy(), p=np.zeros((2, 3)), Lb=np.zeros((2, 3)), Q=d["Q0"].copy())
    st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"], None, float(d["rc"]))
    assert sysm.run(st, int(d["nsteps"]), noise_mode=0, rc=float(d["rc"])) == 0
    for key in ("x", "p", "Lb", "Q"):
        assert close(st[key], d["final_" + key], rtol=1e-10), key


def test_rotation_matrix_matches_genfullmat():
    import ctypes as C
    d = load("rotation.npz")
    for L, R in zip(d["L"], d["R"]):
        out = np.empty(9)
        L = np.ascontiguousarray(L)
        po.orc().orc_rotation_matrix(C.c_double(float(d["dt"])), C.c_double(float(d["inertia"])), po._d(L), po._d(out))
        assert close(out, R)


def test_philox_known_answers():
    # Random123 philox4x32-10 known-answer vectors (kat_vectors)
    assert po.philox([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert po.philox([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert po.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == \
        [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_philox_noise_moments():
    xi = po.philox_noise(200000, 123, 3, 9)
    assert abs(xi.mean()) < 5e-3
    assert abs(xi.var() - 1.0) < 1e-2
    assert xi.min() >= -1.732050808 and xi.max() < 1.732050808


def test_stencil_dedup_small_grids():
    import ctypes as C
    out = (C.c_int * 27)()
    assert po.orc().orc_neighbor_cells(0, 1, out) == 1
    assert po.orc().orc_neighbor_cells(0, 2, out) == 8
    assert po.orc().orc_neighbor_cells(13, 3, out) == 27


@pytest.mark.skipif(po.ref() is None, reason="reference shim (oracle/_ref) is only built where the reference sources exist")
def test_oracle_vs_reference_live():
    """Fresh random inputs (not in the fixtures) through both the reference and the oracle."""
    from tests.golden.make_golden import make_system, ref_forces, ref_pairs
    for kind, seed in (("tetra", 901), ("tubulin", 902), ("crowded", 903)):
        spec, x, Q = make_system(kind, 500, 0.3, seed, True, min_dist=0.95)
        sysm = po.System(spec)
        rc = sysm.force_range * 1.05
        F, T = sysm.forces(x, Q, rc)
        Fr, Tr = ref_forces(spec, x, Q, rc)
        assert close(F, Fr) and close(T, Tr)
        nc = max(1, int(math.floor(spec.box / 1.7)))
        assert np.array_equal(sorted_pairs(sysm.pairs(x, 1.7, nc)), ref_pairs(spec, x, nc, 1.7))


@pytest.mark.parametrize("k", range(2))
def test_bonded_forces_match_reference(k):
    """Harmonic bonds (MD::calculateforces with HarmonicPotential) alone, and the bonded driver's sum
    bond + HS + patch forces, against the reference's own routines."""
    d = load(f"bonded_{k}.npz")
    sysm = po.System(spec_from(d))
    bk, br = float(d["bond_k"]), float(d["bond_r0"])
    assert close(sysm.bond_forces(d["x"], d["bonds"], bk, br), d["F_bond"])
    sysm.set_bonds(d["bonds"], bk, br)
    F, T = sysm.forces(d["x"], d["Q"], float(d["rc"]))
    assert close(F, d["F"])
    assert close(T, d["T"])


@pytest.mark.skipif(po.ref() is None, reason="the reference shim is only built where the reference sources exist")
def test_bond_forces_live_vs_reference():
    """Fresh chains (not in the fixtures): the oracle's bond forces equal the reference's bit for bit."""
    from mtcode_gb300.workloads import bead_model, box_for, chain_replica
    n_ch, beads = 30, 40
    box = box_for(n_ch * beads, 0.2)
    x, bonds, n_patchy = chain_replica(n_ch, beads, box, 4, 9)
    x = x + np.random.default_rng(3).uniform(-0.05, 0.05, x.shape)
    from mtcode_gb300.system import ReplicaSpec
    spec = ReplicaSpec(n=n_ch * beads, box=box, model=bead_model(n_patchy, n_ch * beads))
    F = po.System(spec).bond_forces(x, bonds, 37.0, 1.1)
    Fr = np.empty_like(F)
    b = np.ascontiguousarray(bonds, dtype=np.intc)
    po.ref().ref_bond_forces(spec.n, spec.box, 1, po._d(np.ascontiguousarray(x)), b.ctypes.data_as(po._I), len(b),
                             37.0, 1.1, po._d(Fr))
    assert np.array_equal(F, Fr)


@pytest.mark.parametrize("k", range(3))
def test_analysis_matches_reference(k):
    """calcg1 histogram and distance_graph labels: integer results, equal to the reference's."""
    d = load(f"analysis_{k}.npz")
    sysm = po.System(spec_from(d))
    assert np.array_equal(sysm.gr(d["x"], float(d["rmax"]), float(d["dr"])), d["hist"])
    assert np.array_equal(sysm.clusters(d["x"], float(d["cut"])), d["labels"])
