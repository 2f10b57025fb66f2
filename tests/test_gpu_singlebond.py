"""GPU parity of the single-bond-per-patch mode (Condensate::run_singlebond's force pass) through the C ABI.

Every case starts from a bond state of the reference fixtures (tests/golden/singlebond_*.npz: unbound,
re-decided, and after new orientations) and compares one mtg_bind_update with the oracle's orc_bind_update
on the same coordinates, in its Philox mode (the GPU's random numbers).  The bond state must agree exactly:
every bond decision is the reference's FP64 test on the stored coordinates (FP32 handles evaluate in float
and re-decide in FP64 within a margin of each threshold).  Forces (WCA core + bound pairs) and torques use
the tolerances of test_gpu_parity.py: relative RMS error <= 1e-12 in FP64 (worst particle <= 1e-11 of the
RMS), <= 1e-5 in FP32 (worst <= 1e-4).  FP64 trajectories: 1e-9 of the state's scale after 25 steps.
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU, MtgError
from mtcode_gb300 import system as S
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
from oracle import pyoracle as po
from tests._util import force_errors, load, spec_from
from tests.test_oracle_bind import binding_of, candidates

pytestmark = pytest.mark.gpu
CONFIGS = [("fp32", "pairs"), ("fp32", "per_particle"), ("fp64", "pairs")]


def check(a, b, precision):
    e = force_errors(a, b)
    rms_tol, max_tol = (1e-12, 1e-11) if precision == "fp64" else (1e-5, 1e-4)
    assert e["rms"] <= rms_tol, e
    assert e["max"] <= max_tol, e


def gpu_model(d):
    kind, args, tables = int(d["bm_kind"]), d["args"], d["tables"]
    if kind == 0:
        return S.binding_single(float(args[0]), float(args[1]))
    if kind == 1:
        return S.binding_binary_equilibrium(int(args[0]))
    extra = [int(a) for a in args[:2 if kind == 2 else 3]]
    return S.binding_tables(kind, tables[:24], tables[24:], *extra)


def oracle_update(sysm, B, x, Q, bt, ib, draw, replica=0):
    bt = np.ascontiguousarray(bt, dtype=np.intc).copy()
    ib = np.ascontiguousarray(ib, dtype=np.uint8).copy()
    st, Fb, Tb = sysm.bind_update(x, Q, candidates(sysm, x, Q, sysm.default_max_ang()), B, bt, ib, rng=0,
                                  seed=sysm.spec.seed, replica=replica, draw=draw)
    assert st == 0
    return bt, ib, sysm.central_forces(x) + Fb, Tb


@pytest.mark.parametrize("precision,kernel", CONFIGS)
@pytest.mark.parametrize("k", range(8))
def test_bind_update_matches_oracle(k, precision, kernel):
    d = load(f"singlebond_{k}.npz")
    spec = spec_from(d)
    sysm = po.System(spec)
    B = binding_of(d)
    z = np.zeros((spec.n, 3))
    with LangevinNVTRGPU([spec], precision=precision, force_kernel=kernel) as s:
        s.set_single_bond(gpu_model(d))
        assert s.num_patches == sysm.total_patches() and s.patch_offset(0) == 0
        for rnd in range(3):
            Q = d["Q"][rnd]
            s.initialize(d["x"], z, z, Q)
            s.set_bind_state(d["bt_in"][rnd], d["ib_in"][rnd])
            draw = s.draw
            F, T = s.bind_update()
            bt, ib = s.get_bind_state()
            bo, io, Fo, To = oracle_update(sysm, B, d["x"], Q, d["bt_in"][rnd], d["ib_in"][rnd], draw)
            assert np.array_equal(ib, io), f"round {rnd}: {int((ib != io).sum())} isbound differ"
            assert np.array_equal(bt, bo), f"round {rnd}: boundto differs"
            assert io.sum() > 0
            check(F, Fo, precision)
            check(T, To, precision)
            assert s.flags == 0


@pytest.mark.parametrize("precision,kernel", CONFIGS)
def test_bind_update_two_replicas(precision, kernel):
    """Two replicas in one handle: patch offsets, replica-keyed random numbers, replica-local boundto."""
    d1, d5 = load("singlebond_1.npz"), load("singlebond_5.npz")
    specs = [spec_from(d1), spec_from(d5)]
    model = S.binding_single(0.7, 0.5)
    B = po.binding_single(0.7, 0.5)
    x = np.concatenate([d1["x"], d5["x"]])
    Q = np.concatenate([d1["Q"][1], d5["Q"][1]])
    bt_in = np.concatenate([d1["bt_in"][1], d5["bt_in"][1]])
    ib_in = np.concatenate([d1["ib_in"][1], d5["ib_in"][1]])
    z = np.zeros((len(x), 3))
    with LangevinNVTRGPU(specs, precision=precision, force_kernel=kernel) as s:
        s.set_single_bond(model)
        assert s.patch_offset(1) == 4 * specs[0].n and s.num_patches == 4 * (specs[0].n + specs[1].n)
        s.initialize(x, z, z, Q)
        s.set_bind_state(bt_in, ib_in)
        draw = s.draw
        F, T = s.bind_update()
        bt, ib = s.get_bind_state()
    po_ = 0
    xo = 0
    for r, (spec, d) in enumerate([(specs[0], d1), (specs[1], d5)]):
        sysm = po.System(spec)
        np_ = 4 * spec.n
        bo, io, Fo, To = oracle_update(sysm, B, d["x"], d["Q"][1], d["bt_in"][1], d["ib_in"][1], draw, replica=r)
        assert np.array_equal(ib[po_:po_ + np_], io) and np.array_equal(bt[po_:po_ + np_], bo)
        check(F[xo:xo + spec.n], Fo, precision)
        check(T[xo:xo + spec.n], To, precision)
        po_ += np_
        xo += spec.n


def test_trajectory_matches_oracle_fp64():
    """init + 25 steps of the run_singlebond loop with Philox noise: candidate lists rebuilt at steps 10, 20."""
    d = load("singlebond_1.npz")
    spec = spec_from(d)
    sysm = po.System(spec)
    n = spec.n
    z = np.zeros((n, 3))
    x0, Q0 = d["x"], d["Q"][0]
    nsteps = 25
    with LangevinNVTRGPU([spec], precision="fp64") as s:
        s.set_single_bond(S.binding_single(0.7, 0.5))
        s.initialize(x0, z, z, Q0)
        s.step(nsteps)
        got = s.get_state()
        bt, ib = s.get_bind_state()
        assert s.flags == 0
    st = dict(x=x0.copy(), p=z.copy(), Lb=z.copy(), Q=Q0.copy(), Ft=z.copy(), Tt=z.copy(),
              boundto=np.zeros(4 * n, dtype=np.intc), isbound=np.zeros(4 * n, dtype=np.uint8))
    status = sysm.run_singlebond(st, po.binding_single(0.7, 0.5), nsteps, sysm.default_max_ang(), init=True,
                                 init_draw=0, noise_mode=2, seed=spec.seed, replica=0, draw0=1)
    assert status == 0
    assert np.array_equal(ib, st["isbound"]) and np.array_equal(bt[ib == 1], st["boundto"][st["isbound"] == 1])
    assert st["isbound"].sum() > 0
    for key in ("x", "p", "Lb", "Q", "Ft", "Tt"):
        scale = max(1.0, float(np.abs(st[key]).max()))
        assert np.abs(got[key] - st[key]).max() <= 1e-9 * scale, key


@pytest.mark.parametrize("precision,kernel", CONFIGS)
def test_steps_keep_bonds_consistent(precision, kernel):
    """100 steps at the C1-like density: every bond is mutual, and bound pairs are within range."""
    n, phi = 2000, 0.15
    box = (n * math.pi / 6 / phi) ** (1 / 3)
    spec = ReplicaSpec(n=n, box=box, model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9)), seed=5)
    x = random_positions(n, box, True, 0.9, 5)
    Q = random_rotations(n, 6)
    z = np.zeros((n, 3))
    with LangevinNVTRGPU([spec], precision=precision, force_kernel=kernel) as s:
        s.set_single_bond(S.binding_single(1.0, 0.05))
        s.initialize(x, z, z, Q)
        s.step(100)
        s.sync()
        bt, ib = s.get_bind_state()
        xs = s.get_state()["x"]
        assert s.flags == 0
    b = np.flatnonzero(ib)
    assert len(b) > 0
    assert np.all(ib[bt[b]] == 1) and np.all(bt[bt[b]] == b)
    d = xs[b // 4] - xs[bt[b] // 4]
    d -= box * np.round(d / box)
    assert np.linalg.norm(d, axis=1).max() < 1.68


def test_switching_off_restores_full_patch_force():
    d = load("singlebond_0.npz")
    spec = spec_from(d)
    z = np.zeros((spec.n, 3))
    with LangevinNVTRGPU([spec]) as ref, LangevinNVTRGPU([spec]) as s:
        ref.initialize(d["x"], z, z, d["Q"][0])
        F0, T0 = ref.calculate_forces_and_torques3D()
        s.set_single_bond(S.binding_single(1.0, 0.1))
        s.initialize(d["x"], z, z, d["Q"][0])
        s.bind_update()
        s.set_single_bond(None)
        F1, T1 = s.calculate_forces_and_torques3D()
    assert np.array_equal(F0, F1) and np.array_equal(T0, T1)


def test_capacity_is_reported():
    """A percolating patch network (wide cones, dense) exceeds the 128-patch cluster capacity: reported
    as MTG_ERR_CAPACITY, never as wrong bonds."""
    n, phi = 600, 0.35
    box = (n * math.pi / 6 / phi) ** (1 / 3)
    spec = ReplicaSpec(n=n, box=box, model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.3)), seed=9)
    z = np.zeros((n, 3))
    with LangevinNVTRGPU([spec], precision="fp64") as s:
        s.set_single_bond(S.binding_single(1.0, 0.1))
        s.initialize(random_positions(n, box, True, 0.9, 9), z, z, random_rotations(n, 10))
        with pytest.raises(MtgError) as e:
            s.bind_update()
        assert e.value.status == 6
        s.clear_flags()


def test_mode_arguments_are_checked():
    d = load("singlebond_0.npz")
    spec = spec_from(d)
    with LangevinNVTRGPU([spec], force_kernel="tiled") as s, pytest.raises(MtgError):
        s.set_single_bond(S.binding_single(1.0, 0.1))
    with LangevinNVTRGPU([spec], neighbor_skin=0.3) as s, pytest.raises(MtgError):
        s.set_single_bond(S.binding_single(1.0, 0.1))
    with LangevinNVTRGPU([spec]) as s:
        with pytest.raises(MtgError):
            s.set_single_bond(S.binding_single(1.0, 0.1), patch_every=0)
        s.set_single_bond(S.binding_single(1.0, 0.1))
        bad = np.zeros(s.num_patches, dtype=np.int32)
        bad[3] = s.num_patches
        with pytest.raises(MtgError):
            s.set_bind_state(bad, np.zeros(s.num_patches, dtype=np.uint8))
