"""GPU checks of the step's observables and error reporting, through the C ABI, against the oracle.

Tolerances (stated once):
  temperature (LangevinNVTR::measured_temperature)   FP64 1e-12 relative; FP32 1e-9 relative to the
      oracle evaluated on the float32-rounded momenta (the device reduces in FP64)
  observables (energies, virial)                     FP64 1e-10 relative; FP32 2e-5 relative to the
      largest of |value| and 1 (FP32 pair terms, FP64 sums)
  observables (bonded patch pairs, pairs in range)   exact (fixtures keep every pair 1e-6 away from a
      threshold)
  unwrapped displacement                             x0 + disp - x is a whole number of box lengths per
      coordinate to 1e-9 (FP64) / 2e-3 absolute (FP32: the stored position is rounded every step)
  walled-box trajectory, FP64, noise off, 100 steps  1e-9 relative to the state's scale
  equipartition with live Philox noise               <p_k^2/2m> and <L_k^2/2I> within 4% of kT/2
  patch energy with live noise, GPU FP32 vs oracle   time averages within 4 standard errors (block
      averages of both runs) plus 2% -- independent trajectories of the same ensemble
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU, MtgError
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
from mtcode_gb300.workloads import box_for, crowded_model, tubulin_model
from oracle import pyoracle as po
from tests._util import load, spec_from

pytestmark = pytest.mark.gpu
PRECISIONS = ["fp32", "fp64"]


def f32(a):
    return np.asarray(a, np.float32).astype(np.float64)


def tetra_spec(n, phi, **kw):
    return ReplicaSpec(n=n, box=box_for(n, phi), model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9)), **kw)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_temperature_matches_oracle(precision):
    specs = [tetra_spec(500, 0.2), ReplicaSpec(n=300, box=box_for(300, 0.2), model=tubulin_model(300), mass=2.0,
                                               inertia=0.3)]
    rng = np.random.default_rng(3)
    xs = [random_positions(sp.n, sp.box, True, 0.95, 10 + r) for r, sp in enumerate(specs)]
    Qs = [random_rotations(sp.n, 20 + r) for r, sp in enumerate(specs)]
    ps = [rng.normal(size=(sp.n, 3)) * (1 + r) for r, sp in enumerate(specs)]
    Ls = [rng.normal(size=(sp.n, 3)) * 0.3 for sp in specs]
    with LangevinNVTRGPU(specs, precision=precision) as s:
        s.initialize(np.concatenate(xs), np.concatenate(ps), np.concatenate(Ls), np.concatenate(Qs))
        got = s.measured_temperature()
    for r, sp in enumerate(specs):
        p, L = (ps[r], Ls[r]) if precision == "fp64" else (f32(ps[r]), f32(Ls[r]))
        want = po.System(sp).temperature(np.ascontiguousarray(p), np.ascontiguousarray(L))
        tol = 1e-12 if precision == "fp64" else 1e-9
        assert np.allclose(got[r], want, rtol=tol, atol=0), (got[r], want)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", range(5))
def test_observables_match_oracle(k, precision):
    d = load(f"forces_{k}.npz")
    spec = spec_from(d)
    sysm = po.System(spec)
    z = np.zeros((spec.n, 3))
    with LangevinNVTRGPU([spec], precision=precision) as s:
        s.initialize(d["x"], z, z, d["Q"])
        got = s.observables()[0]
    want = sysm.observables(d["x"], d["Q"])
    npairs = len(sysm.pairs(d["x"], sysm.force_range))
    tol = 1e-10 if precision == "fp64" else 2e-5
    for i in range(3):
        assert abs(got[i] - want[i]) <= tol * max(1.0, abs(want[i])), (i, got, want)
    assert got[3] == want[3], (got, want)
    assert got[4] == npairs, (got, npairs)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_nonfinite_state_is_reported_and_the_handle_recovers(precision):
    spec = tetra_spec(400, 0.2)
    x = random_positions(spec.n, spec.box, True, 0.95, 5)
    Q = random_rotations(spec.n, 6)
    z = np.zeros((spec.n, 3))
    bad = x.copy()
    bad[17, 1] = np.nan
    with LangevinNVTRGPU([spec], precision=precision) as s:
        s.initialize(bad, z, z, Q)
        s.init_forces()
        s.step(3)
        with pytest.raises(MtgError) as err:
            s.sync()
        assert err.value.status == 5  # MTG_ERR_NONFINITE
        assert s.flags & 0x1
        # a clean state on the same handle steps normally again
        s.initialize(x, z, z, Q)
        s.clear_flags()
        s.init_forces()
        s.step(3)
        s.sync()
        st = s.get_state()
    assert np.isfinite(st["x"]).all() and np.isfinite(st["p"]).all()


@pytest.mark.parametrize("precision", PRECISIONS)
def test_unwrapped_displacement_tracks_the_motion(precision):
    spec = tetra_spec(2000, 0.15, kT=1.0, seed=9)
    x0 = random_positions(spec.n, spec.box, True, 0.95, 7)
    Q = random_rotations(spec.n, 8)
    z = np.zeros((spec.n, 3))
    with LangevinNVTRGPU([spec], precision=precision) as s:
        s.initialize(x0, z, z, Q)
        s.init_forces()
        s.step(400)
        x = s.getdat()
        disp = s.displacement()
    if precision == "fp32":
        x0 = f32(x0)
    wraps = (x0 + disp - x) / spec.box
    tol = 1e-9 if precision == "fp64" else 2e-3
    assert np.abs(wraps - np.round(wraps)).max() * spec.box <= tol
    assert np.isfinite(disp).all() and np.abs(disp).max() > 0.05  # the particles did move


def test_walled_box_trajectory_fp64_vs_oracle():
    """Reflecting walls (cube with periodic = false): positions reflect and momenta flip at the faces
    (geometry.h:403-446).  Fast initial momenta make particles hit the walls within 100 steps."""
    spec = ReplicaSpec(n=300, box=box_for(300, 0.2), model=crowded_model(100, 300), periodic=False, kT=0.0)
    x = random_positions(spec.n, spec.box, False, 0.95, 13)
    Q = random_rotations(spec.n, 14)
    rng = np.random.default_rng(15)
    p = rng.normal(size=(spec.n, 3)) * 6.0
    L = rng.normal(size=(spec.n, 3)) * 0.2
    with LangevinNVTRGPU([spec], precision="fp64") as s:
        s.initialize(x, p, L, Q)
        s.init_forces()
        s.step(100)
        got = s.get_state()
    sysm = po.System(spec)
    st = dict(x=x.copy(), p=p.copy(), Lb=L.copy(), Q=Q.copy())
    st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"])
    assert sysm.run(st, 100, noise_mode=0) == 0
    for key in ("x", "p", "Lb", "Q"):
        scale = max(1.0, np.abs(st[key]).max())
        assert np.abs(got[key] - st[key]).max() <= 1e-9 * scale, key
    assert (got["x"] >= 0).all() and (got["x"] <= spec.box).all()


def test_equipartition_with_live_noise_fp32():
    spec = tetra_spec(4000, 0.10, kT=1.0, seed=21)
    x = random_positions(spec.n, spec.box, True, 0.95, 22)
    Q = random_rotations(spec.n, 23)
    z = np.zeros((spec.n, 3))
    temps = []
    with LangevinNVTRGPU([spec], precision="fp32") as s:
        s.initialize(x, z, z, Q)
        s.init_forces()
        s.step(600)
        for _ in range(100):
            s.step(10)
            temps.append(s.measured_temperature()[0])
    t = np.mean(temps, axis=0)
    assert np.allclose(t, 0.5 * spec.kT, rtol=0.04), t


def test_patch_energy_statistics_match_oracle():
    """Same ensemble, independent trajectories: the FP32 batched path and the FP64 oracle loop, both
    with live Philox noise, give the same mean patch energy and WCA energy per particle."""
    spec = tetra_spec(800, 0.25, kT=0.9, seed=31)
    x = random_positions(spec.n, spec.box, True, 0.95, 32)
    Q = random_rotations(spec.n, 33)
    z = np.zeros((spec.n, 3))
    burn, blocks, per = 1500, 20, 150
    gpu = []
    with LangevinNVTRGPU([spec], precision="fp32") as s:
        s.initialize(x, z, z, Q)
        s.init_forces()
        s.step(burn)
        for _ in range(blocks):
            acc = np.zeros(2)
            for _ in range(3):
                s.step(per // 3)
                acc += s.observables()[0][:2]
            gpu.append(acc / 3)
    sysm = po.System(spec)
    st = dict(x=x.copy(), p=z.copy(), Lb=z.copy(), Q=Q.copy())
    noise0 = po.philox_noise(spec.n, spec.seed + 1000, 0, 0)
    st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"], noise=noise0)
    draw = 1
    sysm.run(st, burn, noise_mode=2, seed=spec.seed + 1000, draw0=draw, check_skin=False)
    draw += burn
    orc = []
    for _ in range(blocks):
        acc = np.zeros(2)
        for _ in range(3):
            sysm.run(st, per // 3, noise_mode=2, seed=spec.seed + 1000, draw0=draw, check_skin=False)
            draw += per // 3
            acc += sysm.observables(st["x"], st["Q"])[:2]
        orc.append(acc / 3)
    gpu, orc = np.array(gpu) / spec.n, np.array(orc) / spec.n
    for i, name in enumerate(("patch energy", "WCA energy")):
        m1, m2 = gpu[:, i].mean(), orc[:, i].mean()
        se = math.sqrt(gpu[:, i].var(ddof=1) / blocks + orc[:, i].var(ddof=1) / blocks)
        assert abs(m1 - m2) <= 4 * se + 0.02 * abs(m2), (name, m1, m2, se)


@pytest.mark.parametrize("precision", PRECISIONS)
def test_step_temperatures_equal_the_step_by_step_read_back(precision):
    """mtg_step_temperatures (per-step sums copied asynchronously, one synchronisation) gives, step by step,
    what mtg_step(1) + mtg_temperature give, and leaves the same state (bit for bit in FP32; the temperature
    sums meet in double-precision atomics, whose order moves the last bits)."""
    spec = tetra_spec(600, 0.2)
    x = random_positions(spec.n, spec.box, True, 0.95, 31)
    Q = random_rotations(spec.n, 32)
    z = np.zeros((spec.n, 3))
    nsteps = 12
    with LangevinNVTRGPU([spec, spec], precision=precision) as s:
        s.initialize(np.concatenate([x, x]), np.concatenate([z, z]), np.concatenate([z, z]), np.concatenate([Q, Q]))
        got = s.step_temperatures(nsteps)
        st_got = s.get_state()
    want = []
    with LangevinNVTRGPU([spec, spec], precision=precision) as s:
        s.initialize(np.concatenate([x, x]), np.concatenate([z, z]), np.concatenate([z, z]), np.concatenate([Q, Q]))
        for _ in range(nsteps):
            s.step(1)
            want.append(s.measured_temperature())
        st_want = s.get_state()
    assert got.shape == (nsteps, 2, 6)
    np.testing.assert_allclose(got, np.array(want), rtol=1e-12, atol=0)
    for key in ("x", "p", "Lb", "Q"):
        if precision == "fp32":  # fixed-point force sums: bit-reproducible
            assert np.array_equal(st_got[key], st_want[key]), key
        else:  # FP64 sums a particle's neighbours in slot order, and ranks within a cell come from atomics
            np.testing.assert_allclose(st_got[key], st_want[key], rtol=1e-10, atol=1e-12, err_msg=key)
    assert got[-1].min() > 0


def test_step_temperatures_across_ring_chunks():
    """The per-step sums of mtg_step_temperatures wait in a device ring of at most 32 MB, copied back once per
    chunk of steps: 3,000 replicas (144 KB of sums a step, 233 steps a chunk) over 250 steps cross a chunk
    boundary, and every step still equals mtg_step(1) + mtg_temperature."""
    nrep, n, nsteps = 3000, 12, 250
    specs = [tetra_spec(n, 0.2) for _ in range(nrep)]
    x = np.concatenate([random_positions(n, specs[0].box, True, 0.95, 100 + r) for r in range(nrep)])
    Q = np.concatenate([random_rotations(n, 200 + r) for r in range(nrep)])
    z = np.zeros((nrep * n, 3))
    with LangevinNVTRGPU(specs) as s:
        s.initialize(x, z, z, Q)
        got = s.step_temperatures(nsteps)
    want = []
    with LangevinNVTRGPU(specs) as s:
        s.initialize(x, z, z, Q)
        for _ in range(nsteps):
            s.step(1)
            want.append(s.measured_temperature())
    assert got.shape == (nsteps, nrep, 6)
    np.testing.assert_allclose(got, np.array(want), rtol=1e-12, atol=0)


@pytest.mark.parametrize("precision,kernel", [("fp32", "pairs"), ("fp32", "tiled"), ("fp64", "pairs")])
def test_temperature_after_steps_matches_oracle(precision, kernel):
    """After steps, mtg_temperature / mtg_step_temperatures (the pair pipeline's epilogue sums where that
    path runs, a reduction over the state otherwise) equal the oracle's temperature of the downloaded
    momenta; replica sizes that are not multiples of 32 put replica boundaries inside warps."""
    specs = [tetra_spec(n, 0.2) for n in (333, 517, 1000)]
    xs = [random_positions(sp.n, sp.box, True, 0.95, 40 + r) for r, sp in enumerate(specs)]
    Qs = [random_rotations(sp.n, 50 + r) for r, sp in enumerate(specs)]
    off = np.concatenate([[0], np.cumsum([sp.n for sp in specs])])
    z = np.zeros((off[-1], 3))
    with LangevinNVTRGPU(specs, precision=precision, force_kernel=kernel) as s:
        s.initialize(np.concatenate(xs), z, z, np.concatenate(Qs))
        s.step(7)
        got = s.measured_temperature()
        st = s.get_state()
        got2 = s.step_temperatures(3)
        st2 = s.get_state()
    for r, sp in enumerate(specs):
        a, b = off[r], off[r + 1]
        sysm = po.System(sp)
        want = sysm.temperature(np.ascontiguousarray(st["p"][a:b]), np.ascontiguousarray(st["Lb"][a:b]))
        np.testing.assert_allclose(got[r], want, rtol=1e-9, atol=0)
        want2 = sysm.temperature(np.ascontiguousarray(st2["p"][a:b]), np.ascontiguousarray(st2["Lb"][a:b]))
        np.testing.assert_allclose(got2[-1][r], want2, rtol=1e-9, atol=0)
        assert want.min() > 0
