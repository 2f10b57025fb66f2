"""Bond decisions at the thresholds of the edge test (single-bond mode, LangevinRforce.cpp:3010-3060).

An FP32 handle tests an edge in float and re-decides in FP64 where a float test falls within a margin of its
threshold (2e-5 on cosines, 1e-5 relative on distances): in the listed edge pass such a patch pair goes to a
recheck list and a second kernel repeats it with the FP64 tests.  Here every patch pair sits at a threshold:
isolated groups of particles where patch 0 of A faces patch 0 of B, at a distance within 3e-5 (relative) of
the range of its bond-state class (disp = 1.4 dis when neither or both-to-each-other are bound, 0.7 disp when
one is bound, 0.5 disp when both are bound elsewhere; at disp the force pass's max_check is the same
number), with both cosines within 3e-5 of cos(thetam) or clear of it.  The bond state after one update must
equal the oracle's exactly, in FP32 (pair pipeline and per particle) and FP64.
"""
import math

import numpy as np
import pytest

from mtcode_gb300.system import PatchModelSpec, ReplicaSpec
from oracle import pyoracle as po

GROUPS = 4 * 4 * 4
SPACING = 8.0
DIS, CTM = 1.2, 0.9
DISP = 1.4 * DIS
N0 = np.array([math.sqrt(8 / 9), 0.0, -1 / 3])   # patch 0 of TetrahedralPatch, body frame


def rotation_to(a, b):
    """Rotation matrix taking unit vector a to unit vector b (Rodrigues)."""
    v = np.cross(a, b)
    c = float(np.dot(a, b))
    K = np.array([[0, -v[2], v[1]], [v[2], 0, -v[0]], [-v[1], v[0], 0]])
    return np.eye(3) + K + K @ K / (1 + c)


def about(axis, phi):
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    return np.eye(3) + math.sin(phi) * K + (1 - math.cos(phi)) * K @ K


def facing(t, rng):
    """Q (lab -> body, rows) whose patch 0 points along lab direction t: Q^T n0 = t, random about n0."""
    return about(N0, rng.uniform(0, 2 * math.pi)) @ rotation_to(t / np.linalg.norm(t), N0)


def cone_dir(sign, cos_t, rng):
    s = math.sqrt(max(0.0, 1 - cos_t * cos_t))
    psi = rng.uniform(0, 2 * math.pi)
    return np.array([sign * cos_t, s * math.cos(psi), s * math.sin(psi)])


def build(seed, precision):
    """Groups of four particles (A, B, C, D) on a periodic lattice; A-B at a threshold of the class the group
    sets up: class 0 (no bonds), class 2 (A0 bound to C0), class 1 (A0 to C0 and B0 to D0)."""
    rng = np.random.default_rng(seed)
    n = 4 * GROUPS
    box = 4 * SPACING
    x = np.zeros((n, 3))
    Q = np.zeros((n, 9))
    bt = np.zeros(4 * n, np.int32)
    ib = np.zeros(4 * n, np.uint8)
    cls = np.zeros(GROUPS, int)
    for g in range(GROUPS):
        o = np.array([g % 4, (g // 4) % 4, g // 16]) * SPACING + 1.0
        c = g % 3
        cls[g] = c
        rng_c = DISP * (1.0, 0.5, 0.7)[c]
        r = rng_c * (1 + rng.uniform(-3e-5, 3e-5))
        a, b, cc, d = 4 * g, 4 * g + 1, 4 * g + 2, 4 * g + 3
        x[a], x[b] = o, o + np.array([r, 0, 0])
        x[cc], x[d] = o + np.array([0, 3.5, 0]), o + np.array([0, 0, 3.5])
        near = lambda: CTM + rng.uniform(-3e-5, 3e-5) if rng.random() < 0.6 else CTM + 0.05
        Q[a] = facing(cone_dir(+1, near(), rng), rng).ravel()
        Q[b] = facing(cone_dir(-1, near(), rng), rng).ravel()
        Q[cc] = facing(rng.normal(size=3), rng).ravel()
        Q[d] = facing(rng.normal(size=3), rng).ravel()
        if c in (1, 2):   # A0 <-> C0
            bt[4 * a], bt[4 * cc] = 4 * cc, 4 * a
            ib[4 * a] = ib[4 * cc] = 1
        if c == 1:        # B0 <-> D0
            bt[4 * b], bt[4 * d] = 4 * d, 4 * b
            ib[4 * b] = ib[4 * d] = 1
    x %= box
    if precision == "fp32":
        x = x.astype(np.float32).astype(np.float64)
        Q = Q.astype(np.float32).astype(np.float64)
    spec = ReplicaSpec(n=n, box=box, periodic=True, model=PatchModelSpec.tetrahedral(n, 8.0, DIS, math.acos(CTM)),
                       kT=1.0, seed=seed)
    return spec, x, Q, bt, ib, cls


def margins(x, Q, cls, box):
    """Per group: the FP64 distance relative to its class range minus 1, and both cosines minus cos(thetam)."""
    out = []
    for g in range(GROUPS):
        a, b = 4 * g, 4 * g + 1
        d = x[a] - x[b]
        d -= box * np.round(d / box)
        r = float(np.linalg.norm(d))
        u = d / r
        m1 = Q[a].reshape(3, 3).T @ N0
        m2 = Q[b].reshape(3, 3).T @ N0
        out.append((r / (DISP * (1.0, 0.5, 0.7)[cls[g]]) - 1, -float(m1 @ u) - CTM, float(m2 @ u) - CTM))
    return np.array(out)


def test_groups_sit_at_the_thresholds():
    """The construction (no GPU): distances and cosines straddle their thresholds, many within the margins."""
    spec, x, Q, bt, ib, cls = build(11, "fp32")
    m = margins(x, Q, cls, spec.box)
    assert (np.abs(m[:, 0]) < 1e-5).sum() >= GROUPS // 5
    assert (m[:, 0] < 0).any() and (m[:, 0] > 0).any()
    assert (np.abs(m[:, 1:]) < 2e-5).sum() >= GROUPS // 4
    assert set(cls) == {0, 1, 2}


@pytest.mark.gpu
@pytest.mark.parametrize("precision,kernel", [("fp32", "pairs"), ("fp32", "per_particle"), ("fp64", "pairs")])
@pytest.mark.parametrize("seed", [11, 12, 13])
def test_bond_decisions_at_thresholds_match_oracle(seed, precision, kernel):
    from mtcode_gb300 import LangevinNVTRGPU
    from mtcode_gb300.system import binding_single
    from tests.test_gpu_singlebond import oracle_update

    spec, x, Q, bt0, ib0, cls = build(seed, precision)
    sysm = po.System(spec)
    B = po.binding_single(1.0, 0.1)
    z = np.zeros((spec.n, 3))
    formed = 0
    with LangevinNVTRGPU([spec], precision=precision, force_kernel=kernel) as s:
        s.set_single_bond(binding_single(1.0, 0.1))
        for rnd in range(3):
            s.initialize(x, z, z, Q)
            s.set_bind_state(bt0, ib0)
            draw = s.draw
            s.bind_update()
            bt, ib = s.get_bind_state()
            bo, io, _, _ = oracle_update(sysm, B, x, Q, bt0, ib0, draw)
            assert np.array_equal(ib, io), f"round {rnd}: {int((ib != io).sum())} isbound differ"
            assert np.array_equal(bt[io == 1], bo[io == 1]), f"round {rnd}: boundto differs"
            assert s.flags == 0
            formed += int(sum(io[16 * g] and bo[16 * g] == 16 * g + 4 for g in range(GROUPS)))   # A0-B0
    assert formed > 0   # some A0-B0 bonds form, so a wrong edge decision would show


@pytest.mark.gpu
def test_bond_decisions_at_thresholds_batched():
    """Three threshold systems in one FP32 handle (pair pipeline): the recheck kernel finds each listed patch
    pair's replica from its global patch index; every replica's bond state equals the oracle's update of that
    replica (its own Philox stream)."""
    from mtcode_gb300 import LangevinNVTRGPU
    from mtcode_gb300.system import binding_single
    from tests.test_gpu_singlebond import oracle_update

    cases = [build(seed, "fp32") for seed in (21, 22, 23)]
    specs = [c[0] for c in cases]
    x = np.concatenate([c[1] for c in cases])
    Q = np.concatenate([c[2] for c in cases])
    bt0 = np.concatenate([c[3] for c in cases])   # replica-local partner indices
    ib0 = np.concatenate([c[4] for c in cases])
    z = np.zeros((len(x), 3))
    B = po.binding_single(1.0, 0.1)
    with LangevinNVTRGPU(specs, precision="fp32", force_kernel="pairs") as s:
        s.set_single_bond(binding_single(1.0, 0.1))
        s.initialize(x, z, z, Q)
        s.set_bind_state(bt0, ib0)
        draw = s.draw
        s.bind_update()
        bt, ib = s.get_bind_state()
        assert s.flags == 0
        for r, (spec, xr, Qr, btr, ibr, _) in enumerate(cases):
            o, npatch = s.patch_offset(r), 4 * spec.n
            bo, io, _, _ = oracle_update(po.System(spec), B, xr, Qr, btr, ibr, draw, replica=r)
            assert np.array_equal(ib[o:o + npatch], io), f"replica {r}"
            assert np.array_equal(bt[o:o + npatch][io == 1], bo[io == 1]), f"replica {r}"
