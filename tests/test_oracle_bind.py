"""Pins the oracle's single-bond restatement (orc_patch_list, orc_bind_update: Condensate::run_singlebond's
force pass) to the reference, and the product's binding-model tables to the oracle's.

The fixtures tests/golden/singlebond_*.npz hold the reference's own calculate_patch_list +
calculate_forces_and_torques3D_onlyone_nonlets (after srand(seed)) over three rounds per case: an unbound
start, the same configuration re-decided with its bonds, then new orientations.  The oracle replays them
with random numbers drawn from the C library's rand() in the reference's order (rng mode 1): the bond
state must match exactly; forces and torques bit for bit on x86-64 (1e-12 elsewhere: long double).
"""
import ctypes
import hashlib
import math
import platform

import numpy as np
import pytest

from oracle import pyoracle as po
from tests._util import load, spec_from

EXACT = platform.machine() in ("x86_64", "AMD64")
CASES = range(8)


def close(a, b, rtol=1e-12):
    if EXACT:
        return np.array_equal(a, b)
    return np.allclose(a, b, rtol=rtol, atol=rtol * max(1.0, np.abs(b).max()))


def binding_of(d) -> po.OrcBinding:
    kind, args, tables = int(d["bm_kind"]), d["args"], d["tables"]
    if kind == 0:
        return po.binding_single(float(args[0]), float(args[1]))
    if kind == 1:
        return po.binding_binary(int(args[0]), tables)
    if kind == 2:
        return po.binding(2, tables[:24], tables[24:], int(args[0]), int(args[1]))
    return po.binding(3, tables[:24], tables[24:], int(args[0]), int(args[1]), int(args[2]))


def candidates(sysm, x, Q, max_ang):
    pairs = sysm.pairs(x, 2.5, max(1, int(math.floor(sysm.spec.box / 2.5))))
    return sysm.patch_list(x, Q, pairs, max_ang)


def plist_sha(pl) -> str:
    pl = np.asarray(pl)[np.lexsort(np.asarray(pl).T[::-1])]
    return hashlib.sha256(np.ascontiguousarray(pl, dtype=np.int32).tobytes()).hexdigest()


@pytest.mark.parametrize("k", CASES)
def test_model_constants_match_reference(k):
    d = load(f"singlebond_{k}.npz")
    sysm = po.System(spec_from(d))
    assert sysm.max_check() == float(d["max_check"])
    assert sysm.default_max_ang() == float(d["max_ang"])
    ppt, cnt = d["patches_per_type"], d["count_per_type"]
    assert sysm.total_patches() == sum(int(ppt[k]) * (int(cnt[k]) - (int(cnt[k - 1]) if k else 0))
                                       for k in range(len(ppt)))


@pytest.mark.parametrize("k", CASES)
def test_candidate_list_matches_reference(k):
    d = load(f"singlebond_{k}.npz")
    sysm = po.System(spec_from(d))
    for rnd in range(3):
        pl = candidates(sysm, d["x"], d["Q"][rnd], float(d["max_ang"]))
        assert len(pl) == int(d["plist_n"][rnd])
        assert plist_sha(pl) == str(d["plist_sha"][rnd])


@pytest.mark.parametrize("k", CASES)
def test_bind_update_matches_reference(k):
    d = load(f"singlebond_{k}.npz")
    sysm = po.System(spec_from(d))
    B = binding_of(d)
    libc = ctypes.CDLL(None)
    for rnd in range(3):
        Q = d["Q"][rnd]
        pl = candidates(sysm, d["x"], Q, float(d["max_ang"]))
        bt = np.ascontiguousarray(d["bt_in"][rnd], dtype=np.intc).copy()
        ib = np.ascontiguousarray(d["ib_in"][rnd], dtype=np.uint8).copy()
        libc.srand(int(d["srand"]) + rnd)
        st, F, T = sysm.bind_update(d["x"], Q, pl, B, bt, ib, rng=1)
        assert st == 0
        assert np.array_equal(ib, d["ib"][rnd]), f"round {rnd}: isbound differs"
        assert np.array_equal(bt, d["bt"][rnd]), f"round {rnd}: boundto differs"
        assert close(F, d["F"][rnd]), f"round {rnd}: F"
        assert close(T, d["T"][rnd]), f"round {rnd}: T"


def test_fixtures_cover_every_cluster_kind():
    """The fixtures reach bound pairs, re-decided bonds and broken bonds under every binding model."""
    kinds = set()
    for k in CASES:
        d = load(f"singlebond_{k}.npz")
        kinds.add(int(d["bm_kind"]))
        assert d["ib"][0].sum() > 0
        kept = (d["ib_in"][1] == 1) & (d["ib"][1] == 1)
        assert kept.sum() > 0
        broken = (d["ib_in"][2] == 1) & (d["ib"][2] == 0)
        assert broken.sum() > 0
    assert kinds == {0, 1, 2, 3}


@pytest.mark.parametrize("seed", [21, 22])
def test_bind_update_live_against_reference(seed):
    """Fresh inputs through the reference shim (present only where the reference sources are)."""
    if po.ref() is None:
        pytest.skip("reference shim not built here")
    from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
    n, phi, cosm = 250, 0.3, 0.72
    box = (n * math.pi / 6 / phi) ** (1 / 3)
    spec = ReplicaSpec(n=n, box=box, model=PatchModelSpec.tetrahedral(n, 7.0, 1.2, math.acos(cosm)), seed=seed)
    x = random_positions(n, box, True, 0.9, seed)
    Q = random_rotations(n, seed + 1)
    sysm = po.System(spec)
    bt = np.zeros(4 * n, dtype=np.intc)
    ib = np.zeros(4 * n, dtype=np.uint8)
    libc = ctypes.CDLL(None)
    for rnd in range(2):
        r = po.ref_singlebond(spec, x, Q, 2.5, 0, [0.8, 0.4], bt, ib, seed + rnd)
        libc.srand(seed + rnd)
        st, F, T = sysm.bind_update(x, Q, candidates(sysm, x, Q, r["max_ang"]), po.binding_single(0.8, 0.4), bt, ib,
                                    rng=1)
        assert st == 0
        assert np.array_equal(ib, r["isbound"]) and np.array_equal(bt, r["boundto"])
        assert np.array_equal(F, r["F"]) and np.array_equal(T, r["T"])


def test_product_binding_tables_match_oracle():
    """mtg_binding_single / mtg_binding_binary_equilibrium (host code of the product, no GPU use) build the
    tables the oracle was pinned with."""
    from mtcode_gb300 import system as S
    m = S.binding_single(0.7, 0.5)
    o = po.binding_single(0.7, 0.5)
    assert m.species_rule == o.rule == 0
    assert np.array_equal(np.ctypeslib.as_array(m.drate), np.ctypeslib.as_array(o.drate))
    assert np.array_equal(np.ctypeslib.as_array(m.trate), np.ctypeslib.as_array(o.trate))
    d = load("singlebond_2.npz")
    div = int(d["args"][0])
    m = S.binding_binary_equilibrium(div)
    o = po.binding_binary(div, d["tables"])
    assert (m.species_rule, m.div1) == (o.rule, o.div1) == (1, div)
    assert np.array_equal(np.ctypeslib.as_array(m.drate), np.ctypeslib.as_array(o.drate))
    assert np.array_equal(np.ctypeslib.as_array(m.trate), np.ctypeslib.as_array(o.trate))


def test_bind_uniform_is_a_fixed_function():
    a = po.bind_uniform(7, 2, 5, 11, 0)
    assert 0.0 <= a < 1.0
    assert a == po.bind_uniform(7, 2, 5, 11, 0)
    assert a != po.bind_uniform(7, 2, 5, 11, 1) and a != po.bind_uniform(7, 2, 6, 11, 0)
    u = np.array([po.bind_uniform(3, 0, 0, i, 0) for i in range(4000)])
    assert abs(u.mean() - 0.5) < 0.02 and u.min() >= 0 and u.max() < 1
