"""The random initial binding (LangevinNVTR::setup_random_binding, LangevinRforceUtil.cpp:749-1010): the oracle's
restatement pinned to the reference, on the single-bond fixtures' configurations and bond states.

The reference walks its edges in a std::random_device shuffle, so no two runs agree; what every run must satisfy
pins the restatement instead.  With E the oracle's edges whose score is below 4 (the edge test of the bond
update plus scr4 = -log(1e-10 + calculate_score)):
  - every bond the reference makes is an edge of E (E holds every edge the reference can take);
  - after the reference's walk no edge of E has both patches unbound (E holds no edge the reference would have
    refused: an extra edge whose patches the walk left free would show here);
  - bonds of the state before the call stay.
The oracle's own walk (the library's seeded order) must satisfy the same, repeat itself for a seed and change
with the seed.  The GPU path is compared with it in tests/test_gpu_setup_binding.py.
"""
import numpy as np
import pytest

from oracle import pyoracle as po
from tests._util import load, spec_from
from tests.test_oracle_bind import binding_of, candidates


def bonds(bt, ib, before_ib):
    return {(min(i, int(bt[i])), max(i, int(bt[i]))) for i in range(len(ib)) if ib[i] and not before_ib[i]}


def check_walk(bt, ib, bt0, ib0, eligible):
    new = bonds(bt, ib, ib0)
    assert new <= eligible, sorted(new - eligible)[:5]
    free = [e for e in eligible if not ib[e[0]] and not ib[e[1]]]
    assert not free, free[:5]
    for i in np.flatnonzero(ib0):
        assert ib[i] and bt[i] == bt0[i]
    for a, b in new:
        assert bt[a] == b and bt[b] == a


def case(k, rnd):
    d = load(f"singlebond_{k}.npz")
    spec = spec_from(d)
    sysm = po.System(spec)
    B = binding_of(d)
    x, Q = d["x"], d["Q"][rnd]
    bt0 = np.ascontiguousarray(d["bt_in"][rnd], dtype=np.intc)
    ib0 = np.ascontiguousarray(d["ib_in"][rnd], dtype=np.uint8)
    pl = candidates(sysm, x, Q, sysm.default_max_ang())
    ab, scr = sysm.setup_edges(x, Q, pl, B, bt0, ib0)
    eligible = {(min(int(a), int(b)), max(int(a), int(b))) for (a, b), s in zip(ab, scr) if s < 4.0}
    return d, spec, sysm, B, x, Q, bt0, ib0, pl, eligible


@pytest.mark.skipif(po.ref() is None, reason="the reference shim (oracle/_ref) is only built where the reference "
                                             "sources exist")
@pytest.mark.parametrize("k", range(8))
@pytest.mark.parametrize("rnd", [0, 1])
def test_reference_walks_are_maximal_matchings_of_the_oracle_edges(k, rnd):
    d, spec, sysm, B, x, Q, bt0, ib0, pl, eligible = case(k, rnd)
    for _ in range(3):
        bt, ib = po.ref_setup_random_binding(spec, x, Q, 2.5, int(d["bm_kind"]), d["args"], bt0, ib0)
        check_walk(bt, ib, bt0, ib0, eligible)


@pytest.mark.parametrize("k", range(8))
@pytest.mark.parametrize("rnd", [0, 1])
def test_oracle_walk_is_a_seeded_maximal_matching(k, rnd):
    d, spec, sysm, B, x, Q, bt0, ib0, pl, eligible = case(k, rnd)
    runs = []
    for seed in (1, 1, 2):
        bt, ib = bt0.copy(), ib0.copy()
        assert sysm.setup_random_binding(x, Q, pl, B, bt, ib, seed=seed) == 0
        check_walk(bt, ib, bt0, ib0, eligible)
        runs.append(bonds(bt, ib, ib0))
    assert runs[0] == runs[1]
    free0 = [e for e in eligible if not ib0[e[0]] and not ib0[e[1]]]
    if len(free0) > 50 and len(runs[0]) < len(free0):
        assert runs[0] != runs[2]   # a contested matching depends on the order


def test_fixtures_exercise_the_score_threshold():
    """Some fixture has edges whose score is 4 or more (calculate_score below ~e^-2) and some has none."""
    fractions = []
    for k in range(8):
        d, spec, sysm, B, x, Q, bt0, ib0, pl, _ = case(k, 0)
        ab, scr = sysm.setup_edges(x, Q, pl, B, bt0, ib0)
        if len(scr):
            fractions.append(float((scr < 4.0).mean()))
    assert min(fractions) < 0.5 and max(fractions) == 1.0
