"""The pair build that allocates nothing (mtg_pairs_noalloc), called through the C ABI.

It serves callers that cannot allocate device memory when they need the pair list (code inside
another framework's memory pool, or a host application that forbids allocations in its step loop);
its scratch is a fixed array inside the library.  Checked here against the allocating entry point
(mtg_pairs through a handle) and the reference's own pair set: the sets must be identical -- the
bit-exact pair-set standard of the other pair tests -- on two calls in a row, which share and reuse
the scratch array.  The file sorts last so that a run stopping at its first failure has already run
every other test; it passes alone in a fresh process as well.
"""
import ctypes as C

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU, _lib
from tests._util import load, sorted_pairs, spec_from

pytestmark = pytest.mark.gpu


def noalloc_pairs(x: np.ndarray, box: float, periodic: bool, rc: float, cap: int):
    import torch
    x = np.ascontiguousarray(np.asarray(x, dtype=np.float64).reshape(-1, 3))
    xd = torch.tensor(x if len(x) else np.zeros((1, 3)), device="cuda")
    pd = torch.full((max(cap, 1), 2), -1, dtype=torch.int32, device="cuda")
    nd = torch.full((1,), -7, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    st = _lib.lib().mtg_pairs_noalloc(C.c_void_p(xd.data_ptr()), len(x), box, int(periodic), rc,
                                     C.c_void_p(pd.data_ptr()), cap, C.c_void_p(nd.data_ptr()),
                                     C.c_void_p(stream.cuda_stream))
    assert st == 0, _lib.STATUS.get(st, st)
    torch.cuda.synchronize()
    n = int(nd.item())
    return pd[: min(n, cap)].cpu().numpy(), n


# fixtures 4-6 are grids of two and three cells per side (the shortened and de-duplicated stencils)
@pytest.mark.parametrize("k", range(7))
def test_noalloc_pairs_match_allocating_entry_point_twice(k):
    d = load(f"pairs_{k}.npz")
    spec = spec_from(d)
    rc = float(d["rc"])
    with LangevinNVTRGPU([spec], precision="fp64") as s:
        s.initialize(d["x"], np.zeros((spec.n, 3)), np.zeros((spec.n, 3)), np.tile(np.eye(3).ravel(), (spec.n, 1)))
        expected = sorted_pairs(s.calculatepairs_parallel(rc))
    assert np.array_equal(expected, d["pairs"])
    for _ in range(2):  # the second call reuses the scratch the first left behind
        got, n = noalloc_pairs(d["x"], spec.box, spec.periodic, rc, cap=len(expected) + 16)
        assert n == len(expected)
        assert np.array_equal(sorted_pairs(got), expected)


def test_noalloc_rejects_sizes_beyond_its_scratch():
    L = _lib.lib()
    n = _lib.MTG_NOALLOC_MAX_PARTICLES + 1
    st = L.mtg_pairs_noalloc(C.c_void_p(1), n, 100.0, 1, 1.5, C.c_void_p(1), 10, C.c_void_p(1), None)
    assert st == 1  # MTG_ERR_ARG, nothing launched
    st = L.mtg_pairs_noalloc(C.c_void_p(1), 10, 1000.0, 1, 1.0, C.c_void_p(1), 10, C.c_void_p(1), None)
    assert st == 1  # 1000^3 cells exceed MTG_NOALLOC_MAX_CELLS


def test_noalloc_short_buffer_reports_the_full_count():
    """cap below the total: npairs is still the full count, and only cap pairs (all of them genuine) are
    written."""
    d = load("pairs_1.npz")
    spec = spec_from(d)
    expected = d["pairs"]
    total = len(expected)
    assert total >= 4
    got, n = noalloc_pairs(d["x"], spec.box, spec.periodic, float(d["rc"]), cap=total // 2)
    assert n == total
    assert len(got) == total // 2
    got = sorted_pairs(got)
    exp_set = {tuple(p) for p in expected.tolist()}
    assert all(tuple(p) in exp_set for p in got.tolist())
    assert len({tuple(p) for p in got.tolist()}) == len(got)   # no pair written twice


def test_noalloc_empty_input():
    got, n = noalloc_pairs(np.zeros((0, 3)), 10.0, True, 1.5, cap=8)
    assert n == 0 and len(got) == 0


@pytest.mark.parametrize("periodic", [True, False])
def test_noalloc_small_box_matches_allocating_entry_point(periodic):
    """A box of fewer than three cells per side (the shortened stencil), against mtg_pairs."""
    from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions
    n, box, rc = 60, 3.3, 1.5   # floor(3.3 / 1.5) = 2 cells per side
    spec = ReplicaSpec(n=n, box=box, periodic=periodic, model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, 0.45))
    x = random_positions(n, box, periodic, 0.5, 5)
    with LangevinNVTRGPU([spec], precision="fp64") as s:
        s.initialize(x, np.zeros((n, 3)), np.zeros((n, 3)), np.tile(np.eye(3).ravel(), (n, 1)))
        expected = sorted_pairs(s.calculatepairs_parallel(rc))
    assert len(expected) > 0
    for _ in range(2):
        got, m = noalloc_pairs(x, box, periodic, rc, cap=len(expected) + 4)
        assert m == len(expected)
        assert np.array_equal(sorted_pairs(got), expected)
