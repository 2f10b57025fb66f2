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
    xd = torch.tensor(np.ascontiguousarray(x, dtype=np.float64), device="cuda")
    pd = torch.full((max(cap, 1), 2), -1, dtype=torch.int32, device="cuda")
    nd = torch.zeros(1, dtype=torch.int64, device="cuda")
    stream = torch.cuda.current_stream()
    st = _lib.lib().mtg_pairs_noalloc(C.c_void_p(xd.data_ptr()), len(x), box, int(periodic), rc,
                                     C.c_void_p(pd.data_ptr()), cap, C.c_void_p(nd.data_ptr()),
                                     C.c_void_p(stream.cuda_stream))
    assert st == 0, _lib.STATUS.get(st, st)
    torch.cuda.synchronize()
    n = int(nd.item())
    return pd[: min(n, cap)].cpu().numpy(), n


@pytest.mark.parametrize("k", [0, 2, 4])
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
