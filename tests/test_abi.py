"""CPU-only checks of the C-ABI library: it loads, exports every symbol include/mtcode_gb300.h
declares, its structs match the ctypes mirror, and its host-side utilities behave.  No GPU calls."""
import ctypes as C
import math
import re
from pathlib import Path

import numpy as np
import pytest

from mtcode_gb300 import _lib
from mtcode_gb300.system import TETRA, PatchModelSpec, random_positions, random_rotations

HEADER = Path(__file__).resolve().parents[1] / "include" / "mtcode_gb300.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mtg_[A-Za-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    bound = {name for name, _, _ in _lib.SIGNATURES}
    assert set(names) == bound, set(names) ^ bound


def test_api_version_and_status_strings():
    L = _lib.lib()
    assert L.mtg_api_version() == 5
    assert L.mtg_status_string(0) == b"ok"
    assert L.mtg_status_string(5) == b"non-finite state on the device"


def test_struct_layout_matches_c():
    L = _lib.lib()
    d = _lib.ReplicaDesc()
    L.mtg_replica_defaults(C.byref(d))
    assert (d.periodic, d.dt, d.kT, d.gamma, d.gammar, d.mass) == (1, 0.005, 1.0, 1.0, 1.0, 1.0)
    assert d.inertia == pytest.approx(0.1) and d.hs_sigma == 1.0 and d.max_dist2 == 2.4
    m = _lib.PatchModel()
    L.mtg_model_tetrahedral(C.byref(m), 8.0, 1.2, math.acos(0.9))
    assert m.n_types == 1 and m.patches_per_type[0] == 4
    assert np.allclose(np.array([list(m.orient[i]) for i in range(4)]), TETRA, atol=0)
    assert all(tuple(m.params[q]) == (8.0, 1.2, math.acos(0.9)) for q in range(16))
    spec = PatchModelSpec.tetrahedral(10, 8.0, 1.2, math.acos(0.9)).to_c()
    assert bytes(spec)[: C.sizeof(_lib.PatchModel)] != b""  # ctypes mirror builds
    L.mtg_model_bivalent(C.byref(m), 3.0, 1.1, 0.5)
    assert m.patches_per_type[0] == 2 and tuple(m.orient[0]) == (-1.0, 0.0, 0.0) and tuple(m.orient[1]) == (1.0, 0, 0)


def test_create_without_device_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    L = _lib.lib()
    reps = (_lib.ReplicaDesc * 1)()
    L.mtg_replica_defaults(C.byref(reps[0]))
    reps[0].n, reps[0].box = 10, 10.0
    L.mtg_model_tetrahedral(C.byref(reps[0].model), 8.0, 1.2, 0.45)
    cfg = _lib.Config(0, 1, C.cast(reps, C.POINTER(_lib.ReplicaDesc)), 0, 1, 0)
    h = C.c_void_p()
    st = L.mtg_create(C.byref(cfg), C.byref(h))
    assert st == 8 and not h.value
    assert L.mtg_last_error(None)


def test_null_handle_is_an_argument_error():
    L = _lib.lib()
    assert L.mtg_step(None, 1) == 1
    assert L.mtg_sync(None) == 1
    assert L.mtg_num_particles(None) == 0


def test_random_positions_respect_min_distance():
    n, box = 3000, 20.0
    x = random_positions(n, box, True, 0.9, 5)
    assert x.shape == (n, 3) and (x >= 0).all() and (x < box).all()
    from oracle import pyoracle as po
    from mtcode_gb300.system import ReplicaSpec
    spec = ReplicaSpec(n=n, box=box, model=PatchModelSpec.tetrahedral(n, 1, 1, 1))
    assert len(po.System(spec).pairs(x, 0.9 * (1 - 1e-12))) == 0
    x2 = random_positions(n, box, True, 0.9, 5)
    assert np.array_equal(x, x2)


def test_random_rotations_are_proper():
    Q = random_rotations(1000, 9).reshape(-1, 3, 3)
    eye = np.einsum("nab,ncb->nac", Q, Q)
    assert np.abs(eye - np.eye(3)).max() < 1e-12
    assert np.allclose(np.linalg.det(Q), 1.0)
    # uniform on SO(3): the mean of every entry vanishes
    assert np.abs(Q.mean(0)).max() < 0.1


def test_overpacked_start_is_rejected():
    with pytest.raises(Exception):
        random_positions(2000, 5.0, True, 0.9, 1)


def test_random_chains_are_self_avoiding_and_seeded():
    """mtg_random_chains (host helper, no GPU): bond length exactly `step`, every pair of beads at least
    min_dist apart (minimum image), in the box, and the same output for the same seed."""
    from mtcode_gb300.system import random_chains
    box = 12.0
    x = random_chains(10, 40, box, True, 1.0, 0.9, 5)
    assert np.array_equal(x, random_chains(10, 40, box, True, 1.0, 0.9, 5))
    assert (x >= 0).all() and (x < box).all()
    d = x[:, None, :] - x[None, :, :]
    d -= box * np.round(d / box)
    r = np.sqrt((d * d).sum(-1))
    np.fill_diagonal(r, np.inf)
    assert r.min() >= 0.9
    idx = np.arange(len(x) - 1)
    bond = idx[idx % 40 != 39]
    assert np.allclose(r[bond, bond + 1], 1.0, rtol=0, atol=1e-12)
    xw = random_chains(6, 30, box, False, 1.0, 0.9, 6)
    assert (xw >= 0).all() and (xw < box).all()
