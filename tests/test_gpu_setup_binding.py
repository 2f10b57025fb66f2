"""GPU parity of the random initial binding (mtg_setup_random_binding; LangevinNVTR::setup_random_binding,
LangevinRforceUtil.cpp:749-1010, which run_singlebond calls before its loop) through the C ABI.

Each case takes a single-bond fixture's configuration and bond state (an unbound start, and the state after the
reference's own bond update), runs one mtg_setup_random_binding with a seed and compares the bond state with the
oracle's walk in the same seeded order (orc_setup_random_binding): it must agree exactly.  The edge test and the
scores are the reference's FP64 arithmetic on the stored coordinates, in every build; FP32 handles store float
coordinates, so both sides get the float-rounded state.  A batch of replicas checks the per-replica streams, and
a run continues from the set-up state without flags.
"""
import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU
from oracle import pyoracle as po
from tests._util import load, spec_from
from tests.test_gpu_singlebond import gpu_model
from tests.test_oracle_bind import binding_of, candidates

pytestmark = pytest.mark.gpu
CONFIGS = [("fp32", "pairs"), ("fp32", "per_particle"), ("fp64", "pairs")]


def rounded(a, precision):
    return np.asarray(a, np.float32).astype(np.float64) if precision == "fp32" else np.asarray(a, np.float64)


def oracle_setup(sysm, B, x, Q, bt, ib, seed, replica=0):
    bt = np.ascontiguousarray(bt, dtype=np.intc).copy()
    ib = np.ascontiguousarray(ib, dtype=np.uint8).copy()
    pl = candidates(sysm, x, Q, sysm.default_max_ang())
    assert sysm.setup_random_binding(x, Q, pl, B, bt, ib, seed=seed, replica=replica) == 0
    return bt, ib


@pytest.mark.parametrize("precision,kernel", CONFIGS)
@pytest.mark.parametrize("k", range(8))
def test_setup_random_binding_matches_oracle(k, precision, kernel):
    d = load(f"singlebond_{k}.npz")
    spec = spec_from(d)
    sysm = po.System(spec)
    B = binding_of(d)
    z = np.zeros((spec.n, 3))
    x = rounded(d["x"], precision)
    with LangevinNVTRGPU([spec], precision=precision, force_kernel=kernel) as s:
        s.set_single_bond(gpu_model(d))
        for rnd in range(2):
            Q = rounded(d["Q"][rnd], precision)
            s.initialize(x, z, z, Q)
            s.set_bind_state(d["bt_in"][rnd], d["ib_in"][rnd])
            seed = 1000 * k + rnd + 1
            s.setup_random_binding(seed)
            bt, ib = s.get_bind_state()
            bo, io = oracle_setup(sysm, B, x, Q, d["bt_in"][rnd], d["ib_in"][rnd], seed)
            assert np.array_equal(ib, io), f"round {rnd}: {int((ib != io).sum())} isbound differ"
            assert np.array_equal(bt[io == 1], bo[io == 1]), f"round {rnd}: boundto differs"
            assert s.flags == 0


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_setup_random_binding_batch_and_run(precision):
    """Three fixture systems in one handle: each replica's walk has its own priority stream (the replica index is
    part of the Philox counter) and matches the oracle's; 20 steps of the run_singlebond loop then follow."""
    ks = [1, 3, 5]
    ds = [load(f"singlebond_{k}.npz") for k in ks]
    specs = [spec_from(d) for d in ds]
    # one binding model for the batch: the first fixture's
    model, B = gpu_model(ds[0]), binding_of(ds[0])
    xs = [rounded(d["x"], precision) for d in ds]
    Qs = [rounded(d["Q"][0], precision) for d in ds]
    n = sum(sp.n for sp in specs)
    z = np.zeros((n, 3))
    with LangevinNVTRGPU(specs, precision=precision) as s:
        s.set_single_bond(model)
        s.initialize(np.concatenate(xs), z, z, np.concatenate(Qs))
        s.setup_random_binding(77)
        bt, ib = s.get_bind_state()
        for r, (sp, x, Q) in enumerate(zip(specs, xs, Qs)):
            sysm = po.System(sp)
            npatch = sysm.total_patches()
            o = s.patch_offset(r)
            bo, io = oracle_setup(sysm, B, x, Q, np.zeros(npatch, np.intc), np.zeros(npatch, np.uint8), 77, replica=r)
            assert np.array_equal(ib[o:o + npatch], io), f"replica {r}"
            assert np.array_equal(bt[o:o + npatch][io == 1], bo[io == 1]), f"replica {r}"
            assert io.sum() > 0
        s.init_forces()
        s.step(20)
        assert s.flags == 0
        st = s.get_state()
        assert np.isfinite(st["x"]).all()


def test_bond_state_starts_zeroed_and_round_trips():
    """A BinaryBindStore starts zeroed (boundto 0 in each replica's own numbering), and a bond state read back
    from the device can be set again, after steps too (unbound patches keep a partner of their own replica)."""
    ds = [load(f"singlebond_{k}.npz") for k in (1, 3)]
    specs = [spec_from(d) for d in ds]
    n = sum(sp.n for sp in specs)
    z = np.zeros((n, 3))
    with LangevinNVTRGPU(specs, precision="fp32") as s:
        s.set_single_bond(gpu_model(ds[0]))
        s.initialize(np.concatenate([d["x"] for d in ds]), z, z, np.concatenate([d["Q"][0] for d in ds]))
        bt, ib = s.get_bind_state()
        assert not ib.any() and not bt.any()
        s.set_bind_state(bt, ib)
        s.setup_random_binding(3)
        s.init_forces()
        s.step(15)
        bt, ib = s.get_bind_state()
        assert ib.any()
        s.set_bind_state(bt, ib)   # every entry a patch of its replica
        assert s.flags == 0
