"""A bounded device wait that runs out: the kernel gives up, returns, and the host reads MTG_ERR_TIMEOUT.

mtg_clusters' union-find kernels wait on other threads' hooks (parent walks, compare-and-swap retries), each
loop bounded.  mtg_set_wait_limit(1) makes every walk longer than one step give up: the call must report
MTG_ERR_TIMEOUT with MTG_FLAG_TIMEOUT latched, nothing hangs, and the same handle must then, with the flags
cleared and the default bound restored, return the labels the oracle computes.  No fault and no endless loop is
involved: the bound only ends loops early.
"""
import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU, MtgError
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
from mtcode_gb300.workloads import box_for
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

MTG_ERR_TIMEOUT = 7
MTG_FLAG_TIMEOUT = 0x4


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_tiny_wait_limit_reports_timeout_and_the_handle_recovers(precision):
    n = 3000
    spec = ReplicaSpec(n=n, box=box_for(n, 0.35), model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, 0.45))
    x = random_positions(n, spec.box, True, 0.95, 3).astype(np.float32).astype(np.float64)
    Q = random_rotations(n, 4)
    z = np.zeros((n, 3))
    cut = 1.3
    expected = po.System(spec).clusters(x, cut)
    assert len(np.unique(expected)) < n // 2   # components with long parent chains exist
    with LangevinNVTRGPU([spec], precision=precision) as s:
        s.initialize(x, z, z, Q)
        s.set_wait_limit(1)
        with pytest.raises(MtgError) as err:
            s.clusters(cut)
        assert err.value.status == MTG_ERR_TIMEOUT
        assert s.flags & MTG_FLAG_TIMEOUT
        s.clear_flags()
        s.set_wait_limit(0)
        assert np.array_equal(s.clusters(cut), expected)
        assert s.flags == 0
        # the handle still steps normally
        s.init_forces()
        s.step(5)
        assert np.isfinite(s.get_state()["x"]).all()
