"""On-device analysis through the C ABI: calcg1 (pair-distance histogram) and distance_graph (connected
components), against the reference's own results (tests/golden/analysis_*.npz) and the oracle.  Both are
integer outputs computed from FP64 distances with explicit roundings, so the check is exact, in FP32 and
FP64 handles (the fixtures' coordinates are float32-representable)."""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU, MtgError
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
from mtcode_gb300.workloads import box_for
from oracle import pyoracle as po
from tests._util import load, spec_from

pytestmark = pytest.mark.gpu
PRECISIONS = ["fp32", "fp64"]


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("k", range(3))
def test_gr_and_clusters_match_reference(k, precision):
    d = load(f"analysis_{k}.npz")
    spec = spec_from(d)
    z = np.zeros((spec.n, 3))
    Q = np.tile(np.eye(3).ravel(), (spec.n, 1))
    with LangevinNVTRGPU([spec], precision=precision) as s:
        s.initialize(d["x"], z, z, Q)
        h = s.gr(float(d["rmax"]), float(d["dr"]))
        lab = s.clusters(float(d["cut"]))
        h2 = s.gr(float(d["rmax"]), float(d["dr"]))  # a second call gives the same counts
    assert np.array_equal(h, d["hist"])
    assert np.array_equal(h2, d["hist"])
    assert np.array_equal(lab, d["labels"])


def test_analysis_of_one_replica_in_a_batch_after_steps():
    """Replica 1 of a three-replica FP32 batch after 30 steps (particles re-sorted on the device):
    labels and histogram equal the oracle's on the downloaded positions."""
    specs = [ReplicaSpec(n=n, box=box_for(n, phi), model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9)),
                         seed=r)
             for r, (n, phi) in enumerate(((700, 0.2), (3000, 0.3), (500, 0.1)))]
    xs = [random_positions(sp.n, sp.box, True, 0.95, 40 + r) for r, sp in enumerate(specs)]
    Qs = [random_rotations(sp.n, 50 + r) for r, sp in enumerate(specs)]
    n = sum(sp.n for sp in specs)
    z = np.zeros((n, 3))
    with LangevinNVTRGPU(specs, precision="fp32") as s:
        s.initialize(np.concatenate(xs), z, z, np.concatenate(Qs))
        s.init_forces()
        s.step(30)
        x = s.getdat()[700:3700]
        h = s.gr(4.0, 0.04, replica=1)
        lab = s.clusters(1.3, replica=1)
        with pytest.raises(MtgError):
            s.gr(1e3, 0.1, replica=1)   # rmax beyond the box
        with pytest.raises(MtgError):
            s.clusters(1.3, replica=3)  # no such replica
    sysm = po.System(specs[1])
    assert np.array_equal(h, sysm.gr(x, 4.0, 0.04))
    assert np.array_equal(lab, sysm.clusters(x, 1.3))
