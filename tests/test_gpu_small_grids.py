"""Replicas too small for the forward half-stencil: boxes of one or two cells per side, where pair finding scans every
cell of the grid and takes the minimum image of each candidate, batched with larger replicas so that one warp holds
lanes of both kinds (the general row loop).  Forces and torques of every replica against the oracle, periodic and
walled, FP32 and FP64, at the tolerances of test_gpu_parity.py.
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
from oracle import pyoracle as po
from tests._util import force_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
@pytest.mark.parametrize("periodic", [True, False])
def test_one_and_two_cell_grids_batched_with_large_ones(precision, periodic):
    # (particles, box): force range 1.549 sigma, so boxes below 3.1 have one cell per side and below 4.65 two
    sizes = [(6, 2.6), (40, 4.2), (1500, 19.0), (12, 3.3), (3, 2.0), (900, 15.0), (25, 4.0)]
    specs, xs, Qs = [], [], []
    for k, (n, box) in enumerate(sizes):
        specs.append(ReplicaSpec(n=n, box=box, periodic=periodic,
                                 model=PatchModelSpec.tetrahedral(n, 6.0, 1.2, math.acos(0.85)), kT=1.0, seed=k))
        x = random_positions(n, box, periodic, 0.95, 300 + k)
        Q = random_rotations(n, 400 + k)
        if precision == "fp32":
            x, Q = x.astype(np.float32).astype(np.float64), Q.astype(np.float32).astype(np.float64)
        xs.append(x)
        Qs.append(Q)
    ntot = sum(n for n, _ in sizes)
    z = np.zeros((ntot, 3))
    with LangevinNVTRGPU(specs, precision=precision) as s:
        s.initialize(np.concatenate(xs), z, z, np.concatenate(Qs))
        F, T = s.calculate_forces_and_torques3D()
        assert s.flags == 0
    rms = 1e-12 if precision == "fp64" else 1e-5
    off = 0
    for spec, x, Q in zip(specs, xs, Qs):
        Fo, To = po.System(spec).forces(x, Q)
        sl = slice(off, off + spec.n)
        off += spec.n
        if np.abs(Fo).max() == 0:
            assert np.abs(F[sl]).max() == 0
            continue
        assert force_errors(F[sl], Fo)["rms"] <= rms, (spec.n, spec.box)
        if np.abs(To).max() > 0:
            assert force_errors(T[sl], To)["rms"] <= rms, (spec.n, spec.box)
