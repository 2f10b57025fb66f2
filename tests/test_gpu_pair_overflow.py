"""Pair finding keeps each warp's pairs in its own part of the block's shared-memory buffer (256 pairs per warp);
the pairs beyond it go to the pair list in HBM, which the pair-force kernel takes after the fused pair stage.
A long patch range (max_distance_check 2.14 sigma, interaction distance 2.24 sigma) at packing fraction 0.30
gives about 12 unordered pairs per particle, ~380 per warp, so most warps overflow (and the list, 16 pairs a
particle, still holds every pair of the separate path): forces, torques and energies must still equal the
oracle's (tolerances of test_gpu_parity.py), in the fused and the separate pair path, and FP64.
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
from mtcode_gb300.workloads import box_for
from oracle import pyoracle as po
from tests._util import force_errors

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,fused", [("fp32", 1), ("fp32", 0), ("fp64", 1)])
def test_warp_buffer_overflow_matches_oracle(precision, fused):
    n = 3000
    spec = ReplicaSpec(n=n, box=box_for(n, 0.30), model=PatchModelSpec.tetrahedral(n, 2.0, 1.6, math.acos(0.8)),
                       kT=1.0, max_dist2=4.6, seed=5)
    x = random_positions(n, spec.box, True, 0.95, 71)
    Q = random_rotations(n, 72)
    if precision == "fp32":
        x = x.astype(np.float32).astype(np.float64)
        Q = Q.astype(np.float32).astype(np.float64)
    sysm = po.System(spec)
    pairs = sysm.pairs(x, math.sqrt(4.6))
    assert 10 * n < len(pairs) < 15 * n   # beyond 256 pairs per 32 particles, within the list's 16 per particle
    z = np.zeros((n, 3))
    with LangevinNVTRGPU([spec], precision=precision) as s:
        cfg = s.launch_config
        cfg["fused_pairs"] = fused
        s.launch_config = cfg
        s.initialize(x, z, z, Q)
        F, T = s.calculate_forces_and_torques3D()
        obs = s.observables()[0]
        assert s.flags == 0
    Fo, To = sysm.forces(x, Q)
    rms, worst = (1e-12, 1e-11) if precision == "fp64" else (1e-5, 1e-4)
    ef, et = force_errors(F, Fo), force_errors(T, To)
    assert ef["rms"] <= rms and et["rms"] <= rms, (ef, et)
    assert ef["max"] <= worst, ef
    obs_o = sysm.observables(x, Q)
    e_tol = 1e-11 if precision == "fp64" else 1e-5
    assert abs(obs[0] - obs_o[0]) <= e_tol * abs(obs_o[0])
