"""mtcode_gb300 -- GB300 (sm_103a) rotational-Langevin step for patchy spheres.

A from-scratch GPU implementation of the per-timestep hot path of osmanovicdino/mtcode
(cell list, WCA core + Kern-Frenkel patch force/torque, translational + rotational Langevin update)
behind a C ABI (include/mtcode_gb300.h).  ``LangevinNVTRGPU`` is the host-side mirror of the
reference's LangevinNVTR interface over that ABI.
"""
from ._lib import MtgError, lib
from .system import LangevinNVTRGPU, PatchModelSpec, ReplicaSpec, random_positions, random_rotations

__all__ = ["LangevinNVTRGPU", "PatchModelSpec", "ReplicaSpec", "MtgError", "lib", "random_positions",
           "random_rotations"]
