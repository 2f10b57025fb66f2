"""Seeded synthetic workloads with the shapes of the reference's patchy-condensate runs.

Every workload uses L = (N pi / 6 / phi)^(1/3), a uniform start with non-overlap rejection at 0.9 sigma,
uniform random rotations (the LangevinNVTR::initialize construction, LangevinR.cpp:239-267), zero momenta
and zero angular momenta.  No public dataset is involved; everything is generated from the seed.

  patchy_c1   N=4,096 tetrahedral (depth 8, range 1.2, cos 0.90), phi 0.10, kT 1, dt 0.005
  patchy_c2   N=65,536 "tubulin-like": poles (depth 10) + laterals at +-65 deg (depth 6), range 1.15,
              cos 0.92, phi 0.20 (pole-lateral cross depth: 0)
  patchy_c3   N=1,048,576 = 262,144 tetrahedral (depth 7) + 786,432 WCA crowders, phi 0.25
  patchy_c4   512 replicas, N_r log-uniform in [1,024, 32,768], phi 0.15, kT_r ~ U[0.8, 1.2],
              depth_r ~ U[6, 10], range 1.2, cos 0.90, own Philox seed per replica
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations


@dataclass
class Workload:
    name: str
    replicas: list           # ReplicaSpec per replica
    x: np.ndarray            # concatenated initial positions (n_total x 3)
    Q: np.ndarray            # concatenated initial orientations (n_total x 9)

    @property
    def n_total(self) -> int:
        return int(sum(r.n for r in self.replicas))

    def zeros3(self) -> np.ndarray:
        return np.zeros((self.n_total, 3))


def box_for(n: int, phi: float) -> float:
    return (n * math.pi / 6.0 / phi) ** (1.0 / 3.0)


def _state(replicas, seed: int, min_dist: float = 0.9):
    xs, qs = [], []
    for r, rep in enumerate(replicas):
        xs.append(random_positions(rep.n, rep.box, rep.periodic, min_dist, seed * 1000003 + 2 * r))
        qs.append(random_rotations(rep.n, seed * 1000003 + 2 * r + 1))
    return np.concatenate(xs), np.concatenate(qs)


def tubulin_model(n: int, depth_pole: float = 10.0, depth_lat: float = 6.0, dis: float = 1.15,
                  cos_max: float = 0.92, depth_cross: float = 0.0) -> PatchModelSpec:
    a = math.radians(65.0)
    orient = np.array([[0, 0, 1.0], [0, 0, -1.0], [math.cos(a), math.sin(a), 0], [math.cos(a), -math.sin(a), 0]])
    th = math.acos(cos_max)
    params = []
    for i in range(4):
        for j in range(4):
            pole_i, pole_j = i < 2, j < 2
            att = depth_pole if (pole_i and pole_j) else depth_lat if (not pole_i and not pole_j) else depth_cross
            params.append([att, dis, th])
    return PatchModelSpec([4], [n], orient, np.array(params))


def crowded_model(n_patchy: int, n_total: int, depth: float = 7.0, dis: float = 1.2,
                  cos_max: float = 0.90) -> PatchModelSpec:
    from .system import TETRA
    th = math.acos(cos_max)
    return PatchModelSpec([4, 0], [n_patchy, n_total], TETRA.copy(), np.tile([depth, dis, th], (16, 1)))


def patchy_c1(seed: int = 0, n: int = 4096, phi: float = 0.10, kT: float = 1.0) -> Workload:
    box = box_for(n, phi)
    rep = ReplicaSpec(n=n, box=box, model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.90)), kT=kT,
                      seed=seed)
    x, Q = _state([rep], seed)
    return Workload("patchy_c1", [rep], x, Q)


def patchy_c2(seed: int = 0, n: int = 65536, phi: float = 0.20) -> Workload:
    rep = ReplicaSpec(n=n, box=box_for(n, phi), model=tubulin_model(n), seed=seed)
    x, Q = _state([rep], seed)
    return Workload("patchy_c2", [rep], x, Q)


def patchy_c3(seed: int = 0, n: int = 1048576, phi: float = 0.25) -> Workload:
    n_patchy = n // 4
    rep = ReplicaSpec(n=n, box=box_for(n, phi), model=crowded_model(n_patchy, n), seed=seed)
    x, Q = _state([rep], seed)
    return Workload("patchy_c3", [rep], x, Q)


def c4_sizes(n_replicas: int = 512, n_min: int = 1024, n_max: int = 32768, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.round(np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_replicas))).astype(int)


def patchy_c4(seed: int = 0, n_replicas: int = 512, n_min: int = 1024, n_max: int = 32768,
              phi: float = 0.15) -> Workload:
    rng = np.random.default_rng(seed + 7)
    sizes = c4_sizes(n_replicas, n_min, n_max, seed)
    reps = []
    for r, n in enumerate(sizes):
        n = int(n)
        kT = float(rng.uniform(0.8, 1.2))
        depth = float(rng.uniform(6.0, 10.0))
        reps.append(ReplicaSpec(n=n, box=box_for(n, phi),
                                model=PatchModelSpec.tetrahedral(n, depth, 1.2, math.acos(0.90)), kT=kT,
                                seed=(seed << 20) + r))
    x, Q = _state(reps, seed)
    return Workload("patchy_c4", reps, x, Q)


WORKLOADS = {"c1": patchy_c1, "c2": patchy_c2, "c3": patchy_c3, "c4": patchy_c4}
