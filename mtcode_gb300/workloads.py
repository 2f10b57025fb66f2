"""Seeded synthetic workloads with the shapes of the reference's patchy-condensate runs.

Every workload uses L = (N pi / 6 / phi)^(1/3), a uniform start with non-overlap rejection at 0.9 sigma,
uniform random rotations (the LangevinNVTR::initialize construction, LangevinR.cpp:239-267), zero momenta
and zero angular momenta.  No public dataset is involved; everything is generated from the seed.

Every builder takes ``gen``, the source of the seeded positions, rotations and chains: the product
library's generators by default, or any object with the same three functions and outputs (the CPU
baselines pass the oracle's, so that they load nothing from the product library).

  patchy_c1   N=4,096 tetrahedral (depth 8, range 1.2, cos 0.90), phi 0.10, kT 1, dt 0.005
  patchy_c2   N=65,536 "tubulin-like": poles (depth 10) + laterals at +-65 deg (depth 6), range 1.15,
              cos 0.92, phi 0.20 (pole-lateral cross depth: 0)
  patchy_c3   N=1,048,576 = 262,144 tetrahedral (depth 7) + 786,432 WCA crowders, phi 0.25
  patchy_c4   512 replicas, N_r log-uniform in [1,024, 32,768], phi 0.15, kT_r ~ U[0.8, 1.2],
              depth_r ~ U[6, 10], range 1.2, cos 0.90, own Philox seed per replica
  polymer_c5  64 replicas x 2,621 chains x 100 beads (262,100 per replica), phi 0.10, harmonic bonds
              k = 100, r0 = 1, WCA core between all beads, every 10th bead carries -x/+x patches
              (depth 8, range 1.2, cos 0.90), self-avoiding random-walk start (step 1, 0.9 sigma), dt 0.002.
              Patchy beads are numbered first (GeneralPatch types are contiguous index ranges) and the
              bond list is renumbered with them.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import system as _system
from .system import PatchModelSpec, ReplicaSpec


@dataclass
class Workload:
    name: str
    replicas: list           # ReplicaSpec per replica
    x: np.ndarray            # concatenated initial positions (n_total x 3)
    Q: np.ndarray            # concatenated initial orientations (n_total x 9)
    bonds: np.ndarray | None = None   # fixed bonds (n_b x 2 global indices), HarmonicPotential(bond_k, bond_r0)
    bond_k: float = 0.0
    bond_r0: float = 0.0

    @property
    def n_total(self) -> int:
        return int(sum(r.n for r in self.replicas))

    def zeros3(self) -> np.ndarray:
        return np.zeros((self.n_total, 3))


def box_for(n: int, phi: float) -> float:
    return (n * math.pi / 6.0 / phi) ** (1.0 / 3.0)


def _state(replicas, seed: int, min_dist: float = 0.9, gen=None):
    gen = gen or _system
    xs, qs = [], []
    for r, rep in enumerate(replicas):
        xs.append(gen.random_positions(rep.n, rep.box, rep.periodic, min_dist, seed * 1000003 + 2 * r))
        qs.append(gen.random_rotations(rep.n, seed * 1000003 + 2 * r + 1))
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


def patchy_c1(seed: int = 0, n: int = 4096, phi: float = 0.10, kT: float = 1.0, gen=None) -> Workload:
    box = box_for(n, phi)
    rep = ReplicaSpec(n=n, box=box, model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.90)), kT=kT,
                      seed=seed)
    x, Q = _state([rep], seed, gen=gen)
    return Workload("patchy_c1", [rep], x, Q)


def patchy_c2(seed: int = 0, n: int = 65536, phi: float = 0.20, gen=None) -> Workload:
    rep = ReplicaSpec(n=n, box=box_for(n, phi), model=tubulin_model(n), seed=seed)
    x, Q = _state([rep], seed, gen=gen)
    return Workload("patchy_c2", [rep], x, Q)


def patchy_c3(seed: int = 0, n: int = 1048576, phi: float = 0.25, gen=None) -> Workload:
    n_patchy = n // 4
    rep = ReplicaSpec(n=n, box=box_for(n, phi), model=crowded_model(n_patchy, n), seed=seed)
    x, Q = _state([rep], seed, gen=gen)
    return Workload("patchy_c3", [rep], x, Q)


def c4_sizes(n_replicas: int = 512, n_min: int = 1024, n_max: int = 32768, seed: int = 0) -> np.ndarray:
    rng = np.random.default_rng(seed)
    return np.round(np.exp(rng.uniform(math.log(n_min), math.log(n_max), n_replicas))).astype(int)


def patchy_c4(seed: int = 0, n_replicas: int = 512, n_min: int = 1024, n_max: int = 32768,
              phi: float = 0.15, gen=None) -> Workload:
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
    x, Q = _state(reps, seed, gen=gen)
    return Workload("patchy_c4", reps, x, Q)


def bead_model(n_patchy: int, n: int, depth: float = 8.0, dis: float = 1.2, cos_max: float = 0.90) -> PatchModelSpec:
    """Two GeneralPatch types: beads 0 .. n_patchy-1 carry the BivalentPatch pair -x/+x, the rest none."""
    th = math.acos(cos_max)
    return PatchModelSpec([2, 0], [n_patchy, n], np.array([[-1.0, 0, 0], [1.0, 0, 0]]),
                          np.tile([depth, dis, th], (4, 1)).astype(float))


def chain_replica(n_chains: int, beads: int, box: float, every: int, seed: int, periodic: bool = True, gen=None):
    """Random-walk chains with every `every`-th bead patchy, renumbered patchy-first.
    Returns (x, bonds, n_patchy) in the new numbering."""
    xc = (gen or _system).random_chains(n_chains, beads, box, periodic, 1.0, 0.9, seed)
    n = n_chains * beads
    idx = np.arange(n)
    patchy = (idx % beads) % every == 0
    order = np.concatenate([idx[patchy], idx[~patchy]])
    new_of_old = np.empty(n, dtype=np.int64)
    new_of_old[order] = idx
    first = (idx % beads) != beads - 1
    bonds = np.stack([new_of_old[idx[first]], new_of_old[idx[first] + 1]], axis=1).astype(np.int32)
    return np.ascontiguousarray(xc[order]), bonds, int(patchy.sum())


def polymer_c5(seed: int = 0, n_replicas: int = 64, n_chains: int = 2621, beads: int = 100, phi: float = 0.10,
               every: int = 10, k: float = 100.0, r0: float = 1.0, dt: float = 0.002, kT: float = 1.0,
               gen=None) -> Workload:
    from concurrent.futures import ThreadPoolExecutor
    n = n_chains * beads
    box = box_for(n, phi)
    reps = []

    def one(r):
        return chain_replica(n_chains, beads, box, every, seed * 1000003 + 2 * r, gen=gen)

    with ThreadPoolExecutor(max_workers=16) as ex:
        parts = list(ex.map(one, range(n_replicas)))
    xs, qs, bs = [], [], []
    for r, (x, b, n_patchy) in enumerate(parts):
        reps.append(ReplicaSpec(n=n, box=box, model=bead_model(n_patchy, n), kT=kT, dt=dt, seed=(seed << 20) + r))
        xs.append(x)
        qs.append((gen or _system).random_rotations(n, seed * 1000003 + 2 * r + 1))
        bs.append(b + r * n)
    return Workload("polymer_c5", reps, np.concatenate(xs), np.concatenate(qs), np.concatenate(bs), k, r0)


WORKLOADS = {"c1": patchy_c1, "c2": patchy_c2, "c3": patchy_c3, "c4": patchy_c4, "c5": polymer_c5}
