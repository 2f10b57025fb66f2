"""Helpers shared by the tests: fixture loading and comparison metrics."""
from __future__ import annotations

import math
from pathlib import Path

import numpy as np

from mtcode_gb300.system import PatchModelSpec, ReplicaSpec

GOLDEN = Path(__file__).resolve().parent / "golden"


def load(name: str) -> dict:
    with np.load(GOLDEN / name, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def spec_from(d: dict, **over) -> ReplicaSpec:
    model = PatchModelSpec([int(v) for v in d["patches_per_type"]], [int(v) for v in d["count_per_type"]],
                           np.asarray(d["orient"], float), np.asarray(d["params"], float))
    kw = dict(n=int(d["n"]), box=float(d["box"]), model=model, periodic=bool(int(d["periodic"])), dt=float(d["dt"]),
              kT=float(d["kT"]), gamma=float(d["gamma"]), gammar=float(d["gammar"]), mass=float(d["mass"]),
              inertia=float(d["inertia"]), hs_eps=float(d["hs_eps"]), hs_sigma=float(d["hs_sigma"]),
              max_dist2=float(d["max_dist2"]), seed=int(d["seed"]))
    kw.update(over)
    return ReplicaSpec(**kw)


def sorted_pairs(p: np.ndarray) -> np.ndarray:
    p = np.sort(np.asarray(p).reshape(-1, 2), axis=1)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def rel_err(a: np.ndarray, b: np.ndarray, floor: float = 1.0) -> float:
    """max over particles of |a_i - b_i| / max(|b_i|, floor): per-particle vector relative error.

    The floor (in force units, eps/sigma) keeps particles whose force nearly cancels from dominating;
    it is stated next to every tolerance that uses it."""
    a = np.asarray(a).reshape(len(b), -1)
    b = np.asarray(b).reshape(len(b), -1)
    num = np.linalg.norm(a - b, axis=1)
    den = np.maximum(np.linalg.norm(b, axis=1), floor)
    return float((num / den).max())


def norm_rel_err(a, b) -> float:
    """||a - b||_2 / ||b||_2 over all particles (global relative error)."""
    a = np.asarray(a).ravel()
    b = np.asarray(b).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def force_errors(a, b) -> dict:
    """Error of a per-particle vector field a against the reference b (both n x 3):
    rms   ||a - b||_2 / ||b||_2 over all particles -- the force relative error of the tests;
    max   max_i |a_i - b_i| / rms_i |b_i|  -- the worst particle, in units of the RMS force.
    (A per-particle relative error |a_i - b_i| / |b_i| is ill-conditioned where pair forces of tens of
    eps/sigma cancel to a small net force, so it is reported only against the RMS scale.)"""
    a = np.asarray(a).reshape(len(b), -1)
    b = np.asarray(b).reshape(len(b), -1)
    d = np.linalg.norm(a - b, axis=1)
    nb = np.linalg.norm(b, axis=1)
    scale = max(float(np.sqrt((nb ** 2).mean())), 1e-300)
    return {"rms": float(np.linalg.norm(d) / max(np.linalg.norm(nb), 1e-300)), "max": float(d.max() / scale)}
