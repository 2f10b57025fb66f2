"""Live-noise statistics: the FP32 batched path and the FP64 oracle loop, each driven by its own independent
Philox noise, must sample the same ensemble.

Sixteen independent replicas (1,000 tetrahedral patchy particles at phi 0.25, depth 8 kT, range 1.2, cos 0.90,
kT 1) start from the same seeded configurations in both arms: the GPU arm advances all of them in one handle,
the oracle arm advances each with the reference's step restated in FP64.  After 1,000 steps each arm samples,
every 100 steps for 1,000 more, the observables the reference's analysis computes:
  g(r)            calcg1 (MDBase/Analysis/PairCorrelation.cpp:9): pair-distance histogram, r < 3, dr = 0.1
  bonds/particle  the distribution of the number of bonded patch pairs per particle, bonded as
                  LangevinNVTR::calculate_bound_pairs decides (LangevinR.cpp:1854-1998): r < max_check = 1.4 dis
                  and both patch cosines above cos(thetam)
  temperature     measured_temperature (LangevinR.cpp:170-193), per axis
Each replica's time average is one block; the replicas are independent, so the blocks of an arm are iid.  For
every observable component the two arms' block means must agree within 4.5 standard errors of the
difference (sqrt(s_gpu^2 / R + s_oracle^2 / R)): a false alarm on one component has probability below 1e-5,
while a wrong patch depth, cone or noise amplitude shifts the bond distribution by many standard errors.
"""
from __future__ import annotations

import math
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, TETRA, random_positions, random_rotations
from mtcode_gb300.workloads import box_for
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

N, PHI, R = 1000, 0.25, 16
BURN, SAMPLES, EVERY = 1000, 10, 100
RMAX, DR = 3.0, 0.1
COS_M = 0.90
MAXB = 6   # bonds per particle histogram: 0 .. MAXB-1, and MAXB or more


def bonds_per_particle(sysm, spec, x, Q) -> np.ndarray:
    """Histogram of bonded patch pairs per particle (calculate_bound_pairs criterion)."""
    rc = 1.4 * 1.2
    pr = sysm.pairs(x, rc)
    i, j = pr[:, 0], pr[:, 1]
    d = x[i] - x[j]
    d -= spec.box * np.round(d / spec.box)
    r = np.linalg.norm(d, axis=1)
    keep = r < rc
    i, j, d, r = i[keep], j[keep], d[keep], r[keep]
    u = d / r[:, None]
    Qi, Qj = Q[i].reshape(-1, 3, 3), Q[j].reshape(-1, 3, 3)
    # lab patch directions n = Q^T n_body; cos_i = -n_i . u, cos_j = n_j . u
    ni = np.einsum("pki,ak->pai", Qi, TETRA)
    nj = np.einsum("pki,ak->pai", Qj, TETRA)
    ci = -np.einsum("pai,pi->pa", ni, u)
    cj = np.einsum("pai,pi->pa", nj, u)
    nb = ((ci[:, :, None] > COS_M) & (cj[:, None, :] > COS_M)).sum(axis=(1, 2))
    per = np.bincount(i, weights=nb, minlength=spec.n) + np.bincount(j, weights=nb, minlength=spec.n)
    return np.bincount(np.minimum(per.astype(int), MAXB), minlength=MAXB + 1) / spec.n


def observables(sysm, spec, x, Q, hist, temp) -> np.ndarray:
    return np.concatenate([hist / spec.n, bonds_per_particle(sysm, spec, x, Q), temp])


def replicas():
    specs, xs, Qs = [], [], []
    box = box_for(N, PHI)
    for r in range(R):
        specs.append(ReplicaSpec(n=N, box=box, model=PatchModelSpec.tetrahedral(N, 8.0, 1.2, math.acos(COS_M)),
                                 kT=1.0, seed=100 + r))
        xs.append(random_positions(N, box, True, 0.95, 500 + r))
        Qs.append(random_rotations(N, 600 + r))
    return specs, xs, Qs


def gpu_arm(specs, xs, Qs) -> np.ndarray:
    z = np.zeros((N * R, 3))
    blocks = [[] for _ in range(R)]
    with LangevinNVTRGPU(specs, precision="fp32") as s:
        s.initialize(np.concatenate(xs), z, z, np.concatenate(Qs))
        s.init_forces()
        s.step(BURN)
        for _ in range(SAMPLES):
            s.step(EVERY)
            temp = s.measured_temperature()
            st = s.get_state()
            for r in range(R):
                a, b = r * N, (r + 1) * N
                sysm = po.System(specs[r])
                hist = s.gr(RMAX, DR, replica=r)
                blocks[r].append(observables(sysm, specs[r], st["x"][a:b], st["Q"][a:b], hist, temp[r]))
        assert s.flags == 0
    return np.array([np.mean(b, axis=0) for b in blocks])


def oracle_arm(specs, xs, Qs) -> np.ndarray:
    def one(r):
        spec = specs[r]
        sysm = po.System(spec)
        z = np.zeros((N, 3))
        seed = spec.seed + 5000   # independent of the GPU arm's noise
        st = dict(x=xs[r].copy(), p=z.copy(), Lb=z.copy(), Q=Qs[r].copy())
        st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"], noise=po.philox_noise(N, seed, 0, 0))
        draw = 1
        sysm.run(st, BURN, noise_mode=2, seed=seed, draw0=draw, check_skin=False)
        draw += BURN
        obs = []
        for _ in range(SAMPLES):
            sysm.run(st, EVERY, noise_mode=2, seed=seed, draw0=draw, check_skin=False)
            draw += EVERY
            hist = sysm.gr(st["x"], RMAX, DR)
            obs.append(observables(sysm, spec, st["x"], st["Q"], hist, sysm.temperature(st["p"], st["Lb"])))
        return np.mean(obs, axis=0)

    po.orc()
    with ThreadPoolExecutor(max_workers=min(R, 16)) as ex:
        return np.array(list(ex.map(one, range(R))))


def test_gr_bond_distribution_and_temperature_match_the_oracle_ensemble():
    specs, xs, Qs = replicas()
    g = gpu_arm(specs, xs, Qs)
    o = oracle_arm(specs, xs, Qs)
    nb = int(math.floor(RMAX / DR))
    names = [f"g(r) bin {k}" for k in range(nb)] + [f"P(bonds={k})" for k in range(MAXB)] + \
            [f"P(bonds>={MAXB})"] + ["<p_x^2/2m>", "<p_y^2/2m>", "<p_z^2/2m>", "<L_x^2/2I>", "<L_y^2/2I>", "<L_z^2/2I>"]
    assert g.shape == o.shape == (R, len(names))
    mg, mo = g.mean(axis=0), o.mean(axis=0)
    se = np.sqrt(g.var(axis=0, ddof=1) / R + o.var(axis=0, ddof=1) / R)
    z = np.abs(mg - mo) / np.maximum(se, 1e-12)
    bad = [(names[k], mg[k], mo[k], se[k]) for k in range(len(names)) if z[k] > 4.5 and abs(mg[k] - mo[k]) > 1e-9]
    assert not bad, bad
    # the ensemble is bonded (so the bond comparison has power) and at the bath temperature
    bonded = 1.0 - mo[nb]
    assert bonded > 0.3, bonded
    assert np.allclose(mo[-6:], 0.5, atol=0.05) and np.allclose(mg[-6:], 0.5, atol=0.05)
