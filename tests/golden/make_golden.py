"""Generates the golden fixtures in this directory by running the REFERENCE's own routines
(osmanovicdino/mtcode, compiled by oracle/build_ref.sh into oracle/_ref/libmtref.so) on seeded inputs.

    python tests/golden/make_golden.py [--reference <reference checkout, the directory holding Code/>]

Inputs are rounded to float32-representable doubles so that the FP32 GPU path, the FP64 GPU path,
the oracle and the reference all start from bit-identical coordinates.  Force cases are re-seeded
until no pair sits within 1e-6 of a branch threshold of the patch potential (cone edge, radial cut,
|c^2-1| = 1e-5): an FP32 evaluation may legitimately fall on the other side of such a threshold.
"""
from __future__ import annotations

import argparse
import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import pyoracle as po  # noqa: E402
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations  # noqa: E402
from mtcode_gb300.workloads import bead_model, box_for, chain_replica, crowded_model, tubulin_model  # noqa: E402

HERE = Path(__file__).resolve().parent
D = po._d


def f32(a):
    return np.ascontiguousarray(np.asarray(a, np.float32).astype(np.float64))


def ref_pairs(spec, x, ncell, rc, parallel=False):
    R = po.ref()
    cap = 64 * len(x) + 64
    out = np.empty((cap, 2), dtype=np.intc)
    fn = R.ref_pairs_parallel if parallel else R.ref_pairs
    n = fn(spec.n, spec.box, int(spec.periodic), D(x), ncell, rc, out.ctypes.data_as(po._I), cap)
    assert n <= cap
    p = np.sort(out[:n], axis=1)
    return p[np.lexsort((p[:, 1], p[:, 0]))]


def ref_forces(spec, x, Q, rc):
    R = po.ref()
    args = po.ref_model_args(spec.model)
    F = np.empty((spec.n, 3))
    T = np.empty((spec.n, 3))
    ncell = max(1, int(math.floor(spec.box / rc)))
    kind, att, dis, th, nt, ppt, npt, orient, params = args
    R.ref_forces(spec.n, spec.box, int(spec.periodic), D(x), D(Q), ncell, rc, spec.hs_eps, spec.hs_sigma, kind, att,
                 dis, th, nt, ppt.ctypes.data_as(po._I), npt.ctypes.data_as(po._I), D(orient), D(params), D(F), D(T))
    return F, T


def ref_forces_bonded(spec, x, Q, rc, bonds, k, r0):
    R = po.ref()
    _, _, _, _, nt, ppt, npt, orient, params = po.ref_model_args(spec.model)
    F = np.empty((spec.n, 3))
    T = np.empty((spec.n, 3))
    ncell = max(1, int(math.floor(spec.box / rc)))
    b = np.ascontiguousarray(bonds, dtype=np.intc)
    R.ref_forces_bonded(spec.n, spec.box, int(spec.periodic), D(x), D(Q), ncell, rc, spec.hs_eps, spec.hs_sigma, nt,
                        ppt.ctypes.data_as(po._I), npt.ctypes.data_as(po._I), D(orient), D(params),
                        b.ctypes.data_as(po._I), len(b), k, r0, D(F), D(T))
    return F, T


def ref_bond_forces(spec, x, bonds, k, r0):
    F = np.empty((spec.n, 3))
    b = np.ascontiguousarray(bonds, dtype=np.intc)
    po.ref().ref_bond_forces(spec.n, spec.box, int(spec.periodic), D(x), b.ctypes.data_as(po._I), len(b), k, r0, D(F))
    return F


def bonded_cases():
    """F. bonded bead systems: harmonic bonds + WCA + patches on every `every`-th bead (patchy first)."""
    cases = [(20, 30, 0.35, 2, True), (24, 25, 0.35, 2, False)]
    for k, (nch, beads, phi, every, per) in enumerate(cases):
        n = nch * beads
        box = box_for(n, phi)
        for seed in range(50):
            x, bonds, n_patchy = chain_replica(nch, beads, box, every, 300 + 10 * k + seed, per)
            # stretch and compress the bonds: +-0.06 per coordinate keeps every bead > 0.78 sigma apart
            x = x + np.random.default_rng(500 + 10 * k + seed).uniform(-0.06, 0.06, x.shape)
            x = f32(np.mod(x, box) if per else np.clip(x, 0.0, np.nextafter(box, 0)))
            spec = ReplicaSpec(n=n, box=box, model=bead_model(n_patchy, n), periodic=per, kT=1.0, dt=0.002,
                               seed=seed)
            Q = f32(random_rotations(n, 400 + 10 * k + seed))
            rc = po.System(spec).force_range * 1.05
            if threshold_margin(spec, x, Q, rc) > 1e-6:
                break
        F, T = ref_forces_bonded(spec, x, Q, rc, bonds, 100.0, 1.0)
        Fb = ref_bond_forces(spec, x, bonds, 100.0, 1.0)
        np.savez_compressed(HERE / f"bonded_{k}.npz", x=x, Q=Q, rc=rc, bonds=bonds, bond_k=100.0, bond_r0=1.0, F=F,
                            T=T, F_bond=Fb, **spec_record(spec))
        print(f"bonded_{k}: n={n} patchy={n_patchy} bonds={len(bonds)} periodic={per} |F|max={np.abs(F).max():.3g} "
              f"|F_bond|max={np.abs(Fb).max():.3g} torqued={(np.abs(T).sum(1) > 0).sum()}")


# awkward inputs for importcsv: short rows, empty cells, a trailing ',', no final newline.  (An empty
# line is not among them: importcsv reads past the row there -- a[i].size() - 1 wraps around -- and
# crashes; mtg_csv_read gives such a row zeros.)
CSV_CASES = ["1,2,3\n4,5\n6\n", "1.5,,-2\n3e2,4,\n", "7,8,9", "-0,1e-300,nan,inf\n5\n"]


def frame_cases():
    """G. frame files: the reference's writer (matrix operator<<=) and reader (importcsv)."""
    import tempfile
    rng = np.random.default_rng(11)
    a = rng.normal(size=(40, 9)) * 10.0 ** rng.integers(-9, 9, (40, 1))
    a = np.ascontiguousarray(np.concatenate([a, [[0.0, -0.0, 1e-300, 1e300, 123456789.0, 1 / 3, -2.5, 7.0, 1e-5]]]))
    tmp = Path(tempfile.mkdtemp())
    po.ref().ref_write_csv(str(tmp / "w.csv").encode(), D(a), a.shape[0], a.shape[1])
    written = (tmp / "w.csv").read_bytes()
    parsed = []
    for k, text in enumerate(CSV_CASES):
        (tmp / f"r{k}.csv").write_text(text)
        out = np.empty(256)
        cols = po.C.c_int(0)
        nr = po.ref().ref_import_csv(str(tmp / f"r{k}.csv").encode(), D(out), 256, po.C.byref(cols))
        parsed.append(out[: nr * cols.value].reshape(nr, cols.value).copy())
    np.savez_compressed(HERE / "frames.npz", data=a, written=np.frombuffer(written, dtype=np.uint8),
                        **{f"csv_{k}": np.frombuffer(t.encode(), dtype=np.uint8) for k, t in enumerate(CSV_CASES)},
                        **{f"parsed_{k}": p for k, p in enumerate(parsed)})
    print(f"frames.npz: writer {len(written)} bytes, {len(CSV_CASES)} importcsv cases "
          f"shapes {[p.shape for p in parsed]}")


def analysis_cases():
    """H. analysis: calcg1 histograms and distance_graph component labels from the reference."""
    cases = [(2000, 0.30, True, 4.0, 0.05, 1.25), (900, 0.20, False, 3.0, 0.02, 1.1), (400, 0.05, True, 5.0, 0.1, 1.6)]
    for k, (n, phi, per, rmax, dr, cut) in enumerate(cases):
        spec, x, _ = make_system("tetra", n, phi, 700 + k, per)
        h = np.zeros(100000, dtype=np.int64)
        m = po.ref().ref_calcg1(n, spec.box, int(per), D(x), rmax, dr, h.ctypes.data_as(po.C.POINTER(po.C.c_long)),
                                len(h))
        labels = np.empty(n, dtype=np.intc)
        po.ref().ref_distance_graph(n, spec.box, int(per), D(x), cut, labels.ctypes.data_as(po._I))
        np.savez_compressed(HERE / f"analysis_{k}.npz", x=x, rmax=rmax, dr=dr, hist=h[:m].copy(), cut=cut,
                            labels=labels, **spec_record(spec))
        print(f"analysis_{k}: n={n} periodic={per} bins={m} pairs<rmax={h[:m].sum()} "
              f"components={len(np.unique(labels))} largest={np.bincount(labels).max()}")


# binding models of the single-bond fixtures: (reference kind, args); the Ternary setups take six binding
# strengths then nine asymmetries (BindingModelTernary.cpp:29-140)
TERNARY_SETUP = [0.6, 0.5, 0.4, 0.55, 0.45, 0.35] + [0.1, -0.2, 0.3, 0.0, 0.15, -0.1, 0.2, -0.3, 0.05]
SINGLEBOND_CASES = [
    # (n, phi, cos thetam, periodic, seed, bm_kind, args[, model]): tetrahedral unless a model is named
    (400, 0.15, 0.90, True, 11, 0, [1.0, 0.1]),
    (300, 0.30, 0.70, True, 12, 0, [0.7, 0.5]),
    (300, 0.30, 0.70, True, 13, 1, [600]),
    (300, 0.30, 0.70, True, 14, 2, [400, 900] + TERNARY_SETUP),
    (300, 0.30, 0.70, True, 15, 3, [300, 800, 3] + TERNARY_SETUP),
    (300, 0.30, 0.75, False, 16, 0, [1.0, 0.2]),
    (300, 0.30, 0.70, True, 17, 2, [300, 700] + TERNARY_SETUP, "three_types"),
    (300, 0.30, 0.75, True, 18, 1, [500], "tubulin"),
]


def three_type_model(n: int, cosm: float) -> PatchModelSpec:
    """GeneralPatch with three types, as the production drivers use: 4 tetrahedral patches (half the
    particles), 2 polar patches (a third), crowders without patches; wider cones between unlike types."""
    from mtcode_gb300.system import TETRA
    n0, n1 = n // 2, n // 2 + n // 3
    orient = np.vstack([TETRA, [[0, 0, 1.0], [0, 0, -1.0]]])
    params = []
    for (a, b), (att, dis, c) in {(0, 0): (8.0, 1.2, cosm), (0, 1): (6.0, 1.15, cosm - 0.05),
                                  (1, 1): (7.0, 1.1, cosm + 0.05)}.items():
        for _ in range([4, 2][a] * [4, 2][b]):
            params.append([att, dis, math.acos(c)])
    return PatchModelSpec([4, 2, 0], [n0, n1, n], orient, np.array(params))


def singlebond_cases():
    """I. single-bond force pass: the reference's calculate_patch_list + onlyone_nonlets (srand(seed) first)
    over three rounds from an unbound start: round 1 re-decides the round-0 bonds in place, round 2 after
    new orientations (bonds break)."""
    import hashlib
    for k, case in enumerate(SINGLEBOND_CASES):
        n, phi, cosm, per, seed, kind, args = case[:7]
        model_name = case[7] if len(case) > 7 else "tetra"
        box = box_for(n, phi)
        if model_name == "three_types":
            model = three_type_model(n, cosm)
        elif model_name == "tubulin":
            model = tubulin_model(n, cos_max=cosm)
        else:
            model = PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(cosm))
        spec = ReplicaSpec(n=n, box=box, model=model, periodic=per, seed=seed)
        x = f32(random_positions(n, box, per, 0.9, 3000 + seed))
        Qs = [f32(random_rotations(n, 4000 + seed))] * 2 + [f32(random_rotations(n, 5000 + seed))]
        npatch = po.System(spec).total_patches()
        bt = np.zeros(npatch, dtype=np.intc)
        ib = np.zeros(npatch, dtype=np.uint8)
        rec = dict(x=x, Q=np.stack(Qs), bm_kind=kind, args=np.asarray(args, float), srand=seed)
        outs = {key: [] for key in ("bt_in", "ib_in", "bt", "ib", "F", "T", "plist_sha", "plist_n")}
        for rnd in range(3):
            r = po.ref_singlebond(spec, x, Qs[rnd], 2.5, kind, args, bt, ib, seed + rnd)
            pl = r["plist"][np.lexsort(r["plist"].T[::-1])]
            outs["bt_in"].append(bt.copy())
            outs["ib_in"].append(ib.copy())
            outs["bt"].append(r["boundto"])
            outs["ib"].append(r["isbound"])
            outs["F"].append(r["F"])
            outs["T"].append(r["T"])
            outs["plist_sha"].append(hashlib.sha256(np.ascontiguousarray(pl, dtype=np.int32).tobytes()).hexdigest())
            outs["plist_n"].append(len(pl))
            bt, ib = r["boundto"].copy(), r["isbound"].copy()
        rec.update({key: np.asarray(v) for key, v in outs.items()})
        rec.update(tables=r["tables"], max_ang=r["max_ang"], max_check=r["max_check"])
        np.savez_compressed(HERE / f"singlebond_{k}.npz", **rec, **spec_record(spec))
        print(f"singlebond_{k}: {model_name} n={n} phi={phi} cos={cosm} binding={kind} candidates={outs['plist_n']} "
              f"bound={[int(v.sum()) for v in outs['ib']]}")


def ref_run(spec, st, nsteps, rc, rebuild, noise=None, init=True, noise0=None):
    R = po.ref()
    kind, att, dis, th, nt, ppt, npt, orient, params = po.ref_model_args(spec.model)
    ncell = max(1, int(math.floor(spec.box / rc)))
    temps = np.empty((nsteps, 6))
    R.ref_run(spec.n, spec.box, int(spec.periodic), D(st["x"]), D(st["p"]), D(st["Lb"]), D(st["Q"]), D(st["Ft"]),
              D(st["Tt"]), spec.dt, spec.kT, spec.gamma, spec.gammar, spec.hs_eps, spec.hs_sigma, kind, att, dis, th,
              nt, ppt.ctypes.data_as(po._I), npt.ctypes.data_as(po._I), D(orient), D(params), ncell, rc, rebuild,
              nsteps, D(noise), int(init), D(noise0), D(temps))
    return temps


def threshold_margin(spec, x, Q, rc):
    """Smallest distance of any in-range pair quantity to a branch threshold of the force routine."""
    sysm = po.System(spec)
    pr = sysm.pairs(x, rc)
    if len(pr) == 0:
        return 1.0
    d = x[pr[:, 0]] - x[pr[:, 1]]
    if spec.periodic:
        d = np.where(d * d > (spec.box / 2) ** 2, d - np.sign(d) * spec.box, d)
    r2 = (d * d).sum(1)
    r = np.sqrt(r2)
    m = spec.model
    margins = [np.abs(r2 - spec.max_dist2).min(), np.abs(r - 1.12246 * spec.hs_sigma).min()]
    ppt = list(m.patches_per_type)
    cum = np.asarray(m.count_per_type)
    types = np.searchsorted(cum, np.arange(spec.n), side="right")
    ooff = np.concatenate([[0], np.cumsum(ppt)])
    params = np.asarray(m.params).reshape(-1, 3)
    orient = np.asarray(m.orient).reshape(-1, 3)
    Qm = Q.reshape(-1, 3, 3)
    u = d / r[:, None]
    ps = 0
    for a in range(len(ppt)):
        for b in range(a, len(ppt)):
            sel = (types[pr[:, 0]] == a) & (types[pr[:, 1]] == b) & (r2 < spec.max_dist2)
            for i in range(ppt[a]):
                for j in range(ppt[b]):
                    q = ps + i * ppt[b] + j
                    att, dis, th = params[q]
                    n1 = np.einsum("k,pkc->pc", orient[ooff[a] + i], Qm[pr[sel, 0]])
                    n2 = np.einsum("k,pkc->pc", orient[ooff[b] + j], Qm[pr[sel, 1]])
                    ci = -(n1 * u[sel]).sum(1)
                    cj = (n2 * u[sel]).sum(1)
                    cm = math.cos(th)
                    live = (ci > cm - 1e-3) & (cj > cm - 1e-3)
                    if live.any():
                        margins.append(np.abs(ci[live] - cm).min())
                        margins.append(np.abs(cj[live] - cm).min())
                        margins.append(np.abs(np.abs(ci[live] ** 2 - 1) - 1e-5).min())
                        margins.append(np.abs(np.abs(cj[live] ** 2 - 1) - 1e-5).min())
                        margins.append(np.abs(r[sel][live] - 1.4 * dis).min())
            ps += ppt[a] * ppt[b]
    return float(min(margins))


def make_system(kind, n, phi, seed, periodic=True, min_dist=0.9, kT=1.0):
    box = box_for(n, phi)
    if kind == "tetra":
        model = PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.90))
    elif kind == "tubulin":
        model = tubulin_model(n)
    elif kind == "crowded":
        model = crowded_model(n // 4, n)
    elif kind == "bivalent":
        model = PatchModelSpec.bivalent(n, 8.0, 1.2, math.acos(0.90))
    else:
        raise ValueError(kind)
    spec = ReplicaSpec(n=n, box=box, model=model, periodic=periodic, kT=kT, seed=seed)
    x = f32(random_positions(n, box, periodic, min_dist, 1000 + seed))
    Q = f32(random_rotations(n, 2000 + seed))
    return spec, x, Q


def spec_record(spec):
    m = spec.model
    return dict(n=spec.n, box=spec.box, periodic=int(spec.periodic), dt=spec.dt, kT=spec.kT, gamma=spec.gamma,
                gammar=spec.gammar, mass=spec.mass, inertia=spec.inertia, hs_eps=spec.hs_eps, hs_sigma=spec.hs_sigma,
                max_dist2=spec.max_dist2, seed=spec.seed, patches_per_type=np.asarray(m.patches_per_type),
                count_per_type=np.asarray(m.count_per_type), orient=np.asarray(m.orient, float),
                params=np.asarray(m.params, float))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None,
                    help="reference checkout (default: MTCODE_REFERENCE, else ../reference beside this repository)")
    ap.add_argument("--only", choices=["bonded", "frames", "analysis", "singlebond"],
                    help="regenerate one group of fixtures only")
    args = ap.parse_args()
    po.build_oracle()
    po.build_ref(args.reference)
    assert po.ref() is not None, "reference shim not built"
    if args.only == "bonded":
        bonded_cases()
        return
    if args.only == "frames":
        frame_cases()
        return
    if args.only == "analysis":
        analysis_cases()
        return
    if args.only == "singlebond":
        singlebond_cases()
        return

    # ---- A. pair sets (MD::calculatepairs and calculatepairs_parallel)
    pair_cases = [("tetra", 1000, 0.10, 1, True, 1.68), ("tetra", 1000, 0.30, 2, True, 1.5),
                  ("tetra", 600, 0.10, 3, False, 1.68), ("tetra", 800, 0.10, 4, True, 3.5),
                  ("tetra", 10, 0.10, 5, True, 1.68), ("tetra", 3, 0.05, 6, True, 1.2),
                  ("tetra", 40, 0.15, 7, False, 1.68)]
    for k, (kind, n, phi, seed, per, rc) in enumerate(pair_cases):
        spec, x, Q = make_system(kind, n, phi, seed, per)
        ncell = max(1, int(math.floor(spec.box / rc)))
        p1 = ref_pairs(spec, x, ncell, rc)
        p2 = ref_pairs(spec, x, ncell, rc, parallel=True)
        assert np.array_equal(p1, p2)
        np.savez_compressed(HERE / f"pairs_{k}.npz", x=x, rc=rc, ncell=ncell, pairs=p1, **spec_record(spec))
        print(f"pairs_{k}: n={n} L={spec.box:.3f} ncell={ncell} periodic={per} pairs={len(p1)}")

    # ---- B. forces and torques (calculateforces(HS) + calculate_forces_and_torques3D(ComboPatch))
    force_cases = [("tetra", 800, 0.30), ("tubulin", 800, 0.30), ("crowded", 800, 0.30), ("bivalent", 600, 0.30),
                   ("tetra", 200, 0.10)]
    for k, (kind, n, phi) in enumerate(force_cases):
        for seed in range(50):
            spec, x, Q = make_system(kind, n, phi, 10 * k + seed, True, min_dist=0.95)
            rc = po.System(spec).force_range * 1.05
            if threshold_margin(spec, x, Q, rc) > 1e-6:
                break
        F, T = ref_forces(spec, x, Q, rc)
        np.savez_compressed(HERE / f"forces_{k}.npz", x=x, Q=Q, rc=rc, F=F, T=T, **spec_record(spec))
        print(f"forces_{k}: {kind} n={n} |F|max={np.abs(F).max():.3g} |T|max={np.abs(T).max():.3g} "
              f"patch-torqued particles={(np.abs(T).sum(1) > 0).sum()}")

    # ---- C. 100-step trajectories: noise off (kT = 0) and shared pre-generated noise
    traj_cases = [("tetra", 256, 0.30, 0.0, "off"), ("tetra", 256, 0.30, 1.0, "shared"),
                  ("tubulin", 256, 0.30, 1.0, "shared"), ("crowded", 256, 0.30, 1.0, "shared")]
    for k, (kind, n, phi, kT, mode) in enumerate(traj_cases):
        spec, x, Q = make_system(kind, n, phi, 100 + k, True, min_dist=0.95, kT=kT)
        st0 = dict(x=x.copy(), p=np.zeros((n, 3)), Lb=np.zeros((n, 3)), Q=Q.copy(), Ft=np.zeros((n, 3)),
                   Tt=np.zeros((n, 3)))
        nsteps = 100
        noise = po.philox_noise(n * (nsteps + 1), 77 + k, 0, 0).reshape(nsteps + 1, n, 6) if mode == "shared" else None
        st = {kk: v.copy() for kk, v in st0.items()}
        rc = 1.68
        temps = ref_run(spec, st, nsteps, rc, 1, None if noise is None else np.ascontiguousarray(noise[1:]), True,
                        None if noise is None else np.ascontiguousarray(noise[0]))
        np.savez_compressed(HERE / f"traj_{k}.npz", x0=st0["x"], Q0=st0["Q"], nsteps=nsteps, noise_seed=77 + k,
                            noise_mode=mode, rc=rc, temps=temps, **{"final_" + kk: v for kk, v in st.items()},
                            **spec_record(spec))
        print(f"traj_{k}: {kind} kT={kT} noise={mode} <p^2/2>={temps[-1, :3].mean():.4f}")

    # ---- D. two-particle torque cases (kT = 0), after Code/BugReports/TorqueBug.md
    rng = np.random.default_rng(5)
    cases = []
    for k in range(6):
        spec = ReplicaSpec(n=2, box=10.0, model=PatchModelSpec.tetrahedral(2, 8.0, 1.2, math.acos(0.90)), kT=0.0)
        x = np.array([[5.0, 5.0, 5.0], [5.0 + 1.05 + 0.05 * k, 5.0, 5.0]])
        # rotate each body so that one patch points (almost) at the other particle
        Qs = []
        for a, target in ((0, np.array([1.0, 0, 0])), (1, np.array([-1.0, 0, 0]))):
            v = target + 0.2 * rng.normal(size=3)
            v /= np.linalg.norm(v)
            nb = po.System(spec).spec.model.orient[k % 4]
            # lab patch = Q^T nb; pick Q = R(nb -> v)^T so that Q^T nb = v
            ax = np.cross(nb, v)
            s, c = np.linalg.norm(ax), float(nb @ v)
            K = np.array([[0, -ax[2], ax[1]], [ax[2], 0, -ax[0]], [-ax[1], ax[0], 0]]) / (s if s > 0 else 1)
            Rm = np.eye(3) + s * K + (1 - c) * K @ K
            Qs.append(Rm.T.reshape(9))
        Q = f32(np.array(Qs))
        x = f32(x)
        st = dict(x=x.copy(), p=np.zeros((2, 3)), Lb=np.zeros((2, 3)), Q=Q.copy(), Ft=np.zeros((2, 3)),
                  Tt=np.zeros((2, 3)))
        x0, Q0 = x.copy(), Q.copy()
        ref_run(spec, st, 200, 3.0, 1)
        np.savez_compressed(HERE / f"torque_{k}.npz", x0=x0, Q0=Q0, nsteps=200, rc=3.0,
                            **{"final_" + kk: v for kk, v in st.items()}, **spec_record(spec))
        cases.append(np.abs(st["Lb"]).max())
    print("torque cases: max |L| after 200 steps", np.round(cases, 4))

    # ---- E. free-rotor rotation matrices (genfullmat)
    Ls = rng.normal(size=(64, 3)) * np.array([[0.1], [1.0], [10.0], [50.0]]).repeat(16, 0)
    Rs = np.empty((64, 9))
    for i, L in enumerate(Ls):
        L = np.ascontiguousarray(L)
        po.ref().ref_rotation_matrix(0.005, D(L), D(Rs[i]))
    np.savez_compressed(HERE / "rotation.npz", L=Ls, R=Rs, dt=0.005, inertia=0.1)
    print("rotation.npz written")

    bonded_cases()
    frame_cases()
    analysis_cases()
    singlebond_cases()


if __name__ == "__main__":
    main()
