"""ctypes bindings of the oracle (liboracle.so, the FP64 CPU restatement) and, where it has been built,
of the reference's own routines (_ref/libmtref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
reference arm -- never by the product package.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_SO = HERE / "liboracle.so"
REF_SO = HERE / "_ref" / "libmtref.so"

MAX_TYPES, MAX_ORIENT, MAX_POTS = 8, 64, 2048


def build_oracle(force: bool = False) -> Path:
    """gcc build of oracle.c (no FMA contraction, so x86-64 and aarch64 round alike)."""
    src = HERE / "oracle.c"
    if force or not ORACLE_SO.exists() or ORACLE_SO.stat().st_mtime < max(src.stat().st_mtime,
                                                                          (HERE / "oracle.h").stat().st_mtime):
        tmp = ORACLE_SO.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-fPIC", "-shared", str(src), "-lm", "-o",
                        str(tmp)], check=True)
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def build_ref(reference_root: str | Path = "/root/reference") -> Path | None:
    """Compile the reference's own routines through ref_driver.cpp (only where the sources exist)."""
    root = Path(reference_root)
    if not (root / "Code").is_dir():
        return None
    subprocess.run(["sh", str(HERE / "build_ref.sh"), str(root)], check=True)
    return REF_SO


class OrcModel(C.Structure):
    _fields_ = [("n_types", C.c_int), ("patches_per_type", C.c_int * MAX_TYPES),
                ("num_per_type", C.c_int * MAX_TYPES), ("orient", (C.c_double * 3) * MAX_ORIENT),
                ("n_pots", C.c_int), ("att", C.c_double * MAX_POTS), ("dis", C.c_double * MAX_POTS),
                ("thetam", C.c_double * MAX_POTS)]


class OrcParams(C.Structure):
    _fields_ = [("n", C.c_int), ("box", C.c_double), ("periodic", C.c_int), ("dt", C.c_double),
                ("kT", C.c_double), ("gamma", C.c_double), ("gammar", C.c_double), ("mass", C.c_double),
                ("inertia", C.c_double), ("hs_eps", C.c_double), ("hs_sigma", C.c_double),
                ("max_dist2", C.c_double), ("model", C.POINTER(OrcModel)), ("bonds", C.POINTER(C.c_int)),
                ("nbonds", C.c_long), ("bond_k", C.c_double), ("bond_r0", C.c_double)]


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)


def _d(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


_orc = None


def orc() -> C.CDLL:
    global _orc
    if _orc is None:
        build_oracle()
        L = C.CDLL(str(ORACLE_SO))
        P = C.POINTER(OrcParams)
        L.orc_pairs.restype = C.c_long
        L.orc_pairs.argtypes = [P, _D, C.c_int, C.c_double, _I, C.c_long]
        L.orc_forces.argtypes = [P, _D, _D, C.c_int, C.c_double, _D, _D]
        L.orc_init_forces.argtypes = [P, _D, _D, _D, _D, C.c_int, C.c_double, _D, _D, _D]
        L.orc_run.restype = C.c_int
        L.orc_run.argtypes = [P, _D, _D, _D, _D, _D, _D, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, _D,
                              C.c_uint64, C.c_uint32, C.c_uint64, C.c_int]
        L.orc_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.orc_philox_noise.argtypes = [C.c_int, C.c_uint64, C.c_uint32, C.c_uint64, _D]
        L.orc_temperature.argtypes = [P, _D, _D, _D]
        L.orc_rotation_matrix.argtypes = [C.c_double, C.c_double, _D, _D]
        L.orc_hs_forces.argtypes = [P, _D, _I, C.c_long, _D]
        L.orc_bond_forces.argtypes = [P, _D, _I, C.c_long, C.c_double, C.c_double, _D]
        L.orc_central_forces.argtypes = [P, _D, _I, C.c_long, _D]
        L.orc_gr.restype = C.c_int
        L.orc_gr.argtypes = [P, _D, C.c_double, C.c_double, C.POINTER(C.c_long), C.c_int]
        L.orc_clusters.argtypes = [P, _D, C.c_double, _I]
        L.orc_patch_forces.argtypes = [P, _D, _D, _I, C.c_long, _D, _D]
        L.orc_observables.argtypes = [P, _D, _D, _I, C.c_long, _D]
        L.orc_neighbor_cells.restype = C.c_int
        L.orc_neighbor_cells.argtypes = [C.c_int, C.c_int, _I]
        _orc = L
    return _orc


class System:
    """Parameters of one replica for the oracle, built from a ReplicaSpec-like object."""

    def __init__(self, spec):
        m = spec.model
        self.spec = spec
        self.model = OrcModel()
        self.model.n_types = len(m.patches_per_type)
        for k, (a, b) in enumerate(zip(m.patches_per_type, m.count_per_type)):
            self.model.patches_per_type[k] = int(a)
            self.model.num_per_type[k] = int(b)
        for i, v in enumerate(np.asarray(m.orient, float).reshape(-1, 3)):
            for c in range(3):
                self.model.orient[i][c] = float(v[c])
        params = np.asarray(m.params, float).reshape(-1, 3)
        self.model.n_pots = len(params)
        for q, (att, dis, th) in enumerate(params):
            self.model.att[q], self.model.dis[q], self.model.thetam[q] = float(att), float(dis), float(th)
        p = OrcParams()
        p.n, p.box, p.periodic = int(spec.n), float(spec.box), int(bool(spec.periodic))
        p.dt, p.kT, p.gamma, p.gammar = float(spec.dt), float(spec.kT), float(spec.gamma), float(spec.gammar)
        p.mass, p.inertia, p.hs_eps, p.hs_sigma = float(spec.mass), float(spec.inertia), float(spec.hs_eps), float(
            spec.hs_sigma)
        p.max_dist2 = float(spec.max_dist2)
        p.model = C.pointer(self.model)
        self.params = p
        self.set_bonds(None)

    def set_bonds(self, bonds, k: float = 0.0, r0: float = 0.0) -> None:
        """Fixed bond list (n_b x 2 local particle indices) with HarmonicPotential(k, r0)."""
        p = self.params
        if bonds is None or len(bonds) == 0:
            self._bonds = None
            p.bonds, p.nbonds, p.bond_k, p.bond_r0 = None, 0, 0.0, 0.0
            return
        self._bonds = np.ascontiguousarray(bonds, dtype=np.intc).reshape(-1, 2)
        p.bonds = self._bonds.ctypes.data_as(_I)
        p.nbonds, p.bond_k, p.bond_r0 = len(self._bonds), float(k), float(r0)

    def gr(self, x, rmax: float, dr: float) -> np.ndarray:
        """calcg1: counts of unordered pair distances in bins of dr below floor(rmax / dr) * dr."""
        nb = int(math.floor(rmax / dr))
        out = np.zeros(max(nb, 1), dtype=np.int64)
        orc().orc_gr(C.byref(self.params), _d(np.ascontiguousarray(x, float)), float(rmax), float(dr),
                     out.ctypes.data_as(C.POINTER(C.c_long)), len(out))
        return out[:nb]

    def clusters(self, x, cut: float) -> np.ndarray:
        """distance_graph: per particle the smallest index of its connected component (pairs closer than cut)."""
        out = np.empty(self.spec.n, dtype=np.intc)
        orc().orc_clusters(C.byref(self.params), _d(np.ascontiguousarray(x, float)), float(cut), out.ctypes.data_as(_I))
        return out

    def bond_forces(self, x, bonds, k: float, r0: float) -> np.ndarray:
        b = np.ascontiguousarray(bonds, dtype=np.intc).reshape(-1, 2)
        F = np.empty((self.spec.n, 3))
        orc().orc_bond_forces(C.byref(self.params), _d(np.ascontiguousarray(x, float)), b.ctypes.data_as(_I),
                              len(b), float(k), float(r0), _d(F))
        return F

    @property
    def force_range(self) -> float:
        m = self.spec.model
        dmax = max([1.4 * d for d in np.asarray(m.params)[:, 1]] or [0.0])
        has_patch = any(k > 0 for k in m.patches_per_type)
        patch = min(math.sqrt(self.spec.max_dist2), dmax) if has_patch else 0.0
        return max(1.12246 * self.spec.hs_sigma, patch)

    def ncell(self, rc: float) -> int:
        return max(1, int(math.floor(self.spec.box / rc)))

    def pairs(self, x: np.ndarray, rc: float, ncell: int | None = None) -> np.ndarray:
        x = np.ascontiguousarray(x, float)
        nc = self.ncell(rc) if ncell is None else ncell
        cap = 16 * len(x) + 64
        while True:
            out = np.empty((cap, 2), dtype=np.intc)
            n = orc().orc_pairs(C.byref(self.params), _d(x), nc, rc, out.ctypes.data_as(_I), cap)
            if n <= cap:
                return out[:n].copy()
            cap = n

    def forces(self, x, Q, rc: float | None = None):
        rc = rc or self.force_range * 1.05
        F = np.empty((self.spec.n, 3))
        T = np.empty((self.spec.n, 3))
        orc().orc_forces(C.byref(self.params), _d(np.ascontiguousarray(x, float)), _d(np.ascontiguousarray(Q, float)),
                         self.ncell(rc), rc, _d(F), _d(T))
        return F, T

    def init_forces(self, x, p, Lb, Q, noise=None, rc: float | None = None):
        rc = rc or self.force_range * 1.05
        Ft = np.empty((self.spec.n, 3))
        Tt = np.empty((self.spec.n, 3))
        orc().orc_init_forces(C.byref(self.params), _d(x), _d(p), _d(Lb), _d(Q), self.ncell(rc), rc,
                              _d(None if noise is None else np.ascontiguousarray(noise, float)), _d(Ft), _d(Tt))
        return Ft, Tt

    def run(self, state: dict, nsteps: int, noise_mode: int = 0, noise=None, seed: int = 0, replica: int = 0,
            draw0: int = 0, rc: float | None = None, rebuild: int = 1, check_skin: bool = True) -> int:
        """Advance state (dict of x, p, Lb, Q, Ft, Tt float64 arrays, modified in place)."""
        rc = rc or self.force_range + 0.15
        return orc().orc_run(C.byref(self.params), _d(state["x"]), _d(state["p"]), _d(state["Lb"]), _d(state["Q"]),
                             _d(state["Ft"]), _d(state["Tt"]), int(nsteps), self.ncell(rc), rc, int(rebuild),
                             int(noise_mode), _d(None if noise is None else np.ascontiguousarray(noise, float)),
                             int(seed) & 0xFFFFFFFFFFFFFFFF, int(replica), int(draw0), int(bool(check_skin)))

    def temperature(self, p, Lb) -> np.ndarray:
        out = np.empty(6)
        orc().orc_temperature(C.byref(self.params), _d(p), _d(Lb), _d(out))
        return out

    def observables(self, x, Q) -> np.ndarray:
        m = self.spec.model
        dmax = max([1.4 * d for d in np.asarray(m.params)[:, 1]] or [0.0])
        rc = max(self.force_range, dmax, 1.0) * 1.01
        pr = self.pairs(x, rc)
        out = np.empty(4)
        orc().orc_observables(C.byref(self.params), _d(np.ascontiguousarray(x, float)),
                              _d(np.ascontiguousarray(Q, float)), pr.ctypes.data_as(_I), len(pr), _d(out))
        return out


def philox(ctr, key) -> list:
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    orc().orc_philox4x32_10(c, k, o)
    return list(o)


def philox_noise(n: int, seed: int, replica: int, draw: int) -> np.ndarray:
    out = np.empty((n, 6))
    orc().orc_philox_noise(int(n), int(seed) & 0xFFFFFFFFFFFFFFFF, int(replica), int(draw), _d(out))
    return out


# ---------------------------------------------------------------- the reference itself (this container only)
_ref = None


def ref() -> C.CDLL | None:
    global _ref
    if _ref is None:
        if not REF_SO.exists():
            return None
        L = C.CDLL(str(REF_SO))
        L.ref_pairs.restype = C.c_long
        L.ref_pairs.argtypes = [C.c_int, C.c_double, C.c_int, _D, C.c_int, C.c_double, _I, C.c_long]
        L.ref_pairs_parallel.restype = C.c_long
        L.ref_pairs_parallel.argtypes = [C.c_int, C.c_double, C.c_int, _D, C.c_int, C.c_double, _I, C.c_long]
        L.ref_forces.argtypes = [C.c_int, C.c_double, C.c_int, _D, _D, C.c_int, C.c_double, C.c_double, C.c_double,
                                 C.c_int, C.c_double, C.c_double, C.c_double, C.c_int, _I, _I, _D, _D, _D, _D]
        L.ref_run.argtypes = [C.c_int, C.c_double, C.c_int, _D, _D, _D, _D, _D, _D, C.c_double, C.c_double,
                              C.c_double, C.c_double, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double,
                              C.c_double, C.c_int, _I, _I, _D, _D, C.c_int, C.c_double, C.c_int, C.c_int, _D,
                              C.c_int, _D, _D]
        L.ref_rotation_matrix.argtypes = [C.c_double, _D, _D]
        L.ref_bond_forces.argtypes = [C.c_int, C.c_double, C.c_int, _D, _I, C.c_long, C.c_double, C.c_double, _D]
        L.ref_calcg1.restype = C.c_long
        L.ref_calcg1.argtypes = [C.c_int, C.c_double, C.c_int, _D, C.c_double, C.c_double, C.POINTER(C.c_long),
                                 C.c_long]
        L.ref_distance_graph.argtypes = [C.c_int, C.c_double, C.c_int, _D, C.c_double, _I]
        L.ref_write_csv.argtypes = [C.c_char_p, _D, C.c_int, C.c_int]
        L.ref_import_csv.restype = C.c_long
        L.ref_import_csv.argtypes = [C.c_char_p, _D, C.c_long, C.POINTER(C.c_int)]
        L.ref_forces_bonded.argtypes = [C.c_int, C.c_double, C.c_int, _D, _D, C.c_int, C.c_double, C.c_double,
                                        C.c_double, C.c_int, _I, _I, _D, _D, _I, C.c_long, C.c_double, C.c_double,
                                        _D, _D]
        _ref = L
    return _ref


def ref_model_args(model):
    """(kind, att, dis, thetam, n_types, ppt, npt, orient, params) for ref_forces/ref_run: GeneralPatch form."""
    ppt = np.asarray(model.patches_per_type, dtype=np.intc)
    npt = np.asarray(model.count_per_type, dtype=np.intc)
    orient = np.ascontiguousarray(np.asarray(model.orient, float).reshape(-1, 3))
    params = np.ascontiguousarray(np.asarray(model.params, float).reshape(-1, 3))
    return 2, 0.0, 0.0, 0.0, len(ppt), ppt, npt, orient, params
