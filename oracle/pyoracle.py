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


def reference_root() -> Path:
    """Where the reference checkout (the directory that holds Code/) is looked for: the directory named by
    the MTCODE_REFERENCE environment variable, else a directory ``reference`` beside this repository."""
    env = os.environ.get("MTCODE_REFERENCE")
    return Path(env) if env else HERE.parent.parent / "reference"


def build_ref(reference_root_dir: str | Path | None = None) -> Path | None:
    """Compile the reference's own routines through ref_driver.cpp (only where the sources exist)."""
    root = Path(reference_root_dir) if reference_root_dir is not None else reference_root()
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


class OrcBinding(C.Structure):
    """orc_binding: species rule + doublet rows (11, 12, 13, 22, 23, 33) + triplet rows (111 ... 333)."""
    _fields_ = [("rule", C.c_int), ("div1", C.c_int), ("div2", C.c_int), ("np", C.c_int),
                ("drate", (C.c_double * 4) * 6), ("trate", (C.c_double * 16) * 10)]


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_U8 = C.POINTER(C.c_ubyte)


def binding(rule: int, drate, trate, div1: int = 0, div2: int = 0, np_: int = 1) -> OrcBinding:
    b = OrcBinding()
    b.rule, b.div1, b.div2, b.np = int(rule), int(div1), int(div2), int(np_)
    d = np.asarray(drate, float).reshape(6, 4)
    t = np.asarray(trate, float).reshape(10, 16)
    for r in range(6):
        for k in range(4):
            b.drate[r][k] = float(d[r, k])
    for r in range(10):
        for k in range(16):
            b.trate[r][k] = float(t[r, k])
    return b


def binding_single(on: float, off: float) -> OrcBinding:
    """BindingModelSingle(on, off) (Bindings/BindingModelSingle.cpp): doublet rates (off, on) whatever the
    state before; triplet rows per state (bound 12, 23, 13, none)."""
    d = np.zeros((6, 4))
    d[0] = [off, on, off, on]
    t = np.zeros((10, 16))
    x = (off / 3.) + 0.001
    t[0] = [on, x, x, x, x, on, x, x, x, x, on, x, on / 3., on / 3., on / 3., off]
    return binding(0, d, t)


def binding_binary(div: int, raw_tables) -> OrcBinding:
    """BindingModelBinary(div) from its rate vectors (doubr11/12/22, tripr111/112/122/222 in the rows of the
    table form); its 122 and 222 triplets take the rate to none-bound from tripr111
    (BindingModelBinary.cpp triplet)."""
    raw = np.asarray(raw_tables, float)
    d = raw[:24].reshape(6, 4).copy()
    t = raw[24:].reshape(10, 16).copy()
    for row in (3, 6):
        for st in range(4):
            t[row, 4 * st + 3] = t[0, 4 * st + 3]
    return binding(1, d, t, div1=div)


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
        L.orc_max_check.restype = C.c_double
        L.orc_max_check.argtypes = [C.POINTER(OrcModel)]
        L.orc_total_patches.restype = C.c_int
        L.orc_total_patches.argtypes = [C.POINTER(OrcModel), C.c_int]
        L.orc_patch_list.restype = C.c_long
        L.orc_patch_list.argtypes = [P, _D, _D, _I, C.c_long, C.c_double, _I, C.c_long]
        L.orc_bind_uniform.restype = C.c_double
        L.orc_bind_uniform.argtypes = [C.c_uint64, C.c_uint32, C.c_uint64, C.c_uint32, C.c_uint32]
        L.orc_bind_update.restype = C.c_int
        L.orc_bind_update.argtypes = [P, _D, _D, _I, C.c_long, C.POINTER(OrcBinding), C.c_int, C.c_uint64,
                                      C.c_uint32, C.c_uint64, _I, C.POINTER(C.c_ubyte), _D, _D]
        L.orc_setup_priority.restype = C.c_uint32
        L.orc_setup_priority.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.c_uint32]
        L.orc_setup_edges.restype = C.c_long
        L.orc_setup_edges.argtypes = [P, _D, _D, _I, C.c_long, C.POINTER(OrcBinding), _I, C.POINTER(C.c_ubyte), _I,
                                      _D]
        L.orc_setup_random_binding.restype = C.c_int
        L.orc_setup_random_binding.argtypes = [P, _D, _D, _I, C.c_long, C.POINTER(OrcBinding), C.c_uint64,
                                               C.c_uint32, _I, C.POINTER(C.c_ubyte)]
        L.orc_run_singlebond.restype = C.c_int
        L.orc_run_singlebond.argtypes = [P, _D, _D, _D, _D, _D, _D, _I, C.POINTER(C.c_ubyte), C.POINTER(OrcBinding),
                                         C.c_double, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int,
                                         C.c_int, C.c_uint64, C.c_int, _D, C.c_uint64, C.c_uint32, C.c_uint64]
        L.orc_langevin_forces.argtypes = [P, _D, _D, _D, _D, _D, _D]
        L.orc_halfkick.argtypes = [C.c_int, C.c_double, _D, _D, _D, _D]
        L.orc_drift.argtypes = [P, _D, _D]
        L.orc_rotate.argtypes = [P, _D, _D]
        L.orc_random_positions.restype = C.c_int
        L.orc_random_positions.argtypes = [C.c_int, C.c_double, C.c_int, C.c_double, C.c_uint64, _D]
        L.orc_random_rotations.argtypes = [C.c_int, C.c_uint64, _D]
        L.orc_random_chains.restype = C.c_int
        L.orc_random_chains.argtypes = [C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double, C.c_uint64, _D]
        _orc = L
    return _orc


class Generators:
    """The seeded synthetic inputs (positions, rotations, chains) computed by the oracle library, with the
    signatures of mtcode_gb300.system's generators: the CPU baselines build their workloads from these, so
    that they load nothing from the product library.  Outputs are identical to the product's generators."""

    @staticmethod
    def random_positions(n: int, box: float, periodic: bool = True, min_dist: float = 0.9, seed: int = 0) -> np.ndarray:
        x = np.empty((n, 3))
        if orc().orc_random_positions(int(n), float(box), int(bool(periodic)), float(min_dist),
                                      int(seed) & 0xFFFFFFFFFFFFFFFF, _d(x)) != 0:
            raise ValueError(f"could not place {n} particles at min_dist {min_dist} in a box of {box}")
        return x

    @staticmethod
    def random_rotations(n: int, seed: int = 0) -> np.ndarray:
        Q = np.empty((n, 9))
        orc().orc_random_rotations(int(n), int(seed) & 0xFFFFFFFFFFFFFFFF, _d(Q))
        return Q

    @staticmethod
    def random_chains(n_chains: int, beads: int, box: float, periodic: bool = True, step: float = 1.0,
                      min_dist: float = 0.9, seed: int = 0) -> np.ndarray:
        x = np.empty((n_chains * beads, 3))
        if orc().orc_random_chains(int(n_chains), int(beads), float(box), int(bool(periodic)), float(step),
                                   float(min_dist), int(seed) & 0xFFFFFFFFFFFFFFFF, _d(x)) != 0:
            raise ValueError(f"could not place {n_chains} chains of {beads} beads in a box of {box}")
        return x


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


    # ---- the loop body's phases one at a time (arrays modified in place)
    def patch_forces(self, x, Q, F, T) -> None:
        """calculate_forces_and_torques3D: adds the patch forces and lab torques of every pair in range."""
        pr = self.pairs(x, self.force_range * 1.05)
        orc().orc_patch_forces(C.byref(self.params), _d(np.ascontiguousarray(x, float)),
                               _d(np.ascontiguousarray(Q, float)), pr.ctypes.data_as(_I), len(pr), _d(F), _d(T))

    def langevin_forces(self, p, Lb, Q, noise, F, T) -> None:
        """create_forces_and_torques_sphere: F (lab), T (lab) -> F~ (lab), T~ (body), in place."""
        orc().orc_langevin_forces(C.byref(self.params), _d(p), _d(Lb), _d(Q), _d(noise), _d(F), _d(T))

    def halfkick(self, p, Lb, F, T) -> None:
        orc().orc_halfkick(int(self.spec.n), float(self.spec.dt), _d(p), _d(Lb), _d(F), _d(T))

    def drift(self, x, p) -> None:
        orc().orc_drift(C.byref(self.params), _d(x), _d(p))

    def rotate(self, Lb, Q) -> None:
        orc().orc_rotate(C.byref(self.params), _d(Lb), _d(Q))

    # ---- single-bond mode
    def central_forces(self, x) -> np.ndarray:
        """MD::calculateforces with the HSPotential (plus any fixed bonds): the central forces alone."""
        x = np.ascontiguousarray(x, float)
        rc = 1.12246 * float(self.spec.hs_sigma) * 1.01
        pr = self.pairs(x, rc)
        F = np.empty((self.spec.n, 3))
        orc().orc_central_forces(C.byref(self.params), _d(x), pr.ctypes.data_as(_I), len(pr), _d(F))
        return F

    def max_check(self) -> float:
        return orc().orc_max_check(C.byref(self.model))

    def total_patches(self) -> int:
        return orc().orc_total_patches(C.byref(self.model), self.spec.n)

    def default_max_ang(self) -> float:
        """ComboPatch::max_ang of the GeneralPatch form: min(0.6, cos(thetam)) over the potentials."""
        th = np.asarray(self.spec.model.params, float).reshape(-1, 3)[:, 2]
        return float(min([0.6] + [math.cos(t) for t in th]))

    def patch_list(self, x, Q, pairs, max_ang: float) -> np.ndarray:
        """calculate_patch_list: (n, 5) rows (p1, p2, potn, wp1, wp2)."""
        x = np.ascontiguousarray(x, float)
        Q = np.ascontiguousarray(Q, float)
        pr = np.ascontiguousarray(pairs, dtype=np.intc).reshape(-1, 2)
        n = orc().orc_patch_list(C.byref(self.params), _d(x), _d(Q), pr.ctypes.data_as(_I), len(pr), float(max_ang),
                                 None, 0)
        out = np.empty((max(n, 1), 5), dtype=np.intc)
        orc().orc_patch_list(C.byref(self.params), _d(x), _d(Q), pr.ctypes.data_as(_I), len(pr), float(max_ang),
                             out.ctypes.data_as(_I), n)
        return out[:n].copy()

    def bind_update(self, x, Q, plist, bind: OrcBinding, boundto, isbound, rng: int = 0, seed: int = 0,
                    replica: int = 0, draw: int = 0):
        """onlyone_nonlets on a candidate list; boundto / isbound (int32 / uint8) are updated in place.
        Returns (status, F, T) of the bound pairs alone."""
        pl = np.ascontiguousarray(plist, dtype=np.intc).reshape(-1, 5)
        assert boundto.dtype == np.intc and isbound.dtype == np.uint8
        F = np.zeros((self.spec.n, 3))
        T = np.zeros((self.spec.n, 3))
        st = orc().orc_bind_update(C.byref(self.params), _d(np.ascontiguousarray(x, float)),
                                   _d(np.ascontiguousarray(Q, float)), pl.ctypes.data_as(_I), len(pl), C.byref(bind),
                                   int(rng), int(seed) & 0xFFFFFFFFFFFFFFFF, int(replica), int(draw),
                                   boundto.ctypes.data_as(_I), isbound.ctypes.data_as(_U8), _d(F), _d(T))
        return st, F, T

    def setup_random_binding(self, x, Q, plist, bind: OrcBinding, boundto, isbound, seed: int = 0,
                             replica: int = 0) -> int:
        """setup_random_binding on a candidate list in the library's seeded order; boundto / isbound (int32 /
        uint8) are updated in place."""
        pl = np.ascontiguousarray(plist, dtype=np.intc).reshape(-1, 5)
        assert boundto.dtype == np.intc and isbound.dtype == np.uint8
        return orc().orc_setup_random_binding(
            C.byref(self.params), _d(np.ascontiguousarray(x, float)), _d(np.ascontiguousarray(Q, float)),
            pl.ctypes.data_as(_I), len(pl), C.byref(bind), int(seed) & 0xFFFFFFFFFFFFFFFF, int(replica),
            boundto.ctypes.data_as(_I), isbound.ctypes.data_as(_U8))

    def setup_edges(self, x, Q, plist, bind: OrcBinding, boundto, isbound):
        """setup_random_binding's edges: (m, 2) patch pairs (wp1, wp2) and their scores (m,)."""
        pl = np.ascontiguousarray(plist, dtype=np.intc).reshape(-1, 5)
        bt = np.ascontiguousarray(boundto, dtype=np.intc)
        ib = np.ascontiguousarray(isbound, dtype=np.uint8)
        ab = np.empty((max(len(pl), 1), 2), dtype=np.intc)
        scr = np.empty(max(len(pl), 1))
        m = orc().orc_setup_edges(C.byref(self.params), _d(np.ascontiguousarray(x, float)),
                                  _d(np.ascontiguousarray(Q, float)), pl.ctypes.data_as(_I), len(pl), C.byref(bind),
                                  bt.ctypes.data_as(_I), ib.ctypes.data_as(_U8), ab.ctypes.data_as(_I), _d(scr))
        return ab[:m].copy(), scr[:m].copy()

    def run_singlebond(self, state: dict, bind: OrcBinding, nsteps: int, max_ang: float, i0: int = 0,
                       pair_cut: float = 2.5, pair_every: int = 20, patch_every: int = 10, init: bool = False,
                       init_draw: int = 0, noise_mode: int = 0, noise=None, seed: int = 0, replica: int = 0,
                       draw0: int = 0) -> int:
        """The run_singlebond loop on state (x, p, Lb, Q, Ft, Tt, boundto, isbound; modified in place)."""
        ncell = max(1, int(math.floor(self.spec.box / pair_cut)))
        return orc().orc_run_singlebond(
            C.byref(self.params), _d(state["x"]), _d(state["p"]), _d(state["Lb"]), _d(state["Q"]), _d(state["Ft"]),
            _d(state["Tt"]), state["boundto"].ctypes.data_as(_I), state["isbound"].ctypes.data_as(_U8),
            C.byref(bind), float(max_ang), int(nsteps), int(i0), ncell, float(pair_cut), int(pair_every),
            int(patch_every), int(bool(init)), int(init_draw), int(noise_mode),
            _d(None if noise is None else np.ascontiguousarray(noise, float)), int(seed) & 0xFFFFFFFFFFFFFFFF,
            int(replica), int(draw0))


def bind_uniform(seed: int, replica: int, draw: int, root: int, it: int) -> float:
    return orc().orc_bind_uniform(int(seed) & 0xFFFFFFFFFFFFFFFF, int(replica), int(draw), int(root), int(it))


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
        L.ref_singlebond.restype = C.c_long
        L.ref_singlebond.argtypes = [C.c_int, C.c_double, C.c_int, _D, _D, C.c_int, C.c_double, C.c_int, C.c_double,
                                     C.c_double, C.c_double, C.c_int, _I, _I, _D, _D, C.c_int, _D, _I, _U8, C.c_uint,
                                     _D, _D, _I, C.c_long, _D, _D]
        L.ref_setup_random_binding.restype = C.c_long
        L.ref_setup_random_binding.argtypes = [C.c_int, C.c_double, C.c_int, _D, _D, C.c_int, C.c_double, C.c_int,
                                               C.c_double, C.c_double, C.c_double, C.c_int, _I, _I, _D, _D, C.c_int,
                                               _D, _I, _U8, _I, C.c_long]
        _ref = L
    return _ref


def ref_model_args(model):
    """(kind, att, dis, thetam, n_types, ppt, npt, orient, params) for ref_forces/ref_run: GeneralPatch form."""
    ppt = np.asarray(model.patches_per_type, dtype=np.intc)
    npt = np.asarray(model.count_per_type, dtype=np.intc)
    orient = np.ascontiguousarray(np.asarray(model.orient, float).reshape(-1, 3))
    params = np.ascontiguousarray(np.asarray(model.params, float).reshape(-1, 3))
    return 2, 0.0, 0.0, 0.0, len(ppt), ppt, npt, orient, params


def ref_setup_random_binding(spec, x, Q, pair_cut: float, bm_kind: int, args, boundto, isbound):
    """The reference's calculate_patch_list + setup_random_binding (std::random_device order) on a copy of the bind
    state.  Returns (boundto, isbound)."""
    L = ref()
    n = int(spec.n)
    _, att, dis, th, nt, ppt, npt, orient, params = ref_model_args(spec.model)
    bt = np.ascontiguousarray(boundto, dtype=np.intc).copy()
    ib = np.ascontiguousarray(isbound, dtype=np.uint8).copy()
    cap = 16 * 16 * n + 64
    plist = np.empty((cap, 5), dtype=np.intc)
    a = np.ascontiguousarray(np.asarray(args, float).reshape(-1))
    ncell = max(1, int(math.floor(float(spec.box) / pair_cut)))
    npl = L.ref_setup_random_binding(n, float(spec.box), int(bool(spec.periodic)), _d(np.ascontiguousarray(x, float)),
                                     _d(np.ascontiguousarray(Q, float)), ncell, float(pair_cut), 2, att, dis, th, nt,
                                     ppt.ctypes.data_as(_I), npt.ctypes.data_as(_I), _d(orient), _d(params),
                                     int(bm_kind), _d(a), bt.ctypes.data_as(_I), ib.ctypes.data_as(_U8),
                                     plist.ctypes.data_as(_I), cap)
    assert npl <= cap, "candidate list larger than the buffer"
    return bt, ib


def ref_singlebond(spec, x, Q, pair_cut: float, bm_kind: int, args, boundto, isbound, seed: int):
    """The reference's calculate_patch_list + onlyone_nonlets (srand(seed) first) on a copy of the bind state.
    Returns dict(F, T, boundto, isbound, plist, tables, max_ang, max_check)."""
    L = ref()
    n = int(spec.n)
    _, att, dis, th, nt, ppt, npt, orient, params = ref_model_args(spec.model)
    bt = np.ascontiguousarray(boundto, dtype=np.intc).copy()
    ib = np.ascontiguousarray(isbound, dtype=np.uint8).copy()
    F = np.empty((n, 3))
    T = np.empty((n, 3))
    cap = 16 * 16 * n + 64   # at most 16 patch pairs for each of the <= 16 n pairs within 2.5 sigma
    plist = np.empty((cap, 5), dtype=np.intc)
    tables = np.empty(184)
    caps = np.empty(2)
    a = np.ascontiguousarray(np.asarray(args, float).reshape(-1))
    ncell = max(1, int(math.floor(float(spec.box) / pair_cut)))
    npl = L.ref_singlebond(n, float(spec.box), int(bool(spec.periodic)), _d(np.ascontiguousarray(x, float)),
                           _d(np.ascontiguousarray(Q, float)), ncell, float(pair_cut), 2, att, dis, th, nt,
                           ppt.ctypes.data_as(_I), npt.ctypes.data_as(_I), _d(orient), _d(params), int(bm_kind), _d(a),
                           bt.ctypes.data_as(_I), ib.ctypes.data_as(_U8), int(seed), _d(F), _d(T),
                           plist.ctypes.data_as(_I), cap, _d(tables), _d(caps))
    assert npl <= cap, "candidate list larger than the buffer"
    return dict(F=F, T=T, boundto=bt, isbound=ib, plist=plist[:npl].copy(), tables=tables,
                max_ang=float(caps[0]), max_check=float(caps[1]))
