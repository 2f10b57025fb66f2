"""Host-side mirror of the reference's LangevinNVTR + ComboPatch interface over the C ABI.

``LangevinNVTRGPU`` keeps the reference's method names (``initialize``, ``getdat``, ``getmom``,
``getangmom``, ``getorientation``, ``calculatepairs_parallel``, ``calculate_forces_and_torques3D``,
``measured_temperature``) and adds the fused ``step(nsteps)`` that replaces the body of
``Condensate::run`` (Condensate/Condensate.cpp:335-378).  Arrays are row-major float64 exactly like the
reference's ``matrix<double>`` (x, p, Lb: n x 3; Q: n x 9; pairs: P x 2).  Every call goes to the CUDA
library; errors raise ``MtgError`` instead of the reference's stdin-blocking ``error()``.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import MtgError, dptr

TETRA = np.array([[math.sqrt(8 / 9), 0.0, -1 / 3],
                  [-math.sqrt(2 / 9), math.sqrt(2 / 3), -1 / 3],
                  [-math.sqrt(2 / 9), -math.sqrt(2 / 3), -1 / 3],
                  [0.0, 0.0, 1.0]])


@dataclass
class PatchModelSpec:
    """GeneralPatch-shaped model (GeneralPatch.cpp:7-121).  ``count_per_type`` is cumulative."""
    patches_per_type: list
    count_per_type: list
    orient: np.ndarray           # (sum patches) x 3 body-frame unit vectors
    params: np.ndarray           # n_pots x 3: (att, dis, thetam)

    @staticmethod
    def tetrahedral(n: int, att: float, dis: float, thetam: float) -> "PatchModelSpec":
        """TetrahedralPatch(att, dis, thetam) (TetrahedralPatch.cpp:4-44)."""
        return PatchModelSpec([4], [n], TETRA.copy(), np.tile([att, dis, thetam], (16, 1)).astype(float))

    @staticmethod
    def bivalent(n: int, att: float, dis: float, thetam: float) -> "PatchModelSpec":
        """BivalentPatch(att, dis, thetam) (BivalentPatch.cpp:4-34): patches at -x and +x."""
        return PatchModelSpec([2], [n], np.array([[-1.0, 0, 0], [1.0, 0, 0]]),
                              np.tile([att, dis, thetam], (4, 1)).astype(float))

    @property
    def n_pots(self) -> int:
        k = self.patches_per_type
        return sum(k[a] * k[b] for a in range(len(k)) for b in range(a, len(k)))

    def to_c(self) -> _lib.PatchModel:
        m = _lib.PatchModel()
        m.n_types = len(self.patches_per_type)
        for k, (npt, cnt) in enumerate(zip(self.patches_per_type, self.count_per_type)):
            m.patches_per_type[k] = int(npt)
            m.count_per_type[k] = int(cnt)
        for i, v in enumerate(np.asarray(self.orient, float).reshape(-1, 3)):
            for c in range(3):
                m.orient[i][c] = float(v[c])
        for q, v in enumerate(np.asarray(self.params, float).reshape(-1, 3)):
            for c in range(3):
                m.params[q][c] = float(v[c])
        return m


@dataclass
class ReplicaSpec:
    """One independent system: cube(box) + LangevinNVTR parameters + HSPotential + ComboPatch."""
    n: int
    box: float
    model: PatchModelSpec
    periodic: bool = True
    dt: float = 0.005
    kT: float = 1.0
    gamma: float = 1.0
    gammar: float = 1.0
    mass: float = 1.0
    inertia: float = 0.25 * 2.0 / 5.0
    hs_eps: float = 1.0
    hs_sigma: float = 1.0
    max_dist2: float = 2.4
    seed: int = 0

    def to_c(self) -> _lib.ReplicaDesc:
        d = _lib.ReplicaDesc()
        d.n, d.box, d.periodic = int(self.n), float(self.box), int(bool(self.periodic))
        d.dt, d.kT, d.gamma, d.gammar = float(self.dt), float(self.kT), float(self.gamma), float(self.gammar)
        d.mass, d.inertia = float(self.mass), float(self.inertia)
        d.hs_eps, d.hs_sigma, d.max_dist2 = float(self.hs_eps), float(self.hs_sigma), float(self.max_dist2)
        d.seed = int(self.seed) & 0xFFFFFFFFFFFFFFFF
        d.model = self.model.to_c()
        return d


def _inplace(a: np.ndarray) -> np.ndarray:
    if not (isinstance(a, np.ndarray) and a.dtype == np.float64 and a.flags.c_contiguous and a.flags.writeable):
        raise TypeError("an in-place argument must be a writeable C-contiguous float64 array")
    return a


def _check(h, status: int) -> None:
    if status != 0:
        msg = _lib.lib().mtg_last_error(h)
        raise MtgError(status, (msg or b"").decode())


class LangevinNVTRGPU:
    """All replicas of one GPU handle (one CUDA stream)."""

    def __init__(self, replicas: list, precision: str = "fp32", device: int = 0, track_displacement: bool = True,
                 force_kernel: str = "pairs", neighbor_skin: float = 0.0):
        """``neighbor_skin`` > 0 (sigma): cells and candidate lists at force range + skin, reused until a
        particle has moved more than half the skin (the same force set as a rebuild every step)."""
        L = _lib.lib()
        self.replicas = list(replicas)
        self._descs = (_lib.ReplicaDesc * len(self.replicas))(*[r.to_c() for r in self.replicas])
        cfg = _lib.Config()
        cfg.precision = _lib.MTG_FP64 if precision == "fp64" else _lib.MTG_FP32
        cfg.n_replicas = len(self.replicas)
        cfg.replicas = C.cast(self._descs, C.POINTER(_lib.ReplicaDesc))
        cfg.device = int(device)
        cfg.track_displacement = int(bool(track_displacement))
        cfg.force_kernel = {"pairs": 0, "per_particle": 1, "tiled": 2}[force_kernel]
        cfg.neighbor_skin = float(neighbor_skin)
        h = C.c_void_p()
        st = L.mtg_create(C.byref(cfg), C.byref(h))
        if st != 0:
            raise MtgError(st, (L.mtg_last_error(None) or b"").decode())
        self._h = h
        self.precision = precision
        self.n = int(L.mtg_num_particles(h))
        self.offsets = np.array([L.mtg_replica_offset(h, r) for r in range(len(self.replicas))] + [self.n])

    # ------------------------------------------------------------------ lifetime
    def close(self) -> None:
        if getattr(self, "_h", None):
            _lib.lib().mtg_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ------------------------------------------------------------------ state
    def initialize(self, x, p, Lb, Q, Ft=None, Tt=None) -> None:
        """LangevinNVTR::initialize(positions, momenta, orientations, angular_momenta) for all replicas."""
        arrs = [np.ascontiguousarray(a, dtype=np.float64) if a is not None else None for a in (x, p, Lb, Q, Ft, Tt)]
        for a, w in zip(arrs, (3, 3, 3, 9, 3, 3)):
            if a is not None and a.size != self.n * w:
                raise ValueError(f"state array of size {a.size}, expected {self.n * w}")
        self._hold = arrs  # host memory must outlive the (staged) copies
        _check(self._h, _lib.lib().mtg_set_state(self._h, *[dptr(a) for a in arrs]))

    def get_state(self, out: dict | None = None) -> dict:
        """The whole state (x, p, Lb, Q, F~, T~).  ``out``: caller arrays to fill (e.g. pinned host memory,
        which the download then reaches by DMA); new arrays otherwise."""
        shapes = (("x", 3), ("p", 3), ("Lb", 3), ("Q", 9), ("Ft", 3), ("Tt", 3))
        if out is None:
            out = {k: np.empty((self.n, w)) for k, w in shapes}
        for k, w in shapes:
            if out[k].size != self.n * w:
                raise ValueError(f"out[{k!r}] holds {out[k].size} values, expected {self.n * w}")
        _check(self._h, _lib.lib().mtg_get_state(self._h, *[dptr(out[k]) for k, _ in shapes]))
        return out

    def getdat(self) -> np.ndarray:
        x = np.empty((self.n, 3))
        _check(self._h, _lib.lib().mtg_get_state(self._h, dptr(x), None, None, None, None, None))
        return x

    def getmom(self) -> np.ndarray:
        p = np.empty((self.n, 3))
        _check(self._h, _lib.lib().mtg_get_state(self._h, None, dptr(p), None, None, None, None))
        return p

    def getangmom(self) -> np.ndarray:
        L = np.empty((self.n, 3))
        _check(self._h, _lib.lib().mtg_get_state(self._h, None, None, dptr(L), None, None, None))
        return L

    def getorientation(self) -> np.ndarray:
        Q = np.empty((self.n, 9))
        _check(self._h, _lib.lib().mtg_get_state(self._h, None, None, None, dptr(Q), None, None))
        return Q

    # ------------------------------------------------------------------ the hot path
    def init_forces(self, noise: np.ndarray | None = None) -> None:
        """Condensate.cpp:312-334: F~, T~ from forces + one noise draw (Philox, or ``noise`` n x 6)."""
        if noise is None:
            _check(self._h, _lib.lib().mtg_init_forces(self._h))
        else:
            noise = np.ascontiguousarray(noise, dtype=np.float64)
            if noise.size != self.n * 6:
                raise ValueError("noise must hold n x 6 values")
            _check(self._h, _lib.lib().mtg_init_forces_noise(self._h, dptr(noise)))

    def step_profile(self, nsteps: int) -> dict:
        """Per-kernel device milliseconds summed over ``nsteps`` instrumented steps."""
        out = np.zeros(_lib.MTG_PROFILE_KERNELS)
        _check(self._h, _lib.lib().mtg_step_profile(self._h, int(nsteps), dptr(out)))
        return dict(zip(_lib.PROFILE_KERNEL_NAMES, out.tolist()))

    def step(self, nsteps: int = 1, noise: np.ndarray | None = None) -> None:
        """nsteps of the Condensate::run loop body; ``noise`` (nsteps x n x 6) replaces Philox."""
        if noise is None:
            _check(self._h, _lib.lib().mtg_step(self._h, int(nsteps)))
        else:
            noise = np.ascontiguousarray(noise, dtype=np.float64)
            if noise.size != nsteps * self.n * 6:
                raise ValueError("noise must hold nsteps x n x 6 values")
            _check(self._h, _lib.lib().mtg_step_noise(self._h, int(nsteps), dptr(noise)))

    def set_bonds(self, bonds, k: float, r0: float) -> None:
        """Fixed bonds with HarmonicPotential(k, r0), added to every force pass (MD::calculateforces over
        the bond list, MD.cpp:1684-1764).  ``bonds``: n_b x 2 host-order (global) particle indices, both
        ends in one replica; an empty list removes them."""
        b = np.ascontiguousarray(np.asarray(bonds, dtype=np.int32).reshape(-1, 2))
        _check(self._h, _lib.lib().mtg_set_bonds(self._h, b.ctypes.data_as(_lib._I32) if len(b) else None, len(b),
                                                 float(k), float(r0)))

    # ------------------------------------------------------------------ single-bond-per-patch mode
    def set_single_bond(self, model: "_lib.BindingModel | None", max_ang: float | None = None, list_cut: float = 2.5,
                        patch_every: int = 10) -> None:
        """Condensate::run_singlebond's force pass (one bond per patch, binding model ``model``); None switches
        back to the full Kern-Frenkel force.  ``max_ang`` None: GeneralPatch's min(0.6, cos thetam)."""
        L = _lib.lib()
        if model is None:
            _check(self._h, L.mtg_set_single_bond(self._h, None))
            return
        sb = _lib.SingleBond()
        L.mtg_single_bond_defaults(C.byref(sb))
        sb.model = model
        sb.max_ang = float("nan") if max_ang is None else float(max_ang)
        sb.list_cut = float(list_cut)
        sb.patch_every = int(patch_every)
        _check(self._h, L.mtg_set_single_bond(self._h, C.byref(sb)))

    @property
    def num_patches(self) -> int:
        return int(_lib.lib().mtg_num_patches(self._h))

    def patch_offset(self, replica: int) -> int:
        return int(_lib.lib().mtg_patch_offset(self._h, int(replica)))

    def set_bind_state(self, boundto, isbound) -> None:
        """BinaryBindStore of every patch: boundto (replica-local partner patch), isbound (0 / 1)."""
        bt = np.ascontiguousarray(boundto, dtype=np.int32)
        ib = np.ascontiguousarray(isbound, dtype=np.uint8)
        if bt.size != self.num_patches or ib.size != self.num_patches:
            raise ValueError("boundto and isbound need one entry per patch")
        _check(self._h, _lib.lib().mtg_set_bind_state(self._h, bt.ctypes.data_as(_lib._I32),
                                                      ib.ctypes.data_as(_lib._U8)))

    def get_bind_state(self) -> tuple:
        n = max(self.num_patches, 1)
        bt = np.empty(n, dtype=np.int32)
        ib = np.empty(n, dtype=np.uint8)
        _check(self._h, _lib.lib().mtg_get_bind_state(self._h, bt.ctypes.data_as(_lib._I32),
                                                      ib.ctypes.data_as(_lib._U8)))
        return bt[: self.num_patches], ib[: self.num_patches]

    def bind_update(self):
        """One calculate_forces_and_torques3D_onlyone_nonlets pass at the current state (bonds decided,
        one draw index consumed): F (WCA core + bonds + bound pairs) and T (bound pairs, lab)."""
        F = np.empty((self.n, 3))
        T = np.empty((self.n, 3))
        _check(self._h, _lib.lib().mtg_bind_update(self._h, dptr(F), dptr(T)))
        return F, T

    def setup_random_binding(self, seed: int = 0) -> None:
        """LangevinNVTR::setup_random_binding at the current state: the candidate edges that can bind, taken in
        a seeded random order, each binding two unbound patches (mtg_setup_random_binding)."""
        _check(self._h, _lib.lib().mtg_setup_random_binding(self._h, int(seed) & 0xFFFFFFFFFFFFFFFF))

    def calculate_forces_and_torques3D(self, with_energy: bool = False):
        """MD::calculateforces(HSPotential) + LangevinNVTR::calculate_forces_and_torques3D: F, T (lab)."""
        F = np.empty((self.n, 3))
        T = np.empty((self.n, 3))
        E = np.empty(self.n) if with_energy else None
        _check(self._h, _lib.lib().mtg_forces(self._h, dptr(F), dptr(T), dptr(E)))
        return (F, T, E) if with_energy else (F, T)

    # ---- the loop body one phase at a time (Condensate.cpp:335-378), arrays by global index
    def calculateforces(self) -> np.ndarray:
        """MD::calculateforces(pairs, HSPotential): the WCA core forces (+ harmonic bonds)."""
        F = np.empty((self.n, 3))
        _check(self._h, _lib.lib().mtg_calculateforces(self._h, dptr(F)))
        return F

    def add_patch_forces_and_torques(self, F: np.ndarray, T: np.ndarray) -> None:
        """calculate_forces_and_torques3D(pairs, ComboPatch, F, T): adds the patch forces to F and the lab
        torques to T, in place (C-contiguous float64 n x 3 arrays)."""
        _check(self._h, _lib.lib().mtg_calculate_forces_and_torques3D(self._h, dptr(_inplace(F)), dptr(_inplace(T))))

    def create_forces_and_torques_sphere(self, F: np.ndarray, T: np.ndarray, R: np.ndarray | None = None) -> None:
        """F (lab), T (lab) -> F~ (lab), T~ (body) in place; R: n x 6 noise, or None for Philox."""
        Rp = None if R is None else dptr(np.ascontiguousarray(R, dtype=np.float64))
        _check(self._h, _lib.lib().mtg_create_forces_and_torques_sphere(self._h, dptr(_inplace(F)), dptr(_inplace(T)),
                                                                         Rp))

    def advancemom_halfstep(self, F: np.ndarray, T: np.ndarray) -> None:
        _check(self._h, _lib.lib().mtg_advancemom_halfstep(self._h, dptr(np.ascontiguousarray(F, dtype=np.float64)),
                                                           dptr(np.ascontiguousarray(T, dtype=np.float64))))

    def advance_pos(self) -> None:
        _check(self._h, _lib.lib().mtg_advance_pos(self._h))

    def rotate(self) -> None:
        _check(self._h, _lib.lib().mtg_rotate(self._h))

    @property
    def launch_config(self) -> dict:
        """The pair pipeline's launch shapes (mtg_get_launch_config)."""
        c = _lib.LaunchConfig()
        _check(self._h, _lib.lib().mtg_get_launch_config(self._h, C.byref(c)))
        return c.as_dict()

    @launch_config.setter
    def launch_config(self, cfg: dict) -> None:
        c = _lib.LaunchConfig(**{k: int(v) for k, v in cfg.items()})
        _check(self._h, _lib.lib().mtg_set_launch_config(self._h, C.byref(c)))

    def autotune(self, steps_per_trial: int = 5) -> tuple:
        """mtg_autotune: returns (chosen launch shapes, ms per step with them); the trials advance the state."""
        c = _lib.LaunchConfig()
        ms = C.c_double()
        _check(self._h, _lib.lib().mtg_autotune(self._h, int(steps_per_trial), C.byref(c), C.byref(ms)))
        return c.as_dict(), float(ms.value)

    def set_wait_limit(self, limit: int) -> None:
        """Bound (iterations) on mtg_clusters' waiting loops; 0 restores their own bound."""
        _check(self._h, _lib.lib().mtg_set_wait_limit(self._h, int(limit)))

    def calculatepairs_parallel(self, rc: float, replica: int = 0) -> np.ndarray:
        """MD::calculatepairs_parallel: sorted (i < j) pairs of one replica within rc."""
        L = _lib.lib()
        npairs = C.c_int64(0)
        st = L.mtg_pairs(self._h, int(replica), float(rc), None, 0, C.byref(npairs))
        if st not in (0, 6):
            _check(self._h, st)
        out = np.empty((max(npairs.value, 1), 2), dtype=np.int32)
        _check(self._h, L.mtg_pairs(self._h, int(replica), float(rc), out.ctypes.data_as(_lib._I32),
                                    out.shape[0], C.byref(npairs)))
        return out[: npairs.value]

    def measured_temperature(self) -> np.ndarray:
        """LangevinNVTR::measured_temperature per replica: (<p^2/2m> xyz, <L^2/2I> xyz)."""
        out = np.empty((len(self.replicas), 6))
        _check(self._h, _lib.lib().mtg_temperature(self._h, dptr(out)))
        return out

    def step_temperatures(self, nsteps: int) -> np.ndarray:
        """nsteps steps, each followed by measured_temperature of that step: (nsteps, replicas, 6).  The
        per-step sums stay on the device and reach pinned host memory once per chunk of steps; one
        synchronisation at the end."""
        out = np.empty((int(nsteps), len(self.replicas), 6))
        _check(self._h, _lib.lib().mtg_step_temperatures(self._h, int(nsteps), dptr(out)))
        return out

    def observables(self) -> np.ndarray:
        """Per replica: patch energy, WCA energy, virial, bonded patch pairs, pairs in range."""
        out = np.empty((len(self.replicas), _lib.MTG_OBS_COUNT))
        _check(self._h, _lib.lib().mtg_observables(self._h, dptr(out)))
        return out

    def displacement(self) -> np.ndarray:
        d = np.empty((self.n, 3))
        _check(self._h, _lib.lib().mtg_get_displacement(self._h, dptr(d)))
        return d

    def sync(self) -> None:
        _check(self._h, _lib.lib().mtg_sync(self._h))

    @property
    def flags(self) -> int:
        return int(_lib.lib().mtg_flags(self._h))

    def gr(self, rmax: float, dr: float, replica: int = 0) -> np.ndarray:
        """calcg1: counts of unordered pair distances of one replica in bins of dr below floor(rmax/dr)*dr."""
        L = _lib.lib()
        nb = C.c_int(0)
        _check(self._h, L.mtg_gr(self._h, int(replica), float(rmax), float(dr), None, 0, C.byref(nb)))
        out = np.zeros(nb.value, dtype=np.int64)
        if nb.value:
            _check(self._h, L.mtg_gr(self._h, int(replica), float(rmax), float(dr),
                                     out.ctypes.data_as(C.POINTER(C.c_int64)), nb.value, C.byref(nb)))
        return out

    def clusters(self, cut: float, replica: int = 0) -> np.ndarray:
        """distance_graph: per particle of one replica, the smallest local index of its connected
        component in the graph of pairs closer than cut."""
        n = self.replicas[replica].n if 0 <= replica < len(self.replicas) else 1  # the library rejects the rest
        out = np.empty(n, dtype=np.int32)
        _check(self._h, _lib.lib().mtg_clusters(self._h, int(replica), float(cut), out.ctypes.data_as(_lib._I32)))
        return out

    def write_frame(self, directory, frame: int, runtime: int, every: int, strbase: str = "",
                    replica: int | None = None) -> tuple:
        """The pos / orientation frame files Condensate::run writes every `every` steps
        (Condensate.cpp:378-418), for the whole handle or one replica.  Returns the two paths."""
        from pathlib import Path
        st = self.get_state()
        x, Q = st["x"], st["Q"]
        if replica is not None:
            off = int(_lib.lib().mtg_replica_offset(self._h, int(replica)))
            n = self.replicas[replica].n
            x, Q = x[off:off + n], Q[off:off + n]
        paths = tuple(Path(directory) / frame_name(kind, frame, runtime, every, strbase) for kind in ("pos", "orientation"))
        write_csv(paths[0], x)
        write_csv(paths[1], Q)
        return paths

    @property
    def rebuilds(self) -> int:
        """Neighbour-list rebuilds so far (0 without a skin)."""
        return int(_lib.lib().mtg_neighbor_rebuilds(self._h))

    def clear_flags(self) -> None:
        """Clear the device-latched condition bits (mtg_clear_flags)."""
        _lib.lib().mtg_clear_flags(self._h)

    @property
    def draw(self) -> int:
        return int(_lib.lib().mtg_get_draw(self._h))

    @draw.setter
    def draw(self, value: int) -> None:
        _check(self._h, _lib.lib().mtg_set_draw(self._h, int(value)))

    @property
    def launches(self) -> int:
        return int(_lib.lib().mtg_launch_count(self._h))

    @property
    def stream(self) -> int:
        return int(_lib.lib().mtg_stream(self._h) or 0)


def random_positions(n: int, box: float, periodic: bool = True, min_dist: float = 0.9, seed: int = 0) -> np.ndarray:
    x = np.empty((n, 3))
    st = _lib.lib().mtg_random_positions(int(n), float(box), int(bool(periodic)), float(min_dist),
                                         int(seed) & 0xFFFFFFFFFFFFFFFF, dptr(x))
    if st != 0:
        raise MtgError(st, f"could not place {n} particles at min_dist {min_dist} in a box of {box}")
    return x


def random_chains(n_chains: int, beads: int, box: float, periodic: bool = True, step: float = 1.0,
                  min_dist: float = 0.9, seed: int = 0) -> np.ndarray:
    """Self-avoiding random-walk chains (bond length ``step``, every bead >= ``min_dist`` from all
    others); chain c's bead b is row c * beads + b."""
    x = np.empty((n_chains * beads, 3))
    st = _lib.lib().mtg_random_chains(int(n_chains), int(beads), float(box), int(bool(periodic)), float(step),
                                      float(min_dist), int(seed) & 0xFFFFFFFFFFFFFFFF, dptr(x))
    if st != 0:
        raise MtgError(st, f"could not place {n_chains} chains of {beads} beads in a box of {box}")
    return x


def frame_name(kind: str, frame: int, runtime: int, every: int, strbase: str = "") -> str:
    """Condensate::run's frame file name, e.g. frame_name("pos", 7, 1000, 10) == "pos_i=007.csv"."""
    L = _lib.lib()
    n = L.mtg_frame_name(None, 0, kind.encode(), strbase.encode(), int(frame), int(runtime), int(every))
    if n < 0:
        raise ValueError("frame_name: every >= 1, runtime >= 0 and frame >= 0 are required")
    buf = C.create_string_buffer(n + 1)
    L.mtg_frame_name(buf, n + 1, kind.encode(), strbase.encode(), int(frame), int(runtime), int(every))
    return buf.value.decode()


def write_csv(path, a) -> None:
    """A matrix as the reference writes it (matrix::operator<<=: ',' separated, %g values)."""
    a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(len(a), -1))
    st = _lib.lib().mtg_csv_write(str(path).encode(), dptr(a), a.shape[0], a.shape[1])
    if st != 0:
        raise MtgError(st, f"could not write {path}")


def read_csv(path) -> np.ndarray:
    """importcsv: rows from lines, atof per ','-cell, short rows padded with 0."""
    L = _lib.lib()
    rows, cols = C.c_int64(0), C.c_int(0)
    st = L.mtg_csv_read(str(path).encode(), None, 0, C.byref(rows), C.byref(cols))
    if st != 0:
        raise MtgError(st, f"could not read {path}")
    out = np.zeros((rows.value, cols.value))
    if out.size:
        st = L.mtg_csv_read(str(path).encode(), dptr(out), out.size, C.byref(rows), C.byref(cols))
        if st != 0:
            raise MtgError(st, f"could not read {path}")
    return out


def random_rotations(n: int, seed: int = 0) -> np.ndarray:
    Q = np.empty((n, 9))
    _lib.lib().mtg_random_rotations(int(n), int(seed) & 0xFFFFFFFFFFFFFFFF, dptr(Q))
    return Q


def binding_single(on_rate: float, off_rate: float) -> "_lib.BindingModel":
    """BindingModelSingle(on_rate, off_rate) in table form (mtg_binding_single)."""
    m = _lib.BindingModel()
    _lib.lib().mtg_binding_single(C.byref(m), float(on_rate), float(off_rate))
    return m


def binding_binary_equilibrium(div: int) -> "_lib.BindingModel":
    """BindingModelBinary(div) + setup_equilibrium() in table form."""
    m = _lib.BindingModel()
    _lib.lib().mtg_binding_binary_equilibrium(C.byref(m), int(div))
    return m


def binding_tables(rule: int, drate, trate, div1: int = 0, div2: int = 0, np_: int = 1) -> "_lib.BindingModel":
    """A binding model from its rate tables (e.g. a BindingModelTernary's doubr** / tripr*** vectors):
    rule 0 one species, 1 binary (patch < div1), 2 SortingFunctionUniform, 3 SortingFunctionNonUniform."""
    m = _lib.BindingModel()
    m.species_rule, m.div1, m.div2, m.np = int(rule), int(div1), int(div2), int(np_)
    d = np.asarray(drate, float).reshape(6, 4)
    t = np.asarray(trate, float).reshape(10, 16)
    for r in range(6):
        for k in range(4):
            m.drate[r][k] = float(d[r, k])
    for r in range(10):
        for k in range(16):
            m.trate[r][k] = float(t[r, k])
    return m
