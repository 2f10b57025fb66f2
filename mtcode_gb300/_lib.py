"""ctypes view of the C ABI in ``include/mtcode_gb300.h`` (libmtcode_gb300.so).

The shared library is the product; this module only binds it.  Loading fails loudly if the library
has not been built -- there is no Python or CPU fallback for any operation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libmtcode_gb300.so"

MTG_MAX_TYPES = 4
MTG_MAX_ORIENT = 16
MTG_MAX_POTS = 64
MTG_OBS_COUNT = 5
MTG_PROFILE_KERNELS = 11
MTG_NOALLOC_MAX_PARTICLES = 65536
MTG_NOALLOC_MAX_CELLS = 65536
PROFILE_KERNEL_NAMES = ("scan_reduce", "scan_top", "scan_down", "scatter", "force", "bind_begin", "bind_decide",
                        "pairfind", "pairforce", "patch_pairs", "epilogue")
MTG_FP32 = 0
MTG_FP64 = 1
MTG_FLAG_NONFINITE = 0x1
MTG_FLAG_FORCE_LIMIT = 0x2
MTG_FLAG_BIND = 0x20

STATUS = {
    0: "MTG_OK", 1: "MTG_ERR_ARG", 2: "MTG_ERR_CUDA", 3: "MTG_ERR_NOMEM", 4: "MTG_ERR_STATE",
    5: "MTG_ERR_NONFINITE", 6: "MTG_ERR_CAPACITY", 7: "MTG_ERR_TIMEOUT", 8: "MTG_ERR_NODEVICE",
}


class PatchModel(C.Structure):
    _fields_ = [
        ("n_types", C.c_int),
        ("patches_per_type", C.c_int * MTG_MAX_TYPES),
        ("count_per_type", C.c_int * MTG_MAX_TYPES),
        ("orient", (C.c_double * 3) * MTG_MAX_ORIENT),
        ("params", (C.c_double * 3) * MTG_MAX_POTS),
    ]


class LaunchConfig(C.Structure):
    _fields_ = [("pairfind_threads", C.c_int), ("pairforce_blocks_per_sm", C.c_int),
                ("patch_blocks_per_sm", C.c_int), ("epilogue_threads", C.c_int), ("fused_pairs", C.c_int)]

    def as_dict(self) -> dict:
        return {name: int(getattr(self, name)) for name, _ in self._fields_}


class ReplicaDesc(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("box", C.c_double),
        ("periodic", C.c_int),
        ("dt", C.c_double),
        ("kT", C.c_double),
        ("gamma", C.c_double),
        ("gammar", C.c_double),
        ("mass", C.c_double),
        ("inertia", C.c_double),
        ("hs_eps", C.c_double),
        ("hs_sigma", C.c_double),
        ("max_dist2", C.c_double),
        ("seed", C.c_uint64),
        ("model", PatchModel),
    ]


class Config(C.Structure):
    _fields_ = [
        ("precision", C.c_int),
        ("n_replicas", C.c_int),
        ("replicas", C.POINTER(ReplicaDesc)),
        ("device", C.c_int),
        ("track_displacement", C.c_int),
        ("force_kernel", C.c_int),
        ("neighbor_skin", C.c_double),
    ]


class BindingModel(C.Structure):
    """mtg_binding_model: species rule, doublet rows (11, 12, 13, 22, 23, 33), triplet rows (111 ... 333)."""
    _fields_ = [
        ("species_rule", C.c_int),
        ("div1", C.c_int),
        ("div2", C.c_int),
        ("np", C.c_int),
        ("drate", (C.c_double * 4) * 6),
        ("trate", (C.c_double * 16) * 10),
    ]


class SingleBond(C.Structure):
    _fields_ = [
        ("model", BindingModel),
        ("max_ang", C.c_double),
        ("list_cut", C.c_double),
        ("patch_every", C.c_int),
    ]


_D = C.POINTER(C.c_double)
_I32 = C.POINTER(C.c_int32)
_U8 = C.POINTER(C.c_uint8)
_H = C.c_void_p

# (name, restype, argtypes) for every entry point of include/mtcode_gb300.h
SIGNATURES = [
    ("mtg_model_tetrahedral", None, [C.POINTER(PatchModel), C.c_double, C.c_double, C.c_double]),
    ("mtg_model_bivalent", None, [C.POINTER(PatchModel), C.c_double, C.c_double, C.c_double]),
    ("mtg_replica_defaults", None, [C.POINTER(ReplicaDesc)]),
    ("mtg_create", C.c_int, [C.POINTER(Config), C.POINTER(_H)]),
    ("mtg_destroy", None, [_H]),
    ("mtg_num_particles", C.c_int64, [_H]),
    ("mtg_replica_offset", C.c_int64, [_H, C.c_int]),
    ("mtg_set_state", C.c_int, [_H, _D, _D, _D, _D, _D, _D]),
    ("mtg_get_state", C.c_int, [_H, _D, _D, _D, _D, _D, _D]),
    ("mtg_init_forces", C.c_int, [_H]),
    ("mtg_init_forces_noise", C.c_int, [_H, _D]),
    ("mtg_step_profile", C.c_int, [_H, C.c_int, _D]),
    ("mtg_calculateforces", C.c_int, [_H, _D]),
    ("mtg_calculate_forces_and_torques3D", C.c_int, [_H, _D, _D]),
    ("mtg_create_forces_and_torques_sphere", C.c_int, [_H, _D, _D, _D]),
    ("mtg_advancemom_halfstep", C.c_int, [_H, _D, _D]),
    ("mtg_advance_pos", C.c_int, [_H]),
    ("mtg_rotate", C.c_int, [_H]),
    ("mtg_set_wait_limit", C.c_int, [_H, C.c_int64]),
    ("mtg_get_launch_config", C.c_int, [_H, C.POINTER(LaunchConfig)]),
    ("mtg_set_launch_config", C.c_int, [_H, C.POINTER(LaunchConfig)]),
    ("mtg_autotune", C.c_int, [_H, C.c_int, C.POINTER(LaunchConfig), C.POINTER(C.c_double)]),
    ("mtg_step", C.c_int, [_H, C.c_int]),
    ("mtg_step_noise", C.c_int, [_H, C.c_int, _D]),
    ("mtg_forces", C.c_int, [_H, _D, _D, _D]),
    ("mtg_set_bonds", C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.c_int64, C.c_double, C.c_double]),
    ("mtg_neighbor_rebuilds", C.c_int64, [_H]),
    ("mtg_gr", C.c_int, [_H, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_int64), C.c_int, C.POINTER(C.c_int)]),
    ("mtg_clusters", C.c_int, [_H, C.c_int, C.c_double, _I32]),
    ("mtg_pairs", C.c_int, [_H, C.c_int, C.c_double, _I32, C.c_int64, C.POINTER(C.c_int64)]),
    ("mtg_temperature", C.c_int, [_H, _D]),
    ("mtg_step_temperatures", C.c_int, [_H, C.c_int, _D]),
    ("mtg_observables", C.c_int, [_H, _D]),
    ("mtg_get_displacement", C.c_int, [_H, _D]),
    ("mtg_get_draw", C.c_uint64, [_H]),
    ("mtg_set_draw", C.c_int, [_H, C.c_uint64]),
    ("mtg_sync", C.c_int, [_H]),
    ("mtg_flags", C.c_uint32, [_H]),
    ("mtg_clear_flags", None, [_H]),
    ("mtg_stream", C.c_void_p, [_H]),
    ("mtg_launch_count", C.c_int64, [_H]),
    ("mtg_last_error", C.c_char_p, [_H]),
    ("mtg_status_string", C.c_char_p, [C.c_int]),
    ("mtg_api_version", C.c_int, []),
    ("mtg_pairs_noalloc", C.c_int, [C.c_void_p, C.c_int, C.c_double, C.c_int, C.c_double, C.c_void_p, C.c_int64,
                                     C.c_void_p, C.c_void_p]),
    ("mtg_random_positions", C.c_int, [C.c_int, C.c_double, C.c_int, C.c_double, C.c_uint64, _D]),
    ("mtg_random_rotations", None, [C.c_int, C.c_uint64, _D]),
    ("mtg_random_chains", C.c_int, [C.c_int, C.c_int, C.c_double, C.c_int, C.c_double, C.c_double, C.c_uint64, _D]),
    ("mtg_csv_write", C.c_int, [C.c_char_p, _D, C.c_int64, C.c_int]),
    ("mtg_csv_read", C.c_int, [C.c_char_p, _D, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int)]),
    ("mtg_frame_name", C.c_int, [C.c_char_p, C.c_int, C.c_char_p, C.c_char_p, C.c_int, C.c_int, C.c_int]),
    ("mtg_binding_single", None, [C.POINTER(BindingModel), C.c_double, C.c_double]),
    ("mtg_binding_binary_equilibrium", None, [C.POINTER(BindingModel), C.c_int]),
    ("mtg_single_bond_defaults", None, [C.POINTER(SingleBond)]),
    ("mtg_set_single_bond", C.c_int, [_H, C.POINTER(SingleBond)]),
    ("mtg_num_patches", C.c_int64, [_H]),
    ("mtg_patch_offset", C.c_int64, [_H, C.c_int]),
    ("mtg_set_bind_state", C.c_int, [_H, _I32, _U8]),
    ("mtg_get_bind_state", C.c_int, [_H, _I32, _U8]),
    ("mtg_bind_update", C.c_int, [_H, _D, _D]),
    ("mtg_setup_random_binding", C.c_int, [_H, C.c_uint64]),
]

_lib = None


def lib() -> C.CDLL:
    """Load (once) and return the shared library with typed signatures."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(
                f"{LIB_PATH} is not built; run `python -m mtcode_gb300.build` (nvcc, sm_103a). "
                "mtcode_gb300 has no CPU fallback.")
        handle = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


class MtgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, "arrays passed to the C ABI must be C-contiguous float64"
    return a.ctypes.data_as(_D)
