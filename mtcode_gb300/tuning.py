"""Launch-shape tuning with a per-device, per-shape cache.

``tuned(handle, key)`` returns the pair pipeline's launch shapes for a workload: from the cache when this
device has tuned the same workload shape before, else from ``mtg_autotune`` on the handle's live state (the
trial steps advance the simulation), stored for next time.  The key names the workload's shape (precision,
replica count, particle count, density, skin, mode), the device (the GPU's name and SM count) and the library
build (a hash of its file).  The cache
is a JSON file in ``$MTCODE_TUNE_CACHE`` (default ``~/.cache/mtcode_gb300/launch_shapes.json``).
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path


def cache_path() -> Path:
    env = os.environ.get("MTCODE_TUNE_CACHE")
    return Path(env) if env else Path.home() / ".cache" / "mtcode_gb300" / "launch_shapes.json"


def device_key(device: int = 0) -> str:
    import torch
    p = torch.cuda.get_device_properties(device)
    return f"{p.name}|sm{p.major}{p.minor}|{p.multi_processor_count}SM"


def library_key() -> str:
    """A fingerprint of the loaded library's file: shapes tuned for other kernels are not reused."""
    from . import _lib
    try:
        return hashlib.sha1(Path(_lib.LIB_PATH).read_bytes()).hexdigest()[:12]
    except OSError:
        return "unknown"


def workload_key(handle, extra: str = "") -> str:
    reps = handle.replicas
    n = sum(r.n for r in reps)
    vol = sum(r.box ** 3 for r in reps)
    return f"{handle.precision}|{len(reps)} replicas|{n} particles|density {n / vol:.4f}|{extra}"


def _load(path: Path) -> dict:
    try:
        return json.loads(path.read_text())
    except (OSError, ValueError):
        return {}


def tuned(handle, extra: str = "", steps_per_trial: int = 5, device: int = 0, path: Path | None = None) -> dict:
    """The tuned launch shapes for this handle's workload; sets them on the handle.  Returns
    {"launch_config": ..., "source": "cache" | "autotune", "ms_per_step": ... (autotune only), "key": ...}."""
    path = path or cache_path()
    key = device_key(device) + "|lib " + library_key() + "||" + workload_key(handle, extra)
    cache = _load(path)
    if key in cache:
        handle.launch_config = cache[key]
        return {"launch_config": handle.launch_config, "source": "cache", "key": key}
    cfg, ms = handle.autotune(steps_per_trial)
    cache = _load(path)
    cache[key] = cfg
    try:
        path.parent.mkdir(parents=True, exist_ok=True)
        tmp = path.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
        os.replace(tmp, path)
    except OSError:
        pass   # a read-only home: the shapes still apply to this handle
    return {"launch_config": cfg, "source": "autotune", "ms_per_step": ms, "key": key}
