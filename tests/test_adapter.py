"""The C++ adapter (include/LangevinNVTRGPU.hpp): the reference-side interface over the C ABI.

CPU: the adapter compiles and links standalone, and -- where the reference sources exist -- with the
reference's own matrix<double>/TetrahedralPatch types exactly as Condensate::run would use it.
GPU: a C++ driver of the Condensate::run loop through the adapter, checked against the oracle.
"""
import math
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

from mtcode_gb300 import _lib
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, random_positions, random_rotations
from mtcode_gb300.workloads import box_for
from oracle import pyoracle as po
from tests._util import sorted_pairs

ROOT = Path(__file__).resolve().parents[1]
BUILD = ROOT / "mtcode_gb300" / "_build"
REF = po.reference_root() / "Code"


def compile_driver(src: str, out: Path, extra=()) -> Path:
    _lib.lib()  # the library must exist to link against
    BUILD.mkdir(exist_ok=True)
    cmd = ["g++", "-std=c++17", "-O2", "-w", "-I", str(ROOT / "include"), *extra, str(ROOT / "tests" / "cpp" / src),
           "-L", str(ROOT / "mtcode_gb300"), "-lmtcode_gb300", f"-Wl,-rpath,{ROOT / 'mtcode_gb300'}", "-o", str(out)]
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert proc.returncode == 0, proc.stdout[-3000:]
    return out


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_adapter_compiles_standalone():
    compile_driver("condensate_gpu.cpp", BUILD / "condensate_gpu")


@pytest.mark.skipif(not REF.is_dir(), reason="the reference sources are only present in the build container")
def test_adapter_compiles_with_the_reference_types():
    compile_driver("reference_dropin.cpp", BUILD / "reference_dropin", extra=("-I", str(REF)))


@pytest.mark.gpu
def test_condensate_loop_through_the_adapter_matches_oracle(tmp_path):
    exe = compile_driver("condensate_gpu.cpp", BUILD / "condensate_gpu")
    n, steps = 300, 25
    spec = ReplicaSpec(n=n, box=box_for(n, 0.3), model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9)),
                       kT=0.0)
    x = random_positions(n, spec.box, True, 0.95, 21)
    Q = random_rotations(n, 22)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([n, _lib.MTG_FP64, steps], dtype=np.int32).tofile(f)
        np.array([spec.box, spec.kT, spec.dt], dtype=np.float64).tofile(f)
        x.tofile(f)
        Q.tofile(f)
    out = tmp_path / "out.bin"
    proc = subprocess.run([str(exe), str(inp), str(out)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stdout
    raw = out.read_bytes()
    npairs = int(np.frombuffer(raw[:8], dtype=np.int64)[0])
    off = 8
    pairs = np.frombuffer(raw[off:off + 8 * npairs], dtype=np.int32).reshape(-1, 2)
    off += 8 * npairs
    vals = np.frombuffer(raw[off:], dtype=np.float64)
    F, T, xf, pf, Qf, Lf = (vals[a:b].reshape(n, -1) for a, b in
                             ((0, 3 * n), (3 * n, 6 * n), (6 * n, 9 * n), (9 * n, 12 * n), (12 * n, 21 * n),
                              (21 * n, 24 * n)))
    sysm = po.System(spec)
    assert np.array_equal(sorted_pairs(pairs), sorted_pairs(sysm.pairs(x, 1.68)))
    Fo, To = sysm.forces(x, Q)
    assert np.linalg.norm(F - Fo) <= 1e-12 * np.linalg.norm(Fo)
    assert np.linalg.norm(T - To) <= 1e-12 * np.linalg.norm(To)
    st = dict(x=x.copy(), p=np.zeros((n, 3)), Lb=np.zeros((n, 3)), Q=Q.copy())
    st["Ft"], st["Tt"] = sysm.init_forces(st["x"], st["p"], st["Lb"], st["Q"])
    assert sysm.run(st, steps, noise_mode=0) == 0
    for got, key in ((xf, "x"), (pf, "p"), (Qf, "Q"), (Lf, "Lb")):
        assert np.abs(got - st[key]).max() <= 1e-9 * max(1.0, np.abs(st[key]).max()), key


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_per_phase_driver_compiles_standalone():
    compile_driver("phases_gpu.cpp", BUILD / "phases_gpu")


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_singlebond_driver_compiles_standalone():
    compile_driver("singlebond_gpu.cpp", BUILD / "singlebond_gpu")


@pytest.mark.gpu
def test_singlebond_loop_through_the_adapter_matches_oracle(tmp_path):
    """run_singlebond through the adapter (FP64, noise off): the first onlyone_nonlets pass (bond state,
    forces, torques) and the bond state and configuration after init + 25 steps equal the oracle's."""
    exe = compile_driver("singlebond_gpu.cpp", BUILD / "singlebond_gpu")
    n, steps = 300, 25
    spec = ReplicaSpec(n=n, box=box_for(n, 0.3), model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.7)),
                       kT=0.0, seed=0)
    x = random_positions(n, spec.box, True, 0.95, 31)
    Q = random_rotations(n, 32)
    inp = tmp_path / "in.bin"
    with open(inp, "wb") as f:
        np.array([n, _lib.MTG_FP64, steps], dtype=np.int32).tofile(f)
        np.array([spec.box, spec.kT, spec.dt], dtype=np.float64).tofile(f)
        x.tofile(f)
        Q.tofile(f)
    out = tmp_path / "out.bin"
    proc = subprocess.run([str(exe), str(inp), str(out)], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                          timeout=300)
    assert proc.returncode == 0, proc.stdout
    raw = out.read_bytes()
    np_ = 4 * n
    F = np.frombuffer(raw, np.float64, 3 * n, 0).reshape(n, 3)
    T = np.frombuffer(raw, np.float64, 3 * n, 24 * n).reshape(n, 3)
    off = 48 * n
    ib1 = np.frombuffer(raw, np.uint8, np_, off)
    ib2 = np.frombuffer(raw, np.uint8, np_, off + np_)
    off += 2 * np_
    bt1 = np.frombuffer(raw, np.int32, np_, off)
    bt2 = np.frombuffer(raw, np.int32, np_, off + 4 * np_)
    off += 8 * np_
    xf = np.frombuffer(raw, np.float64, 3 * n, off).reshape(n, 3)
    Qf = np.frombuffer(raw, np.float64, 9 * n, off + 24 * n).reshape(n, 9)
    sysm = po.System(spec)
    bind = po.binding_single(0.7, 0.5)
    ncell = max(1, int(math.floor(spec.box / 2.5)))
    bt = np.zeros(np_, dtype=np.intc)
    ib = np.zeros(np_, dtype=np.uint8)
    st, Fb, Tb = sysm.bind_update(x, Q, sysm.patch_list(x, Q, sysm.pairs(x, 2.5, ncell), sysm.default_max_ang()),
                                  bind, bt, ib, rng=0, seed=0, replica=0, draw=0)
    assert st == 0 and ib.sum() > 0
    assert np.array_equal(ib1, ib) and np.array_equal(bt1[ib == 1], bt[ib == 1])
    Fo = sysm.central_forces(x) + Fb
    assert np.linalg.norm(F - Fo) <= 1e-12 * np.linalg.norm(Fo)
    assert np.linalg.norm(T - Tb) <= 1e-12 * np.linalg.norm(Tb)
    state = dict(x=x.copy(), p=np.zeros((n, 3)), Lb=np.zeros((n, 3)), Q=Q.copy(), Ft=np.zeros((n, 3)),
                 Tt=np.zeros((n, 3)), boundto=bt, isbound=ib)
    assert sysm.run_singlebond(state, bind, steps, sysm.default_max_ang(), init=True, init_draw=1, seed=0,
                               replica=0, draw0=2) == 0
    assert np.array_equal(ib2, state["isbound"])
    assert np.array_equal(bt2[ib2 == 1], state["boundto"][state["isbound"] == 1])
    assert np.abs(xf - state["x"]).max() <= 1e-9 * max(1.0, np.abs(state["x"]).max())
    assert np.abs(Qf - state["Q"]).max() <= 1e-9
