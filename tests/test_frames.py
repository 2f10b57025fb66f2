"""Frame files in the reference's format (host code of the library, no GPU for the format checks).

CPU: mtg_csv_write reproduces, byte for byte, what the reference's matrix operator<<= writes
(DataStructures/matrix2.cpp:898-912); mtg_csv_read parses like importcsv (matrix2.cpp:1597-1640),
pinned on the reference's own results (tests/golden/frames.npz, made by tests/golden/make_golden.py);
mtg_frame_name follows Condensate::run's naming (Condensate.cpp:296-300, 383-405).
GPU: frames written from a running system read back to the state at six significant digits, and a
system initialised from them carries on.
"""
import math

import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU
from mtcode_gb300.system import PatchModelSpec, ReplicaSpec, frame_name, random_positions, random_rotations, \
    read_csv, write_csv
from mtcode_gb300.workloads import box_for
from tests._util import load


def test_writer_matches_the_reference_bytes(tmp_path):
    d = load("frames.npz")
    write_csv(tmp_path / "m.csv", d["data"])
    assert (tmp_path / "m.csv").read_bytes() == d["written"].tobytes()


@pytest.mark.parametrize("k", range(4))
def test_reader_matches_importcsv(k, tmp_path):
    d = load("frames.npz")
    (tmp_path / "r.csv").write_bytes(d[f"csv_{k}"].tobytes())
    got = read_csv(tmp_path / "r.csv")
    want = d[f"parsed_{k}"]
    assert got.shape == want.shape
    assert np.array_equal(got, want, equal_nan=True)


def test_empty_line_reads_as_zeros(tmp_path):
    (tmp_path / "e.csv").write_text("1,2\n\n3,4\n")
    assert np.array_equal(read_csv(tmp_path / "e.csv"), [[1, 2], [0, 0], [3, 4]])


def test_round_trip_keeps_six_significant_digits(tmp_path):
    a = np.random.default_rng(2).normal(size=(100, 9)) * 37.0
    write_csv(tmp_path / "a.csv", a)
    b = read_csv(tmp_path / "a.csv")
    assert b.shape == a.shape
    assert np.allclose(b, a, rtol=5e-6, atol=0)
    write_csv(tmp_path / "b.csv", b)  # a second round trip is exact
    assert np.array_equal(read_csv(tmp_path / "b.csv"), b)


def test_frame_names_follow_condensate_run():
    assert frame_name("pos", 7, 1000, 10) == "pos_i=007.csv"         # ceil(1000/10) = 100: 3 digits
    assert frame_name("orientation", 7, 10001, 10, "_run2") == "orientation_run2_i=0007.csv"  # 1001: 4 digits
    assert frame_name("pos", 0, 5, 10) == "pos_i=0.csv"              # ceil(0.5) = 1: 1 digit
    assert frame_name("pos", 12, 0, 10) == "pos_i=12.csv"            # 0 -> 1 digit, wider numbers still print


@pytest.mark.gpu
def test_frames_from_a_running_system(tmp_path):
    n = 1000
    spec = ReplicaSpec(n=n, box=box_for(n, 0.15), model=PatchModelSpec.tetrahedral(n, 8.0, 1.2, math.acos(0.9)))
    x = random_positions(n, spec.box, True, 0.95, 3)
    Q = random_rotations(n, 4)
    z = np.zeros((n, 3))
    with LangevinNVTRGPU([spec, spec], precision="fp32") as s:
        s.initialize(np.concatenate([x, x]), np.concatenate([z, z]), np.concatenate([z, z]), np.concatenate([Q, Q]))
        s.init_forces()
        s.step(20)
        pos_path, ori_path = s.write_frame(tmp_path, 2, 100, 10, replica=1)
        st = s.get_state()
    assert pos_path.name == "pos_i=02.csv" and ori_path.name == "orientation_i=02.csv"  # ceil(100/10): 2 digits
    xr, Qr = read_csv(pos_path), read_csv(ori_path)
    assert np.allclose(xr, st["x"][n:], rtol=5e-6, atol=1e-12)
    assert np.allclose(Qr, st["Q"][n:], rtol=5e-6, atol=1e-6)
    # resume from the frame, as a run restarted from importcsv would
    with LangevinNVTRGPU([spec], precision="fp32") as s2:
        s2.initialize(xr, z, z, Qr)
        s2.init_forces()
        s2.step(5)
        s2.sync()
        assert np.isfinite(s2.getdat()).all()
