"""The launch-shape autotuner (mtg_autotune) and its cache.

Every launch shape of the pair pipeline must give the same FP32 trajectory bit for bit (the force sums are fixed
point, so the order in which pairs are found and summed does not matter); the tuner returns a valid shape at
least as fast as it measured the starting one, and the cache hands the same shape back without tuning.
"""
import numpy as np
import pytest

from mtcode_gb300 import LangevinNVTRGPU, workloads
from mtcode_gb300 import tuning

pytestmark = pytest.mark.gpu

SHAPES = [{"pairfind_threads": 256, "pairforce_blocks_per_sm": 16, "patch_blocks_per_sm": 8, "epilogue_threads": 256,
           "fused_pairs": 1},
          {"pairfind_threads": 256, "pairforce_blocks_per_sm": 16, "patch_blocks_per_sm": 8, "epilogue_threads": 256,
           "fused_pairs": 0},
          {"pairfind_threads": 128, "pairforce_blocks_per_sm": 4, "patch_blocks_per_sm": 2, "epilogue_threads": 512,
           "fused_pairs": 1},
          {"pairfind_threads": 512, "pairforce_blocks_per_sm": 32, "patch_blocks_per_sm": 24, "epilogue_threads": 128,
           "fused_pairs": 0}]


def run(W, shape, steps=30):
    z = W.zeros3()
    with LangevinNVTRGPU(W.replicas, precision="fp32") as s:
        s.launch_config = shape
        assert s.launch_config == shape
        s.initialize(W.x, z, z, W.Q)
        s.init_forces()
        s.step(steps)
        return s.get_state()


def test_every_launch_shape_gives_the_same_fp32_trajectory():
    W = workloads.patchy_c4(seed=4, n_replicas=10, n_min=500, n_max=8000)
    ref = run(W, SHAPES[0])
    for shape in SHAPES[1:]:
        got = run(W, shape)
        for key in ("x", "p", "Lb", "Q", "Ft", "Tt"):
            assert np.array_equal(got[key], ref[key]), (shape, key)


def test_autotune_and_cache(tmp_path):
    W = workloads.patchy_c4(seed=5, n_replicas=24, n_min=1000, n_max=16000)
    z = W.zeros3()
    with LangevinNVTRGPU(W.replicas, precision="fp32") as s:
        s.initialize(W.x, z, z, W.Q)
        s.init_forces()
        s.step(5)
        with pytest.raises(Exception):
            s.launch_config = dict(SHAPES[0], pairfind_threads=96)   # not a supported block size
        got = tuning.tuned(s, "test", steps_per_trial=3, path=tmp_path / "shapes.json")
        assert got["source"] == "autotune" and got["ms_per_step"] > 0
        cfg = got["launch_config"]
        assert cfg["pairfind_threads"] in (128, 256, 512) and cfg["epilogue_threads"] in (128, 256, 512)
        assert 1 <= cfg["pairforce_blocks_per_sm"] <= 64 and 1 <= cfg["patch_blocks_per_sm"] <= 64
        assert cfg["fused_pairs"] in (0, 1)
        assert s.launch_config == cfg
        s.step(3)
        assert np.isfinite(s.get_state()["x"]).all() and s.flags == 0
    with LangevinNVTRGPU(W.replicas, precision="fp32") as s2:
        s2.initialize(W.x, z, z, W.Q)
        again = tuning.tuned(s2, "test", path=tmp_path / "shapes.json")
        assert again["source"] == "cache" and again["launch_config"] == cfg
        assert s2.launch_config == cfg
