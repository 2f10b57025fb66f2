"""The oracle's seeded input generators against the product library's (CPU only, no GPU).

The CPU baselines build their workloads with the oracle's generators so that they load nothing from the
product library; that is only fair if the inputs are the same.  Positions, rotations and chains must be
identical bit for bit, and building the batched workload that way must leave libmtcode_gb300.so unmapped.
"""
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

from mtcode_gb300 import system
from mtcode_gb300.workloads import box_for
from oracle import pyoracle as po

ROOT = Path(__file__).resolve().parents[1]
G = po.Generators


@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("n,phi,seed", [(1, 0.1, 0), (500, 0.15, 3), (4096, 0.25, 11), (20000, 0.3, 1234567)])
def test_positions_identical(n, phi, seed, periodic):
    box = box_for(n, phi)
    a = system.random_positions(n, box, periodic, 0.9, seed)
    b = G.random_positions(n, box, periodic, 0.9, seed)
    assert np.array_equal(a, b)


def test_positions_same_failure():
    with pytest.raises(Exception):
        system.random_positions(2000, 5.0, True, 0.9, 1)
    with pytest.raises(ValueError):
        G.random_positions(2000, 5.0, True, 0.9, 1)


@pytest.mark.parametrize("n,seed", [(1, 0), (777, 5), (50000, 2 ** 63 + 17)])
def test_rotations_identical(n, seed):
    assert np.array_equal(system.random_rotations(n, seed), G.random_rotations(n, seed))


@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("chains,beads,phi,seed", [(3, 10, 0.05, 0), (50, 100, 0.10, 9), (400, 25, 0.2, 77)])
def test_chains_identical(chains, beads, phi, seed, periodic):
    box = box_for(chains * beads, phi)
    a = system.random_chains(chains, beads, box, periodic, 1.0, 0.9, seed)
    b = G.random_chains(chains, beads, box, periodic, 1.0, 0.9, seed)
    assert np.array_equal(a, b)


def test_cpu_baseline_workload_leaves_the_product_library_unmapped():
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "from oracle import pyoracle as po\n"
        "from mtcode_gb300 import workloads\n"
        "W = workloads.patchy_c4(seed=0, n_replicas=8, gen=po.Generators)\n"
        "assert W.n_total > 0\n"
        "maps = open('/proc/self/maps').read()\n"
        "print('liboracle' in maps, 'libmtcode_gb300' in maps)\n" % str(ROOT))
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr[-2000:]
    assert out.stdout.split() == ["True", "False"], out.stdout
