"""The Philox4x32-10 of the Langevin noise against cuRAND's implementation.

cuRAND's Philox4x32-10 state (curand_init(seed, subsequence, offset)) runs the
counter {offset/4 (low 64 bits), subsequence (high 64 bits)} under the key
{seed low, seed high}; its first curand4() is the block of that counter.  The
oracle's restatement (oracle/cav_oracle.c:orc_philox4x32_10, the algorithm of
Salmon et al., SC'11) must give the same 128 bits for every case; the device noise
equals the oracle's (tests/test_gpu_parity.py::test_langevin_noise_matches_oracle),
so this ties the GPU path's noise to NVIDIA's generator too.
"""
import os
import subprocess

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def philox_curand(tmp_path_factory):
    """tests/cpp/philox_curand.cu (a test helper that calls cuRAND's device API),
    compiled for sm_103a into a temporary directory."""
    exe = str(tmp_path_factory.mktemp("philox") / "philox_curand")
    nvcc = os.environ.get("NVCC", "nvcc")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
                    os.path.join(ROOT, "tests", "cpp", "philox_curand.cu"), "-o", exe], check=True)
    return exe


def test_oracle_philox_equals_curand(oracle_lib, philox_curand):
    out = subprocess.run([philox_curand], capture_output=True, text=True, check=True).stdout.split("\n")
    rows = [ln.split() for ln in out if ln.strip()]
    assert len(rows) == 64
    for r in rows:
        seed, sub, off = (int(v, 16) for v in r[:3])
        want = [int(v, 16) for v in r[3:]]
        block = off // 4
        ctr = [block & 0xFFFFFFFF, block >> 32, sub & 0xFFFFFFFF, sub >> 32]
        key = [seed & 0xFFFFFFFF, seed >> 32]
        assert oracle_lib.philox(ctr, key) == want, r
