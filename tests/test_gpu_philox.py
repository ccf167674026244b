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
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu


def test_oracle_philox_equals_curand(oracle_lib):
    sys.path.insert(0, os.path.join(ROOT, "caviar-v2_gb300"))
    import build as B

    if not os.path.exists(B.PHILOX):
        B.build()
    out = subprocess.run([B.PHILOX], capture_output=True, text=True, check=True).stdout.split("\n")
    rows = [ln.split() for ln in out if ln.strip()]
    assert len(rows) == 64
    for r in rows:
        seed, sub, off = (int(v, 16) for v in r[:3])
        want = [int(v, 16) for v in r[3:]]
        block = off // 4
        ctr = [block & 0xFFFFFFFF, block >> 32, sub & 0xFFFFFFFF, sub >> 32]
        key = [seed & 0xFFFFFFFF, seed >> 32]
        assert oracle_lib.philox(ctr, key) == want, r
