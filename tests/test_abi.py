"""The C-ABI library loads, exports every symbol include/cavgpu.h declares, and its
parameter struct matches the ctypes mirror.  No GPU is needed: the only
device call made here is the one that must fail without a GPU."""
import ctypes
import os
import re
import subprocess
import sys

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "cavgpu.h")


@pytest.fixture(scope="module")
def built():
    sys.path.insert(0, os.path.join(ROOT, "caviar-v2_gb300"))
    import build as B

    if not os.path.exists(B.LIB):
        B.build()
    import cavgpu

    return cavgpu


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(cavgpu_\w+)\s*\(", txt)))


def test_every_declared_symbol_is_exported(built):
    lib = built.lib()
    names = declared_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n
        assert n in built._SIGS, f"{n} has no ctypes signature"


def test_exports_match_nm(built):
    out = subprocess.run(["nm", "-D", "--defined-only", built.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (cavgpu_\w+)", out))
    assert set(declared_functions()) <= exported


def test_params_layout_matches_c(built, tmp_path):
    src = tmp_path / "sz.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "cavgpu.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu\\n\", sizeof(cavgpu_params),"
        " offsetof(cavgpu_params, mass), offsetof(cavgpu_params, seed),"
        " offsetof(cavgpu_params, precision), offsetof(cavgpu_params, steps_per_graph));return 0;}\n")
    exe = tmp_path / "sz"
    subprocess.run(["gcc", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    P = built.Params
    assert vals == [ctypes.sizeof(P), P.mass.offset, P.seed.offset, P.precision.offset, P.steps_per_graph.offset]


def test_default_params_and_strerror(built):
    p = built.Params()
    built.lib().cavgpu_default_params(ctypes.byref(p))
    assert p.nl_coef == 1.12347 and p.k_b == 1.0 and p.ntypes == 1 and tuple(p.bc) == (1, 1, 1)
    assert built.lib().cavgpu_strerror(built.E_NAN) == b"NaN acceleration"


def test_no_gpu_means_error_not_fallback(built):
    """Without a GPU the library refuses to run (there is no CPU path)."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    p = built.Params()
    built.lib().cavgpu_default_params(ctypes.byref(p))
    for a in range(3):
        p.hi[a] = 10.0
    h = ctypes.c_void_p()
    assert built.lib().cavgpu_create(ctypes.byref(p), ctypes.byref(h)) == built.E_CUDA
