"""The integer float <-> double conversions and the integer truncation of
csrc/fpconv.cuh (used by every form's kernels to keep conversions off GB300's
FP64 pipe) against the host compiler's IEEE conversions, on the CPU:
tests/native/fpconv_check.cpp is compiled with the host C++ compiler and run."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "4hetddft-isotropic_gb300", "csrc")


def _cuda_include():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    return None


def test_integer_conversions_match_ieee(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    inc = _cuda_include()
    if not cxx or not inc:
        pytest.skip("needs a host C++ compiler and the CUDA headers")
    exe = tmp_path / "fpconv_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, "-I", inc, os.path.join(HERE, "native", "fpconv_check.cpp"),
                    "-o", str(exe)], check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout
