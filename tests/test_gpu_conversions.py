"""The integer-pipe FP64 <-> FP32 conversions used by the FP64-bound kernels equal the hardware
conversions bit for bit (tests/csrc/conv_check.cu, built here with nvcc for sm_103a)."""
import importlib
import os
import subprocess
import tempfile

import pytest

B = importlib.import_module("maestro_gb300.build")   # the module (the package exports build())

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_conversions_match_hardware(cuda_lib):
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "conv_check")
        cmd = [B.nvcc(), *B.ARCH, "-O3", "-std=c++17", "-I", os.path.join(B.ROOT, "include"),
               "-I", B.CSRC, os.path.join(HERE, "csrc", "conv_check.cu"), "-o", exe]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        assert "mismatches_to_float 0 mismatches_to_double 0" in r.stdout
