"""The integer-pipe FP64 <-> FP32 conversions used by the FP64-bound kernels equal the hardware
conversions bit for bit (tests/csrc/conv_check.cu), and the FP64 reciprocal recip_nr is within one
ulp of the IEEE division (tests/csrc/recip_check.cu); both harnesses built here with nvcc for
sm_103a."""
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


def test_recip_nr_within_one_ulp_of_division(cuda_lib):
    """recip_nr (reciprocal estimate + one third-order Newton step, used in place of the FP64
    division by the coefficient and bottom kernels and the nodal cell kernels' 1/rhohalf) is within 1 ulp of the IEEE division 1.0/x
    on every input it refines (biased exponents 64..1980), and inputs outside that range take the
    division itself (bitwise equal)."""
    import re
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "recip_check")
        cmd = [B.nvcc(), *B.ARCH, "-O3", "-std=c++17", "-I", os.path.join(B.ROOT, "include"),
               "-I", B.CSRC, os.path.join(HERE, "csrc", "recip_check.cu"), "-o", exe]
        subprocess.run(cmd, check=True, capture_output=True, text=True)
        r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stdout + r.stderr
        m = re.search(r"max_ulp (\d+) differing (\d+) fallback_mismatches (\d+)", r.stdout)
        assert m, r.stdout
        max_ulp, differing, fallback = (int(v) for v in m.groups())
        print(r.stdout.strip())
        assert max_ulp <= 1, r.stdout
        assert fallback == 0, r.stdout
