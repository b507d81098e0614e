"""The integer-pipe IEEE binary64 arithmetic (csrc/svm_softf64.cuh) that the FP64 kernels use for
their divisions and square roots: bit for bit the IEEE results.  On the CPU the header is compiled
for the host and checked against the host's operations; the GPU check runs the device build against
the hardware instructions through svm_softf64_check."""
import json
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "curvedspacevertexmodel_gb300", "csrc")


def test_softf64_bit_exact_on_the_host():
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "softf64_check")
        subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC,
                        os.path.join(ROOT, "tests", "native", "softf64_check.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe, "1500000"], capture_output=True, text=True, timeout=300)
    out = json.loads(r.stdout)
    assert r.returncode == 0 and all(out[k] == 0 for k in ("mul", "add", "div", "sqrt", "sub", "widen", "narrow")), out


@pytest.mark.gpu
def test_softf64_bit_exact_on_the_device(svm_lib):
    """2^28 random operand pairs per operation (every bit pattern, exponents near 1, near-cancelling
    pairs, short significands, divisors next to powers of two; conversions at and next to rounding
    ties), the device functions against the hardware's correctly rounded instructions."""
    from curvedspacevertexmodel_gb300 import _lib
    bad = np.zeros(6, dtype=np.uint64)
    _lib.call("svm_softf64_check", 1 << 28, 7, bad.ctypes.data)
    assert not bad.any(), bad
