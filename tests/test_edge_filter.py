"""The FP32 pre-check of the T1 length test (csrc/svm_edge_filter.h): an edge it calls clearly
longer than the threshold has an exact chord, hence an arc, beyond the threshold by the documented
margin, so the FP64 test it skips (geodesic < t, sphericalVertexModel.cpp:475) could not have found
it shorter.  The header is compiled for the host: the same IEEE FP32 operations as the device."""
import json
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "curvedspacevertexmodel_gb300", "csrc")


def test_clearly_longer_keeps_its_margin():
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "edge_filter_check")
        subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I" + CSRC,
                        os.path.join(ROOT, "tests", "native", "edge_filter_check.cpp"), "-o", exe], check=True)
        r = subprocess.run([exe, "3000000"], capture_output=True, text=True, timeout=300)
    out = json.loads(r.stdout)
    assert r.returncode == 0 and out["violations"] == 0 and out["special_failures"] == 0, out
    # it decides a large share of the edges (those away from the threshold), so it is not vacuous
    assert out["decided"] > 0.3 * out["cases"], out
    assert out["worst_margin"] >= 9e-4, out
