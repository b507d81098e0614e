"""The allocation-free energy entry point (svm_energy_noalloc), called through the C ABI.

It exists for callers that cannot allocate device memory (hosts whose device memory belongs to
their own pool allocator; per-step code that must not take cudaMalloc's implicit device-wide
synchronisation).  Its scratch is a fixed static device array shared by all calls, so this test
calls it twice in a row on caller-owned buffers and checks both results against the allocating
entry point, svm_model_compute_energy.  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12  # both are deterministic block-tree reductions of the same FP64 terms


def test_noalloc_energy_matches_model_energy_twice(svm_lib):
    svm = svm_lib
    if svm.device_count() < 1:
        pytest.fail("no CUDA device")
    torch = pytest.importorskip("torch")
    from curvedspacevertexmodel_gb300 import _lib

    n = 3000
    noise = svm.noiseSource()
    noise.setReproducibleSeed(21)
    m = svm.sphericalVertexModel(n, noise, 1.0, 3.7)
    m.setScalarModelParameter(1.3)
    m.computeGeometry()
    expected = m.computeEnergy()
    ap = torch.tensor(m.areaPerimeter().reshape(-1), dtype=torch.float64, device="cuda")
    pref = torch.tensor(np.tile([1.0, 3.7], n), dtype=torch.float64, device="cuda")
    out = torch.full((1,), -1.0, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for _ in range(2):
        out.fill_(-1.0)
        _lib.call("svm_energy_noalloc", C.c_void_p(ap.data_ptr()), C.c_void_p(pref.data_ptr()), 1.3, n,
                  C.c_void_p(out.data_ptr()), C.c_void_p(stream))
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - expected) <= RTOL * abs(expected), (got, expected)
    # sizes beyond the fixed scratch are rejected before any device work
    rc = _lib.lib().svm_energy_noalloc(C.c_void_p(ap.data_ptr()), C.c_void_p(pref.data_ptr()), 1.0,
                                       _lib.SVM_NOALLOC_MAX_CELLS + 1, C.c_void_p(out.data_ptr()), None)
    assert rc == _lib.SVM_ERR_ARG
