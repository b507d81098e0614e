"""The launch-parameter autotuner (svm_tuner_*) against the restated reference kernelTuner
(oracle/tuner.py, kernelTuner.cpp:4-126): the same sequences of measured times give the same
parameter after every call, the same medians and the same completion state.  Host logic only: no
CUDA call is made (times are fed with svm_tuner_record)."""
import ctypes as C

import numpy as np
import pytest

from tuner import KernelTunerOracle


@pytest.fixture(scope="module")
def lib(svm_lib):
    return svm_lib.lib()


def make(lib, *args):
    h = C.c_void_p()
    assert lib.svm_tuner_create(*args, None, C.byref(h)) == 0
    return h


def param(lib, h):
    v = C.c_int()
    assert lib.svm_tuner_parameter(h, C.byref(v)) == 0
    return v.value


@pytest.mark.parametrize("args,calls,seed", [((64, 1024, 64, 3, 20), 400, 1), ((32, 256, 32, 4, 5), 300, 2),
                                             ((128, 128, 32, 1, 0), 50, 3), ((64, 512, 64, 5, 37), 1000, 4)])
def test_tuner_matches_reference_state_machine(lib, args, calls, seed):
    h = make(lib, *args)
    o = KernelTunerOracle(*args)
    rng = np.random.default_rng(seed)
    # times with a clear optimum that moves half-way through, plus noise and exact ties
    best_a, best_b = o.candidates[len(o.candidates) // 3], o.candidates[-1]
    try:
        for i in range(calls):
            best = best_a if i < calls // 2 else best_b
            p = param(lib, h)
            assert p == o.parameter
            ms = 1.0 + abs(p - best) / 256.0 + float(rng.integers(0, 3)) * 0.01
            assert lib.svm_tuner_record(h, C.c_float(ms)) == 0
            o.call(float(np.float32(ms)))
            done = C.c_int()
            lib.svm_tuner_sampling_complete(h, C.byref(done))
            assert bool(done.value) == (o.state != 0)
        n = C.c_int()
        cand = np.zeros(64, dtype=np.int32)
        med = np.zeros(64, dtype=np.float32)
        assert lib.svm_tuner_timing_data(h, cand, med, 64, C.byref(n)) == 0
        assert list(cand[: n.value]) == o.candidates
        assert np.array_equal(med[: n.value], np.array(o.medians, dtype=np.float32))
    finally:
        lib.svm_tuner_destroy(h)


def test_tuner_picks_the_fastest_candidate(lib):
    h = make(lib, 64, 512, 64, 3, 1000)
    try:
        for _ in range(200):
            p = param(lib, h)
            lib.svm_tuner_record(h, C.c_float(1.0 + abs(p - 320) / 100.0))
        assert param(lib, h) == 320
    finally:
        lib.svm_tuner_destroy(h)


def test_tuner_rejects_bad_arguments(lib):
    h = C.c_void_p()
    assert lib.svm_tuner_create(64, 32, 32, 3, 10, None, C.byref(h)) != 0
    assert lib.svm_tuner_create(64, 128, 0, 3, 10, None, C.byref(h)) != 0
