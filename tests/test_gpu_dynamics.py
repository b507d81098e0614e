"""Dynamical observables on the device (svm_model_dynamics) against the oracle's restatement of
dynamicalFeatures (src/analysis/dynamicalFeatures.cpp:17-53), and the trajectory driver's files."""
import numpy as np
import pytest

import oracle
from gpu_helpers import stabilised

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_msd_and_overlap_match_oracle(svm, precision):
    m, bd = stabilised(svm, 5000, seed=4, stab=30, steps=30)
    m.precision = precision
    m.computeGeometry()
    ref = m.cellPositions()
    dyn = svm.dynamicalFeatures(m)
    bd.setT(0.05)
    bd.run(150)
    m.computeGeometry()
    cur = m.cellPositions()
    for fraction in (1.0, 0.37):
        for cutoff in (0.5, 0.2, 2.0):
            dyn.fraction = fraction
            msd_g, ov_g = dyn._both(cutoff)
            msd_o, ov_o = oracle.dynamics(ref, cur, m.radius, fraction, cutoff)
            assert abs(msd_g - msd_o) <= 1e-12 * msd_o and ov_g == ov_o, (fraction, cutoff)
    assert msd_g > 0.0


def test_trajectory_driver_writes_the_reference_layout(svm, tmp_path):
    netcdf = pytest.importorskip("scipy.io")
    out = svm.run_trajectory(N=120, maximumIterations=400, fIdx=0, temperature=0.01, dt=0.01, outdir=str(tmp_path),
                             seed=9)
    steps = [o[0] for o in out]
    assert steps[:6] == [1, 2, 3, 4, 5, 6] and steps[-1] == 398
    tag = "N120_p3.7800_T0.01000_kr1.000_fidx0"
    with netcdf.netcdf_file(str(tmp_path / f"cellPositions_{tag}.nc"), "r", mmap=False) as f:
        vec = np.array(f.variables["vector"][:])
        val = np.array(f.variables["value"][:])
    assert vec.shape == (len(out), 360) and np.allclose(val[:, 0], [o[1] for o in out])
    with netcdf.netcdf_file(str(tmp_path / f"msd_{tag}.nc"), "r", mmap=False) as f:
        msd = np.array(f.variables["vector"][:])
    assert np.allclose(msd[:, 0], np.array(steps) * 0.01)   # (time, MSD) records
    assert np.allclose(msd[:, 1], [o[2] for o in out]) and msd[-1, 1] > msd[0, 1] > 0.0
