"""The portable arccosine (csrc/svm_acos.h) on the CPU: its accuracy, its special values, and the
restatement's switch between it and the C library's acos."""
import math

import numpy as np
import pytest


def _samples():
    rng = np.random.default_rng(7)
    return np.concatenate([rng.uniform(-1, 1, 200000), 1 - rng.uniform(0, 1e-6, 20000),
                           -1 + rng.uniform(0, 1e-6, 20000), rng.uniform(-1e-3, 1e-3, 20000),
                           np.array([0.5, -0.5, np.nextafter(0.5, 1), np.nextafter(-0.5, -1), 0.0, -0.0,
                                     np.nextafter(1.0, 0), np.nextafter(-1.0, 0)])])


def test_portable_acos_special_values(oracle_mod):
    x = np.array([1.0, -1.0, 0.0, 1.0 + 2 ** -52, -1.0 - 2 ** -52, 2.0, np.inf, -np.inf, np.nan])
    y = oracle_mod.acos_portable(x)
    assert y[0] == 0.0 and y[1] == math.pi and y[2] == math.pi / 2
    assert np.all(np.isnan(y[3:]))


def test_portable_acos_within_two_ulp_of_libm(oracle_mod):
    x = _samples()
    y = oracle_mod.acos_portable(x)
    ref = np.arccos(x)
    ulps = np.abs(y - ref) / np.spacing(ref)
    assert ulps.max() <= 2.0, ulps.max()
    assert np.mean(y == ref) > 0.7


def test_portable_acos_against_high_precision(oracle_mod):
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    x = _samples()[::40]
    y = oracle_mod.acos_portable(x)
    worst = 0.0
    for xi, yi in zip(x, y):
        t = mp.acos(mp.mpf(float(xi)))
        worst = max(worst, float(abs(mp.mpf(float(yi)) - t) / np.spacing(float(t))))
    assert worst < 1.5, worst


def test_oracle_switch_changes_only_the_arccosine(oracle_mod):
    """The restatement's geometry with the portable acos stays close to the library one (areas and
    perimeters of the golden initial state), and the switch restores the library.  An area is
    sum(theta) - (n - 2) pi, about 200 times smaller than the angle sum at this cell size, so an ulp
    of one angle is ~1e-14 of the area."""
    from gpu_helpers import load_gold, oracle_model
    g = load_gold()
    om = oracle_model(oracle_mod, g)
    om.compute_geometry()
    ap_lib = om.area_perimeter()
    try:
        oracle_mod.set_portable_acos(True)
        om.compute_geometry()
        ap_port = om.area_perimeter()
    finally:
        oracle_mod.set_portable_acos(False)
    om.compute_geometry()
    assert np.array_equal(om.area_perimeter(), ap_lib)
    assert np.array_equal(ap_lib, g["init_ap"])
    assert np.max(np.abs(ap_port - ap_lib) / np.abs(ap_lib)) < 1e-12
