"""The CPU reference of the warm-start network (oracle/mlp.py) pinned by central finite
differences of its own loss, and its BF16 rounding by known values."""
import numpy as np

import mlp


def test_backprop_matches_finite_differences():
    rng = np.random.default_rng(0)
    w = rng.normal(0, 0.3, mlp.N_PARAMS)
    X = rng.normal(0, 1, (40, mlp.N_IN))
    T = rng.normal(0, 1, (40, mlp.N_OUT))
    loss, g = mlp.loss_and_grad(w, X, T)
    idx = np.concatenate([rng.choice(mlp.N_PARAMS, 60, replace=False),
                          [mlp.O_B1, mlp.O_B2, mlp.O_B3, mlp.N_PARAMS - 1]])
    for i in idx:
        h = 1e-6
        wp, wm = w.copy(), w.copy()
        wp[i] += h
        wm[i] -= h
        fd = (mlp.loss_and_grad(wp, X, T)[0] - mlp.loss_and_grad(wm, X, T)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i]))


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 2 ** -7, 1.0 + 3 * 2 ** -8, -2.5, 3.1415926], dtype=np.float32)
    r = mlp.bf16(v)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: to even (1); 1 + 3 2^-8 ties up to 1 + 2^-6
    assert list(r[:5]) == [1.0, 1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -6, -2.5]
    assert abs(r[5] - 3.140625) < 1e-12


def test_warm_start_fallback_decision_takes_nan():
    """A diverged warm start (NaN energy or NaN force) falls back to plain FIRE, as do a raised
    energy and a missed force tolerance; a warm start that lowered the energy and converged does not."""
    from curvedspacevertexmodel_gb300.warm_start import fallback_reason
    nan = float("nan")
    assert fallback_reason(10.0, nan) == "warm start raised the energy"
    assert fallback_reason(10.0, 11.0) == "warm start raised the energy"
    assert fallback_reason(10.0, 9.0) is None
    assert fallback_reason(10.0, 9.0, nan) == "iteration budget exceeded"
    assert fallback_reason(10.0, 9.0, 2e-9) == "iteration budget exceeded"
    assert fallback_reason(10.0, 9.0, 5e-10) is None
