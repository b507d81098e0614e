"""The oracle's restatements of the rows built beside the step against fixtures the reference's own
classes made (tests/golden/make_golden_next.py): neighbour lists, the self-propelled and Vicsek
updaters over 100 steps, the dynamical observables and the save schedule, all bit for bit.  These
run wherever the oracle builds; the reference sources are needed only to regenerate the file."""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "next_rows.npz")


@pytest.fixture(scope="module")
def g():
    return np.load(GOLD)


@pytest.mark.parametrize("case,rng_,sub", [("box", 0.7, 2), ("model", 1.0, 1)])
def test_neighbor_lists(oracle_mod, g, case, rng_, sub):
    pts = g[f"nl_{case}_pts"]
    radius = 3.0 if case == "box" else float(g["nl_model_radius"])
    nm, npp, idx, vec, dist = oracle_mod.neighbor_list(pts, rng_, radius, sub)
    assert nm == int(g[f"nl_{case}_nmax"])
    assert np.array_equal(npp, g[f"nl_{case}_npp"])
    assert np.array_equal(idx, g[f"nl_{case}_idx"])
    assert np.array_equal(vec, g[f"nl_{case}_vec"])
    assert np.array_equal(dist, g[f"nl_{case}_dist"])


@pytest.mark.parametrize("kind", [0, 1])
def test_active_updaters(oracle_mod, g, kind):
    p = f"active{kind}_"
    m = oracle_mod.OracleModel(g[p + "pos0"], g[p + "rings"], g[p + "counts"], g[p + "vcells"], g[p + "vnbrs"],
                               float(g[p + "radius"]))
    m.set_preferred(1.0, 3.8)
    m.set_kr(1.0)
    m.set_t1_threshold(0.04)
    m.set_directors(g[p + "dir0"])
    noise = oracle_mod.OracleNoise(55)
    nv = g[p + "pos0"].shape[0]
    for _ in range(100):
        if kind == 0:
            m.spp_step_noise(noise.uniforms(nv, -0.5, 0.5), 0.01, 1.0, 0.3, 0.7)
        else:
            m.vicsek_step_noise(noise.uniforms(2 * nv, 0.0, 1.0), 0.01, 1.0, 0.3, 0.5, 0.7)
    assert np.array_equal(m.positions(), g[p + "pos"])
    assert np.array_equal(m.directors(), g[p + "dir"])


def test_dynamics_and_schedule(oracle_mod, g):
    for (f, c), want in zip(g["dyn_cases"], g["dyn_out"]):
        assert oracle_mod.dynamics(g["dyn_a"], g["dyn_b"], float(g["dyn_radius"]), f, c) == tuple(want)
    assert np.array_equal(oracle_mod.log_spaced(37, 0.05, 150), g["lsi_steps"])
