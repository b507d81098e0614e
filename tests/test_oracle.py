"""The CPU oracle pinned against the reference: golden fixtures made from the reference compiled
from its sources (tests/golden/make_golden.py), and, where oracle/_ref is built, the reference
itself on further configurations."""
import platform

import numpy as np
import pytest

GOLD = "tests/golden/brownian_n200.npz"
EXACT = platform.machine() in ("x86_64", "AMD64")  # fixtures were generated on x86-64


def close(a, b, rtol=1e-12, atol=1e-12):
    if EXACT:
        return np.array_equal(a, b)
    return np.allclose(a, b, rtol=rtol, atol=atol)


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def oracle_from(oracle_mod, g, prefix="init_"):
    m = oracle_mod.OracleModel(g[prefix + "pos"], g[prefix + "rings"], g[prefix + "counts"], g[prefix + "vcells"],
                               g[prefix + "vnbrs"], float(g["init_radius"]))
    N, SEED, BD_SEED, A0, P0, KR, T, MU, DT, T1 = g["params"]
    m.set_preferred(A0, P0)
    m.set_kr(KR)
    m.set_t1_threshold(T1)
    return m


def test_initial_geometry_and_forces(oracle_mod, gold):
    m = oracle_from(oracle_mod, gold)
    m.compute_forces()
    assert close(m.area_perimeter(), gold["init_ap"])
    assert close(m.cell_positions(), gold["init_cellpos"])
    assert close(m.forces(), gold["init_forces"])
    assert close(np.array(m.energy()), gold["init_energy"])


def test_brownian_trajectory_matches_reference(oracle_mod, gold):
    g = gold
    m = oracle_from(oracle_mod, g)
    N, SEED, BD_SEED, A0, P0, KR, T, MU, DT, T1 = g["params"]
    noise = oracle_mod.OracleNoise(int(BD_SEED))
    flips = []
    for step in range(1, 1001):
        m.brownian_step(noise, T, DT, MU)
        flips.extend((step, a, b) for a, b in m.flips())
        if step in (1, 10, 100, 1000):
            p = f"s{step}_"
            rings, counts = m.rings(16)
            assert np.array_equal(rings, g[p + "rings"]) and np.array_equal(counts, g[p + "counts"]), step
            assert np.array_equal(m.vertex_cells(), g[p + "vcells"]), step
            assert np.array_equal(m.vertex_neighbors(), g[p + "vnbrs"]), step
            assert close(m.positions(), g[p + "pos"]), step
            m.compute_geometry()
            assert close(m.area_perimeter(), g[p + "ap"]), step
            assert close(np.array(m.energy()), g[p + "energy"]), step
    assert np.array_equal(np.array(flips, dtype=np.int32).reshape(-1, 3), g["flips"])


def test_cell_list_matches_reference(oracle_mod, gold):
    g = gold
    R = float(g["init_radius"])
    cl = oracle_mod.oracle_cell_list(g["s1000_pos"], 1.0, R + 2.5)
    assert cl["nside"] == int(g["cl_nside"]) and cl["nmax"] == int(g["cl_nmax"])
    nz = np.nonzero(cl["counts"])[0]
    assert np.array_equal(nz, g["cl_bins"])
    assert np.array_equal(cl["counts"][nz], g["cl_counts"])
    assert np.array_equal(cl["idx"][nz], g["cl_slots"])
    assert cl["counts"].sum() == g["s1000_pos"].shape[0]


def test_fire_matches_reference(oracle_mod, gold):
    g = gold
    m = oracle_from(oracle_mod, g, "s1000_")
    m.set_restricted(True)
    fp = g["fire_params"]
    f = oracle_mod.OracleFire(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], int(fp[6]), fp[7], fp[8], 100)
    f.minimize(m, 0)
    assert close(m.positions(), g["fire100_pos"])
    assert close(np.array(f.state()["force_rms_over_n"]), g["fire100_force"])
    f2 = oracle_mod.OracleFire(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], int(fp[6]), fp[7], fp[8], int(fp[9]))
    m2 = oracle_from(oracle_mod, g, "s1000_")
    m2.set_restricted(True)
    f2.minimize(m2, 0)
    assert f2.state()["iterations"] == int(g["fire_iterations"])
    assert close(m2.positions(), g["fire_pos"])
    m2.compute_geometry()
    assert close(np.array(m2.energy()), g["fire_energy"])


def test_planted_mistake_is_caught(oracle_mod, gold):
    """A perturbed oracle state must fail the same comparison (the checker is not vacuous)."""
    g = gold
    m = oracle_from(oracle_mod, g)
    p = m.positions()
    t = np.cross(p[17], [0.0, 0.0, 1.0])
    p[17] += 1e-8 * t / np.linalg.norm(t)  # tangential: moves the vertex along the sphere
    m.set_positions(p)
    m.compute_forces()
    assert not np.allclose(m.forces(), g["init_forces"], rtol=1e-12, atol=1e-12)


# ---- against the reference itself (needs oracle/_ref, built here from the reference sources) ----
ref_only = pytest.mark.skipif("not __import__('oracle').ref_available()", reason="oracle/_ref not built")


@ref_only
@pytest.mark.parametrize("n,seed,p0,T,t1,steps", [(120, 7, 3.95, 0.05, 0.08, 300), (64, 3, 3.7, 0.02, 0.1, 300)])
def test_oracle_bit_exact_against_reference(oracle_mod, n, seed, p0, T, t1, steps):
    ref = oracle_mod.RefModel(n, seed, 1.0, p0, 1.0, t1)
    topo = ref.topology()
    m = oracle_mod.OracleModel(topo["pos"], topo["rings"], topo["counts"], topo["vcells"], topo["vnbrs"], topo["radius"])
    m.set_preferred(1.0, p0)
    m.set_t1_threshold(t1)
    ref.bd_setup(seed + 100, T, 0.01, 1.0)
    noise = oracle_mod.OracleNoise(seed + 100)
    nflips = 0
    for step in range(steps):
        ref.steps(1)
        m.brownian_step(noise, T, 0.01, 1.0)
        nflips += len(m.flips())
        assert np.array_equal(ref.positions(), m.positions()), step
    r1, c1 = ref.rings(32)
    r2, c2 = m.rings(32)
    assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
    assert np.array_equal(ref.area_perimeter(), m.area_perimeter())
    assert ref.energy() == m.energy()
    assert nflips > 0


@ref_only
def test_area_fallback_against_reference(oracle_mod):
    """A vertex pushed across its cell makes the angle-sum area wrong; both sides must take the
    triangle-fan fallback (sphericalVertexModel.cpp:304-310) and agree."""
    ref = oracle_mod.RefModel(80, 11, 1.0, 3.8, 1.0, 0.04)
    topo = ref.topology()
    p = topo["pos"].copy()
    v = 1
    nb = topo["vnbrs"][v]
    p[v] = p[v] + 2.5 * (p[nb[0]] - p[v])  # overshoot a neighbour: the rings fold over
    p[v] *= ref.radius / np.linalg.norm(p[v])
    ref.set_positions(p)
    ref.compute_geometry()
    m = oracle_mod.OracleModel(p, topo["rings"], topo["counts"], topo["vcells"], topo["vnbrs"], topo["radius"])
    m.compute_geometry()
    assert m.fallback_count() == 1 and abs(m.excess_area()) > 1e-6
    assert np.array_equal(ref.area_perimeter(), m.area_perimeter())
    ref.compute_forces()
    m.compute_forces()
    assert np.array_equal(ref.forces(), m.forces())


def test_vector_form_forces_match_reference(oracle_mod, gold):
    """The host FP64 vector-form force (the mixed-precision kernels' formulas) against the
    reference's closed-form forces on the golden N = 200 state and on an N = 2000 state after the
    stabilised preparation: agreement to rounding except where the reference's triangle-gradient
    formula loses digits on a nearly degenerate centroid-fan triangle, and there the vector form
    matches a central finite difference of the reference energy."""
    from gpu_helpers import vector_forces
    from curvedspacevertexmodel_gb300 import Topology, random_cell_centres

    g = gold
    m = oracle_from(oracle_mod, g)
    m.compute_forces()
    N, SEED, BD_SEED, A0, P0, KR, T, MU, DT, T1 = g["params"]
    pref = np.tile([A0, P0], (int(N), 1))
    rings, counts = m.rings(32)
    f = vector_forces(m.positions(), rings, counts, m.area_perimeter(), pref, m.cell_positions(),
                      float(g["init_radius"]), KR)
    fref = m.forces()
    err = np.linalg.norm(f - fref, axis=1) / np.max(np.linalg.norm(fref, axis=1))
    assert err.max() < 1e-9

    n = 2000
    topo = Topology(random_cell_centres(5, n))
    R = np.sqrt(n / (4 * np.pi))
    om = oracle_mod.OracleModel(topo.vertexPositions, topo.rings, topo.ringCounts, topo.vertexCells,
                                topo.vertexNeighbors, R)
    om.set_t1_threshold(0.04)
    noise = oracle_mod.OracleNoise(6)
    om.set_preferred(1.0, 1.0)
    for _ in range(100):
        om.brownian_step(noise, 0.0, 0.01)
    om.set_preferred(1.0, 3.8)
    for _ in range(300):
        om.brownian_step(noise, 0.01, 0.01)
    om.compute_forces()
    pos, fref = om.positions(), om.forces()
    rings, counts = om.rings(32)
    f = vector_forces(pos, rings, counts, om.area_perimeter(), np.tile([1.0, 3.8], (n, 1)), om.cell_positions(), R)
    fmax = np.max(np.linalg.norm(fref, axis=1))
    err = np.linalg.norm(f - fref, axis=1) / fmax
    assert np.quantile(err, 0.99) < 1e-9
    assert err.max() < 1e-4
    w = int(np.argmax(err))
    p = pos[w]
    a = p / np.linalg.norm(p)
    e1 = np.cross(a, [0.0, 0.0, 1.0])
    e1 /= np.linalg.norm(e1)
    for e in (e1, np.cross(a, e1)):
        en = []
        for sgn in (1.0, -1.0):
            q = pos.copy()
            q[w] = p + sgn * 1e-6 * e
            q[w] *= R / np.linalg.norm(q[w])
            om.set_positions(q)
            om.compute_geometry()
            en.append(om.energy())
        fd = -(en[0] - en[1]) / 2e-6
        assert abs(f[w] @ e - fd) <= abs(fref[w] @ e - fd) + 1e-7 * fmax
    om.set_positions(pos)


@ref_only
def test_neighbor_list_against_reference(oracle_mod):
    """orc_neighbor_list against the reference's neighborList::computeCPU: the model's vertices
    with the model's parameters (range 1, radius R + 2.5), and points filling a periodic box so
    that minimum images cross its faces; Nmax grows from 4 through the recompute loop."""
    ref = oracle_mod.RefModel(400, 11)
    R = ref.radius
    cases = [(ref.positions(), 1.0, R + 2.5, 1), (ref.positions(), 1.0, R + 2.5, 2)]
    rng = np.random.default_rng(3)
    box = rng.uniform(-4.0, 4.0 * (1 - 1e-12), (1500, 3))
    box[:30, 0] = 4.0 * (1 - 1e-9)
    box[30:60, 0] = -4.0
    cases += [(box, 0.7, 4.0, 1), (box, 0.7, 4.0, 2), (box, 1.3, 4.0, 3)]
    for pts, rng_, radius, sub in cases:
        a = oracle_mod.neighbor_list(pts, rng_, radius, sub)
        b = oracle_mod.neighbor_list(pts, rng_, radius, sub, reference=True)
        assert a[0] == b[0] and a[0] > 4, (rng_, sub)
        for x, y in zip(a[1:], b[1:]):
            assert np.array_equal(x, y), (rng_, sub)
    # edge cases: one point, a close pair, a pair across the periodic faces, a pair exactly at range
    small = [np.array([[0.5, -0.25, 1.0]]), np.array([[0.1, 0.2, 0.3], [0.15, 0.2, 0.3]]),
             np.array([[3.99, 0.0, 0.0], [-3.99, 0.0, 0.0]]), np.array([[0.0, 0.0, 0.0], [0.5, 0.0, 0.0]])]
    for pts in small:
        for sub in (1, 2):
            a = oracle_mod.neighbor_list(pts, 0.5, 4.0, sub)
            b = oracle_mod.neighbor_list(pts, 0.5, 4.0, sub, reference=True)
            assert a[0] == b[0] == 4
            for x, y in zip(a[1:], b[1:]):
                assert np.array_equal(x, y), pts


@ref_only
@pytest.mark.parametrize("kind", [0, 1])
def test_active_updaters_against_reference(oracle_mod, kind):
    """orc_spp_step_noise (kind 0) and orc_vicsek_step_noise (kind 1) against the reference's
    sphericalSelfPropelledParticle and sphericalVectorialVicsek driving its vertex model: the
    oracle fed the same mt19937 uniforms the reference's updater draws, 300 steps with T1 flips,
    positions and directors equal bit for bit after every step."""
    n, seed = 120, 7
    ref = oracle_mod.RefModel(n, seed, 1.0, 3.8, 1.0, 0.04)
    topo = ref.topology()
    m = oracle_mod.OracleModel(topo["pos"], topo["rings"], topo["counts"], topo["vcells"], topo["vnbrs"], topo["radius"])
    m.set_preferred(1.0, 3.8)
    m.set_t1_threshold(0.04)
    d0 = ref.directors()  # the reference's come from a random_device-seeded source: start from them
    p = ref.positions()
    assert np.abs(np.sum(d0 * p, axis=1)).max() < 1e-12 and np.abs(np.linalg.norm(d0, axis=1) - 1).max() < 1e-14
    m.set_directors(d0)
    dt, mu, v0, eta, tau = 0.01, 1.0, 0.3, 0.5, 0.7
    ref.active_setup(kind, 55, dt, mu, v0, eta, tau)
    draws = oracle_mod.OracleNoise(55)
    nv = ref.nVertices
    flips = 0
    for step in range(300):
        ref.steps(1)
        if kind == 0:
            m.spp_step_noise(draws.uniforms(nv, -0.5, 0.5), dt, mu, v0, tau)
        else:
            m.vicsek_step_noise(draws.uniforms(2 * nv, 0.0, 1.0), dt, mu, v0, eta, tau)
        flips += len(m.flips())
        assert np.array_equal(ref.positions(), m.positions()), step
        assert np.array_equal(ref.directors(), m.directors()), step
    assert flips > 0


@ref_only
def test_dynamics_against_reference(oracle_mod):
    """orc_dynamics against the reference's dynamicalFeatures (MSD with NaN distances skipped,
    overlap below a cutoff, the first floor(N f) points): equal bit for bit, including a point
    whose geodesic distance is NaN (acos of a rounding above 1)."""
    rng = np.random.default_rng(8)
    n, R = 3000, 15.45
    a = rng.normal(size=(n, 3))
    a *= R / np.linalg.norm(a, axis=1, keepdims=True)
    b = a + rng.normal(scale=0.3, size=(n, 3))
    b *= R / np.linalg.norm(b, axis=1, keepdims=True)
    b[5] = a[5] * (1 + 1e-16)   # a rounding-level copy
    for fraction in (1.0, 0.37, 0.999):
        for cutoff in (0.5, 0.2, 2.0):
            o = oracle_mod.dynamics(a, b, R, fraction, cutoff)
            r = oracle_mod.dynamics(a, b, R, fraction, cutoff, reference=True)
            assert o == r, (fraction, cutoff)


@ref_only
@pytest.mark.parametrize("first,exponent,count", [(0, 0.05, 150), (0, 0.1, 80), (37, 0.05, 150), (1000, 0.02, 150)])
def test_log_spaced_against_reference(oracle_mod, first, exponent, count):
    """orc_log_spaced against the reference's logSpacedIntegers, schedule for schedule."""
    assert np.array_equal(oracle_mod.log_spaced(first, exponent, count),
                          oracle_mod.log_spaced(first, exponent, count, reference=True))


def test_reference_trajectory_spread_under_faithful_acos(oracle_mod):
    """The reference's N = 200 trajectory (the restatement, bit-exact with the reference build)
    under twelve other faithful arccosines: one step stays at the last bit, and the largest
    deviations from the golden fixture after 10, 100 and 1000 steps are ACOS_SPREAD, which sets the
    GPU trajectory tolerances (gpu_helpers.traj_tol)."""
    from gpu_helpers import ACOS_SPREAD, ACOS_SPREAD_VARIANTS, load_gold, oracle_model, params, trajectory_deviation
    g = load_gold()
    p = params(g)
    R = float(g["init_radius"])
    env = {s: dict(pos=0.0, ap=0.0, energy=0.0) for s in ACOS_SPREAD}
    try:
        for mode, seed in ACOS_SPREAD_VARIANTS:
            oracle_mod.set_acos_mode(mode, seed)
            om = oracle_model(oracle_mod, g)
            noise = oracle_mod.OracleNoise(p["bd_seed"])
            for step in range(1, 1001):
                om.brownian_step_noise(noise.normals(3 * 396), p["T"], p["dt"], p["mu"])
                if step == 1:
                    assert np.max(np.abs(om.positions() - g["s1_pos"])) / R < 1e-15
                if step in env:
                    om.compute_geometry()
                    d = trajectory_deviation(om.positions(), om.area_perimeter(), om.energy(), g, step)
                    for q in d:
                        env[step][q] = max(env[step][q], d[q])
    finally:
        oracle_mod.set_acos_mode(0, 0)
    for step, d in env.items():
        for q, v in d.items():
            assert abs(v / ACOS_SPREAD[step][q] - 1) < 1e-3, (step, q, v)
