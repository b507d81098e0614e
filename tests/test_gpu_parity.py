"""Parity of the GPU path (libsvm through its C ABI) with the CPU oracle and the reference's golden
fixtures.  FP64 tolerances are stated per test; connectivity and the T1 flip set are compared
exactly."""
import numpy as np
import pytest

from gpu_helpers import gpu_model, load_gold, oracle_model, params, rel_err, same_rings, stabilised, traj_tol

pytestmark = pytest.mark.gpu

# Trajectories.  One step agrees with the CPU to ~1e-15 (RTOL_STEP).  Over many noisy steps the
# reference's closed-form gradients divide by 1 - s^2 ~ theta^2 for collapsing edges (theta ~ 1e-4
# rad before a T1), amplifying last-bit differences of acos by up to ~1e8.  CUDA's acos and glibc's
# differ in the last bit (neither is correctly rounded: glibc's misrounds ~10% of arguments, by up to
# 0.81 ulp), so no device acos reproduces glibc's bits and the trajectories separate: after 1000
# steps of the N=200 configuration by 8e-10 (positions), 3e-10 (areas/perimeters), 3e-11 (energy),
# with the T1 flip set identical at every step.  The reference itself moves as far when only the
# last bits of its acos change (gpu_helpers.ACOS_SPREAD: the largest deviation over twelve faithful
# arccosines), so the tolerance after 10, 100 and 1000 steps is twice that spread (traj_tol); with
# one arccosine on both sides the GPU and CPU paths are equal bit for bit
# (test_gpu_portable_acos.py).
RTOL_STEP = 1e-12
# One evaluation of the geometry differs from the CPU only by rounding (acos, FMA).
RTOL_EVAL = 1e-12
# Forces are closed forms with 1 - s^2 (s = cosine of a short arc) in their denominators; their
# conditioning turns last-bit differences into ~1e-12 relative differences of single forces.
RTOL_FORCE = 1e-11


@pytest.fixture(scope="module")
def svm(svm_lib):
    if svm_lib.device_count() < 1:
        pytest.fail("no CUDA device: the GPU tests need a GB300")
    return svm_lib


@pytest.fixture(scope="module")
def gold():
    return load_gold()


def test_geometry_forces_energy_match_golden(svm, gold):
    m = gpu_model(svm, gold)
    m.computeForces()
    assert rel_err(m.areaPerimeter(), gold["init_ap"]) < RTOL_EVAL
    assert rel_err(m.cellPositions(), gold["init_cellpos"]) < RTOL_EVAL
    assert rel_err(m.returnForces(), gold["init_forces"]) < RTOL_FORCE
    assert abs(m.computeEnergy() - float(gold["init_energy"])) / float(gold["init_energy"]) < RTOL_EVAL
    assert m.deviceStatus() == 0


def test_brownian_1000_steps_match_oracle_and_golden(svm, gold, oracle_mod):
    """Config 1: N=200, T=0.01, dt=0.01, T1 threshold 0.04, the reference's mt19937 noise stream
    injected into both sides: the ordered T1 flip list identical at every step, connectivity
    identical, positions/areas/perimeters/energy within RTOL_STEP after one step and within
    traj_tol (twice the reference's own spread under faithful changes of acos) after 10, 100 and
    1000 steps."""
    p = params(gold)
    gm = gpu_model(svm, gold)
    om = oracle_model(oracle_mod, gold)
    bd = svm.brownianDynamics()
    bd.setModel(gm)
    bd.setT(p["T"])
    bd.setDeltaT(p["dt"])
    bd.mu = p["mu"]
    noise = oracle_mod.OracleNoise(p["bd_seed"])
    nv = gm.nVertices
    total_flips = 0
    for step in range(1, 1001):
        xi = noise.normals(3 * nv)
        bd.injectNoise(xi)
        bd.integrateEquationOfMotion()
        om.brownian_step_noise(xi, p["T"], p["dt"], p["mu"])
        f_gpu = gm.takeFlips()
        f_orc = om.flips()
        assert np.array_equal(f_gpu, f_orc), f"T1 flips differ at step {step}: {f_gpu} vs {f_orc}"
        total_flips += len(f_orc)
        if step in (1, 10, 100, 1000):
            tol = {q: RTOL_STEP if step == 1 else traj_tol(step, q) for q in ("pos", "ap", "energy")}
            assert same_rings(gm, om), step
            assert np.array_equal(gm.vertexCellNeighbors(), om.vertex_cells()), step
            assert np.array_equal(gm.vertexNeighbors(), om.vertex_neighbors()), step
            R = float(gold["init_radius"])
            assert rel_err(gm.returnPositions(), om.positions(), R) < tol["pos"], step
            gm.computeGeometry()
            om.compute_geometry()
            ap_g, ap_o = gm.areaPerimeter(), om.area_perimeter()
            assert np.max(np.abs(ap_g - ap_o) / np.abs(ap_o)) < tol["ap"], step
            e_g, e_o = gm.computeEnergy(), om.energy()
            assert abs(e_g - e_o) / e_o < tol["energy"], step
            # and the fixtures made from the reference itself
            g = f"s{step}_"
            assert rel_err(gm.returnPositions(), gold[g + "pos"], R) < tol["pos"], step
            assert abs(e_g - float(gold[g + "energy"])) / float(gold[g + "energy"]) < tol["energy"], step
    assert total_flips == len(gold["flips"]) and total_flips > 100
    assert gm.deviceStatus() == 0


def test_forced_t1_matches_oracle(svm, gold, oracle_mod):
    """A hand-shortened edge: enforceTopology flips it exactly as the CPU does."""
    g = gold
    gm = gpu_model(svm, g)
    om = oracle_model(oracle_mod, g)
    pos = g["init_pos"].copy()
    nbrs = g["init_vnbrs"]
    edits = []
    for v in (3, 40, 101, 250):
        u = int(nbrs[v][0])
        pos[u] = pos[v] + 0.02 * (pos[u] - pos[v])
        pos[u] *= float(g["init_radius"]) / np.linalg.norm(pos[u])
        edits.append((min(u, v), max(u, v)))
    gm.setPositions(pos)
    om.set_positions(pos)
    gm.enforceTopology()
    om.lib.orc_enforce_topology(om.h)
    fg, fo = gm.takeFlips(), om.flips()
    assert len(fo) >= 3 and np.array_equal(fg, fo)
    assert same_rings(gm, om)
    assert np.array_equal(gm.vertexCellNeighbors(), om.vertex_cells())
    assert np.array_equal(gm.vertexNeighbors(), om.vertex_neighbors())
    assert rel_err(gm.returnPositions(), om.positions(), float(g["init_radius"])) < 1e-14
    gm.computeForces()
    om.compute_forces()
    assert rel_err(gm.returnForces(), om.forces()) < RTOL_FORCE


def test_cell_list_matches_golden(svm, gold):
    import ctypes as C
    from curvedspacevertexmodel_gb300 import _lib
    gm = gpu_model(svm, gold, "s1000_")
    R = float(gold["init_radius"])
    h = C.c_void_p()
    _lib.call("svm_cell_list_create", 1.0, R + 2.5, gm.nVertices, 16, None, C.byref(h))
    try:
        _lib.call("svm_cell_list_compute_model", h, gm.handle)
        nside, nmax = C.c_int(), C.c_int()
        _lib.call("svm_cell_list_get", h, C.byref(nside), C.byref(nmax), None, None, 0)
        total = nside.value ** 3
        counts = np.empty(total, dtype=np.uint32)
        slots = np.empty(total * nmax.value, dtype=np.int32)
        _lib.call("svm_cell_list_get", h, C.byref(nside), C.byref(nmax), counts, slots, slots.size)
    finally:
        _lib.lib().svm_cell_list_destroy(h)
    assert nside.value == int(gold["cl_nside"]) and nmax.value == int(gold["cl_nmax"])
    nz = np.nonzero(counts)[0]
    assert np.array_equal(nz, gold["cl_bins"])
    assert np.array_equal(counts[nz], gold["cl_counts"])
    assert np.array_equal(slots.reshape(total, -1)[nz], gold["cl_slots"])


def test_cell_list_large_matches_oracle(svm, oracle_mod):
    import ctypes as C
    from curvedspacevertexmodel_gb300 import _lib
    n = 20000
    m = svm.sphericalVertexModel(n, svm.noiseSource())
    R = m.radius
    pts = m.returnPositions()
    ref = oracle_mod.oracle_cell_list(pts, 1.0, R + 2.5)
    h = C.c_void_p()
    _lib.call("svm_cell_list_create", 1.0, R + 2.5, m.nVertices, 16, None, C.byref(h))
    try:
        for _ in range(2):  # the second call exercises the incremental clear
            _lib.call("svm_cell_list_compute_model", h, m.handle)
        nside, nmax = C.c_int(), C.c_int()
        _lib.call("svm_cell_list_get", h, C.byref(nside), C.byref(nmax), None, None, 0)
        total = nside.value ** 3
        counts = np.empty(total, dtype=np.uint32)
        slots = np.empty(total * nmax.value, dtype=np.int32)
        _lib.call("svm_cell_list_get", h, C.byref(nside), C.byref(nmax), counts, slots, slots.size)
        bins = np.empty(m.nVertices, dtype=np.int32)
        _lib.call("svm_cell_list_bins", h, bins)
    finally:
        _lib.lib().svm_cell_list_destroy(h)
    assert nmax.value == ref["nmax"]
    assert np.array_equal(bins, ref["bins"])
    assert np.array_equal(counts, ref["counts"])
    assert np.array_equal(slots.reshape(total, -1), ref["idx"])


def test_fire_matches_oracle_and_golden(svm, gold, oracle_mod):
    """FIRE from the Brownian snapshot (T1 off): 100 iterations close to the oracle, and the full
    quench reaching the reference's final energy."""
    g = gold
    fp = g["fire_params"]
    gm = gpu_model(svm, g, "s1000_")
    gm.restrictedMotion = True
    fire = svm.energyMinimizerFIRE(gm)
    fire.setFIREParameters(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], int(fp[6]), fp[7], fp[8])
    fire.setMaximumIterations(100)
    fire.minimize()
    R = float(g["init_radius"])
    om = oracle_model(oracle_mod, g, "s1000_")
    om.set_restricted(True)
    of = oracle_mod.OracleFire(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], int(fp[6]), fp[7], fp[8], 100)
    of.minimize(om, 0)
    assert fire.getCurrentIterations() == 100
    assert rel_err(gm.returnPositions(), om.positions(), R) < 1e-10
    assert rel_err(gm.returnPositions(), g["fire100_pos"], R) < 1e-10
    st, ost = fire.state(), of.state()
    assert abs(st["dt"] - ost["dt"]) < 1e-12 and abs(st["alpha"] - ost["alpha"]) < 1e-12
    # the full quench
    fire.setMaximumIterations(int(fp[9]))
    gm2 = gpu_model(svm, g, "s1000_")
    gm2.restrictedMotion = True
    fire2 = svm.energyMinimizerFIRE(gm2)
    fire2.setFIREParameters(fp[0], fp[1], fp[2], fp[3], fp[4], fp[5], int(fp[6]), fp[7], fp[8])
    fire2.setMaximumIterations(int(fp[9]))
    fire2.minimize()
    gm2.computeGeometry()
    e = gm2.computeEnergy()
    assert abs(e - float(g["fire_energy"])) / float(g["fire_energy"]) < 1e-8


def test_graph_run_equals_step_loop(svm, gold):
    """svm_brownian_run (captured graph) reproduces svm_brownian_step bit for bit."""
    a = gpu_model(svm, gold)
    b = gpu_model(svm, gold)
    for m in (a, b):
        m.setPreferredParameters(1.0, 3.8)
    bda, bdb = svm.brownianDynamics(), svm.brownianDynamics()
    for bd, m in ((bda, a), (bdb, b)):
        bd.setModel(m)
        bd.setT(0.01)
        bd.noise.setReproducibleSeed(77)
    for _ in range(37):
        bda.integrateEquationOfMotion()
    bdb.run(37)
    assert np.array_equal(a.returnPositions(), b.returnPositions())
    assert np.array_equal(a.vertexNeighbors(), b.vertexNeighbors())
    r1, c1 = a.rings()
    r2, c2 = b.rings()
    assert np.array_equal(r1, r2) and np.array_equal(c1, c2)


def test_philox_noise_statistics(svm):
    """Brownian displacements with negligible forces over four steps: the tangential components are
    standard normals times sqrt(2 dt mu T) (variance, mean, kurtosis, two- and three-sigma tail
    fractions), as the in-kernel Philox + ziggurat sampler must give."""
    n = 20000
    m = svm.sphericalVertexModel(n, svm.noiseSource())
    m.setScalarModelParameter(0.0)
    m.setPreferredParameters(1.0, 0.0)  # forces ~ 2 P dP are O(10); T large makes them negligible
    m.restrictedMotion = True
    bd = svm.brownianDynamics()
    bd.setModel(m)
    T, dt = 1e6, 1e-8
    bd.setT(T)
    bd.setDeltaT(dt)
    z = []
    for _ in range(4):
        p0 = m.returnPositions()
        bd.integrateEquationOfMotion()
        d = m.returnPositions() - p0
        nrm = p0 / np.linalg.norm(p0, axis=1, keepdims=True)
        ref = np.where(np.abs(nrm[:, 2:3]) < 0.9, np.array([[0.0, 0.0, 1.0]]), np.array([[1.0, 0.0, 0.0]]))
        e1 = np.cross(nrm, ref)
        e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
        e2 = np.cross(nrm, e1)
        z.append(np.sum(d * e1, axis=1))
        z.append(np.sum(d * e2, axis=1))
    z = np.concatenate(z) / np.sqrt(2 * dt * T)
    k = z.size  # 320k samples
    assert abs(np.mean(z * z) - 1.0) < 0.01
    assert abs(np.mean(z)) < 5.0 / np.sqrt(k)
    assert abs(np.mean(z ** 4) / np.mean(z * z) ** 2 - 3.0) < 0.05
    assert abs(np.mean(np.abs(z) > 2.0) - 0.0455003) < 0.002
    assert abs(np.mean(np.abs(z) > 3.0) - 0.0026998) < 0.0005


def test_large_sphere_invariants(svm):
    """Size-independent properties at N = 20k after the stabilised preparation and 200 noisy steps
    with T1: total area 4 pi R^2, tangential forces, trivalent connectivity, rings consistent with
    the vertex lists, a physical energy per cell."""
    n = 20000
    m, bd = stabilised(svm, n)
    m.computeForces()
    ap = m.areaPerimeter()
    R = m.radius
    assert abs(ap[:, 0].sum() - 4 * np.pi * R * R) / (4 * np.pi * R * R) < 1e-9
    p, f = m.returnPositions(), m.returnForces()
    radial = np.abs(np.sum(p * f, axis=1)) / R
    assert np.max(radial) < 1e-9 * max(1.0, np.max(np.abs(f)))
    rings, counts = m.rings()
    vc = m.vertexCellNeighbors()
    assert counts.sum() == 3 * m.nVertices
    for c in range(0, n, 97):
        for v in rings[c, : counts[c]]:
            assert c in vc[v]
    assert 0 < m.computeEnergy() / n < 0.2
    assert m.deviceStatus() == 0


def test_area_fallback_matches_oracle(svm, oracle_mod):
    """A vertex pushed across its cell folds the ring: the total-area check fails and the areas
    come from the triangle-fan fallback (sphericalVertexModel.cpp:162-207, 304-310) on both sides."""
    pts = svm.random_cell_centres(11, 80)
    topo = svm.Topology(pts)
    R = np.sqrt(80 / (4 * np.pi))
    p = topo.vertexPositions.copy()
    nb = topo.vertexNeighbors[1]
    p[1] = p[1] + 2.5 * (p[nb[0]] - p[1])
    p[1] *= R / np.linalg.norm(p[1])
    gm = svm.sphericalVertexModel(80, topology=topo, radius=R)
    gm.setPositions(p)
    gm.computeForces()
    om = oracle_mod.OracleModel(p, topo.rings, topo.ringCounts, topo.vertexCells, topo.vertexNeighbors, R)
    om.compute_forces()
    total, excess, taken = gm.areaCheck()
    assert taken and om.fallback_count() == 1
    assert gm.fallbackCount() >= 1 and gm.fallbackCount() == 0  # counted, then cleared
    assert abs(excess - om.excess_area()) < 1e-9 * abs(om.excess_area())
    assert rel_err(gm.areaPerimeter(), om.area_perimeter()) < 1e-12
    assert rel_err(gm.returnForces(), om.forces()) < RTOL_FORCE


@pytest.mark.parametrize("blocks", [1, 4, 64])
def test_mass_t1_matches_oracle(svm, oracle_mod, blocks):
    """Hundreds of shortened edges, many sharing vertices and cells, in one enforceTopology pass:
    the parallel pass must give the flips, connectivity and positions of the CPU's sequential loop,
    in one block and spread over a cooperative grid."""
    n = 2000
    pts = svm.random_cell_centres(17, n)
    topo = svm.Topology(pts)
    R = np.sqrt(n / (4 * np.pi))
    rng = np.random.default_rng(3)
    pos = topo.vertexPositions.copy()
    for v in rng.choice(topo.nVertices, 600, replace=False):
        u = int(topo.vertexNeighbors[v][rng.integers(3)])
        pos[u] = pos[v] + rng.uniform(0.01, 0.05) * (pos[u] - pos[v])
        pos[u] *= R / np.linalg.norm(pos[u])
    gm = svm.sphericalVertexModel(n, topology=topo, radius=R)
    gm.setT1Threshold(0.04)
    gm.setT1Blocks(blocks)
    gm.setPositions(pos)
    om = oracle_mod.OracleModel(pos, topo.rings, topo.ringCounts, topo.vertexCells, topo.vertexNeighbors, R)
    om.set_t1_threshold(0.04)
    gm.enforceTopology()
    om.lib.orc_enforce_topology(om.h)
    fg, fo = gm.takeFlips(), om.flips()
    assert len(fo) > 100
    assert np.array_equal(fg, fo)
    assert same_rings(gm, om, 32)
    assert np.array_equal(gm.vertexCellNeighbors(), om.vertex_cells())
    assert np.array_equal(gm.vertexNeighbors(), om.vertex_neighbors())
    assert rel_err(gm.returnPositions(), om.positions(), R) < 1e-14
    assert gm.deviceStatus() == 0


def test_t1_trajectory_n20k_matches_oracle(svm, oracle_mod):
    """N = 20k from the stabilised preparation: 30 Brownian steps with the reference's noise stream
    on both sides, the oracle restarted from the device's state before every step; the T1 flips
    (CPU order), the connectivity and the positions agree after every step.  (Run freely, the two
    drift apart at the last-bit level through acos, and after some steps an edge within rounding of
    the threshold is decided differently; restarting each step keeps every decision comparable.)"""
    n = 20000
    m, _ = stabilised(svm, n, seed=8, stab=100, steps=100)
    R = m.radius
    bd = svm.brownianDynamics()
    bd.setModel(m)
    bd.setT(0.01)
    noise = oracle_mod.OracleNoise(99)
    m.takeFlips(1 << 20)  # drop the preparation's flips
    total = 0
    for step in range(30):
        rings, counts = m.rings(32)
        om = oracle_mod.OracleModel(m.returnPositions(), rings, counts, m.vertexCellNeighbors(), m.vertexNeighbors(), R)
        om.set_preferred(1.0, 3.8)
        om.set_t1_threshold(0.04)
        xi = noise.normals(3 * m.nVertices)
        bd.injectNoise(xi)
        bd.integrateEquationOfMotion()
        om.brownian_step_noise(xi, 0.01, 0.01, 1.0)
        fg, fo = m.takeFlips(1 << 20), om.flips()
        assert np.array_equal(fg, fo), step
        assert same_rings(m, om, 32), step
        assert np.array_equal(m.vertexNeighbors(), om.vertex_neighbors()), step
        # one step from the same state: the reference's 1/theta^2-conditioned gradients at
        # collapsing edges amplify acos's last-bit differences, the bulk stays at the last bit
        d = np.abs(m.returnPositions() - om.positions()).max(axis=1) / R
        assert np.quantile(d, 0.5) < 1e-13 and d.max() < 1e-6, (step, np.quantile(d, 0.5), d.max())
        total += len(fo)
    assert total > 30


def test_fire_outliving_its_model(svm, gold):
    """A FIRE minimizer whose model was destroyed first reports an argument error instead of
    touching the freed model; destroying it afterwards is safe."""
    m = gpu_model(svm, gold)
    fire = svm.energyMinimizerFIRE(m)
    fire.setMaximumIterations(5)
    fire.minimize()
    m.close()
    with pytest.raises(svm.SVMError):
        fire.minimize()
    del fire


def test_host_io_step_equals_the_call_sequence(svm, gold):
    """svm_brownian_step_io (positions in, step, energy and positions out, one synchronisation)
    gives bit for bit what set_positions + brownian_step + compute_energy + get_positions give."""
    import ctypes as C
    from curvedspacevertexmodel_gb300 import _lib
    a, b = gpu_model(svm, gold), gpu_model(svm, gold)
    pos = a.returnPositions()
    pos[0] *= 1.0 + 1e-9
    out = np.empty(3 * a.nVertices)
    e_io = C.c_double()
    _lib.call("svm_brownian_step_io", a.handle, 0.01, 0.01, 1.0, 99, np.ascontiguousarray(pos).reshape(-1), out,
              C.byref(e_io))
    b.setPositions(pos)
    _lib.call("svm_brownian_step", b.handle, 0.01, 0.01, 1.0, _lib.SVM_NOISE_PHILOX, None, 99)
    e_seq = b.computeEnergy()
    assert np.array_equal(out.reshape(-1, 3), b.returnPositions())
    assert e_io.value == e_seq


@pytest.mark.parametrize("pinned", [False, True])
def test_host_io_steps_chained_with_flips(svm, pinned):
    """Chained svm_brownian_step_io calls (each step's positions fed back in) follow the
    device-resident step loop bit for bit over steps with T1 flips: positions, topology, flip
    count and energies.  (The host-io step defers the moved state's corners to the next step;
    with page-locked buffers it runs as a replayed graph, re-captured when the seed changes.)"""
    import ctypes as C
    import torch
    from curvedspacevertexmodel_gb300 import _lib
    a, _ = stabilised(svm, 3000, seed=11, stab=40, steps=60)
    b, _ = stabilised(svm, 3000, seed=11, stab=40, steps=60)
    for m in (a, b):
        m.setT1Threshold(0.08)   # flips every step
    a.t1Stats(), b.t1Stats()   # counters restart
    n = 3 * a.nVertices
    if pinned:
        pos = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
        out = torch.empty(n, dtype=torch.float64).pin_memory().numpy()
    else:
        pos, out = np.empty(n), np.empty(n)
    pos[:] = a.returnPositions().reshape(-1)
    e_io = C.c_double()
    for k in range(25):
        seed = 4242 + k // 10   # a new seed (a new capture) every ten steps
        _lib.call("svm_brownian_step_io", a.handle, 0.05, 0.01, 1.0, seed, pos, out, C.byref(e_io))
        _lib.call("svm_brownian_step", b.handle, 0.05, 0.01, 1.0, _lib.SVM_NOISE_PHILOX, None, seed)
        # both report the energy of the state the step started from (the areas of its geometry)
        assert e_io.value == b.computeEnergy(), k
        pos, out = out, pos
    assert np.array_equal(pos.reshape(-1, 3), b.returnPositions())
    assert np.array_equal(a.vertexNeighbors(), b.vertexNeighbors())
    r1, c1 = a.rings()
    r2, c2 = b.rings()
    assert np.array_equal(r1, r2) and np.array_equal(c1, c2)
    fa, fb = a.t1Stats()["flips"], b.t1Stats()["flips"]
    assert fa == fb and fa > 25
    assert a.computeEnergy() == b.computeEnergy()


def test_t1_pass_block_count_does_not_change_the_run(svm):
    """N = 20k (whose automatic T1 pass is a cooperative grid) against the same run with the pass
    in one block and in 152 blocks: positions, connectivity and flips bit for bit over 40 steps at
    a raised threshold (several hundred flips a step)."""
    runs = []
    for blocks in (1, 0, 152):
        m, bd = stabilised(svm, 20000, seed=21, stab=60, steps=40)
        m.setT1Threshold(0.06)
        m.setT1Blocks(blocks)
        m.takeFlips(1 << 20)
        bd.noise.setReproducibleSeed(5)
        bd.run(20)
        for _ in range(20):
            bd.integrateEquationOfMotion()
        runs.append((m.returnPositions(), m.vertexNeighbors(), m.rings(32), m.takeFlips(1 << 20),
                     m.deviceStatus()))
    ref = runs[0]
    assert len(ref[3]) > 1000
    for r in runs[1:]:
        assert np.array_equal(r[0], ref[0])
        assert np.array_equal(r[1], ref[1])
        assert np.array_equal(r[2][0], ref[2][0]) and np.array_equal(r[2][1], ref[2][1])
        assert np.array_equal(r[3], ref[3])
        assert r[4] == 0


def test_exhausted_t1_barrier_wait_is_reported(svm, gold):
    """A cooperative T1 pass whose grid-barrier waits may poll only once: the blocks that arrive
    first give up, the kernel ends instead of hanging, and SVM_DEV_T1_TIMEOUT comes back; the
    device stays usable (a fresh model steps and reads back normally)."""
    from curvedspacevertexmodel_gb300 import _lib
    m, bd = stabilised(svm, 20000, seed=21, stab=20, steps=20)
    m.setT1Threshold(0.08)   # flagged edges every step, so the cooperative pass runs
    m.setT1Blocks(64)
    m.setT1WaitLimit(0)
    status = 0
    for _ in range(5):
        bd.integrateEquationOfMotion()
        status |= m.deviceStatus()
        if status & _lib.SVM_DEV_T1_TIMEOUT:
            break
    assert status & _lib.SVM_DEV_T1_TIMEOUT, status
    m.close()
    fresh = gpu_model(svm, gold)
    bd2 = svm.brownianDynamics()
    bd2.setModel(fresh)
    bd2.setT(0.01)
    for _ in range(10):
        bd2.integrateEquationOfMotion()
    fresh.computeGeometry()
    assert np.isfinite(fresh.computeEnergy()) and fresh.deviceStatus() == 0
