"""Host-side mirror of the reference's model / updater / simulation classes over libsvm.

Class and method names follow the reference (src/model/sphericalVertexModel.h,
src/updaters/brownianDynamics.h, src/updaters/energyMinimizerFIRE.h, src/simulation/simulation.h)
so that a driver written against the reference reads the same.  Everything runs on the GPU through
the C ABI; there is no CPU branch: setCPUOperation(True) raises.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _lib
from ._lib import call

PI = 3.141592653589793115997963468544185161590576171875


class Topology:
    """Initial spherical Voronoi topology of a set of cell centres (the convexHullCGAL contract)."""

    @classmethod
    def from_arrays(cls, vertexPositions, rings, ringCounts, vertexCells, vertexNeighbors) -> "Topology":
        """A topology given directly in the reference layouts (e.g. a saved state)."""
        t = cls.__new__(cls)
        t.vertexPositions = np.ascontiguousarray(vertexPositions, dtype=np.float64).reshape(-1, 3)
        t.rings = np.ascontiguousarray(rings, dtype=np.int32)
        t.ringCounts = np.ascontiguousarray(ringCounts, dtype=np.uint32)
        t.vertexCells = np.ascontiguousarray(vertexCells, dtype=np.int32).reshape(-1, 3)
        t.vertexNeighbors = np.ascontiguousarray(vertexNeighbors, dtype=np.int32).reshape(-1, 3)
        t.nCells = t.rings.shape[0]
        t.nVertices = t.vertexPositions.shape[0]
        t.maxRing = int(t.ringCounts.max())
        t.radius = float(np.linalg.norm(t.vertexPositions[0]))
        return t

    def __init__(self, centres: np.ndarray, triangles: np.ndarray | None = None, device: bool = False):
        """The hull of `centres` on the host (svm_topology_from_points), on the device
        (device=True, svm_topology_from_points_gpu: the same arrays), or the given triangles."""
        pts = np.ascontiguousarray(centres, dtype=np.float64).reshape(-1)
        n = pts.size // 3
        h = C.c_void_p()
        if triangles is None and device:
            call("svm_topology_from_points_gpu", pts, n, None, C.byref(h))
        elif triangles is None:
            call("svm_topology_from_points", pts, n, C.byref(h))
        else:
            tri = np.ascontiguousarray(triangles, dtype=np.int32).reshape(-1)
            call("svm_topology_from_triangles", pts, n, tri, tri.size // 3, C.byref(h))
        try:
            nc, nv, mr = C.c_int(), C.c_int(), C.c_int()
            call("svm_topology_sizes", h, C.byref(nc), C.byref(nv), C.byref(mr))
            self.nCells, self.nVertices, self.maxRing = nc.value, nv.value, mr.value
            W = self.maxRing
            self.vertexPositions = np.empty(3 * self.nVertices)
            self.rings = np.empty(self.nCells * W, dtype=np.int32)
            self.ringCounts = np.empty(self.nCells, dtype=np.uint32)
            self.vertexCells = np.empty(3 * self.nVertices, dtype=np.int32)
            self.vertexNeighbors = np.empty(3 * self.nVertices, dtype=np.int32)
            call("svm_topology_get", h, self.vertexPositions, self.rings, W, self.ringCounts, self.vertexCells,
                 self.vertexNeighbors)
        finally:
            _lib.lib().svm_topology_free(h)
        self.vertexPositions = self.vertexPositions.reshape(-1, 3)
        self.rings = self.rings.reshape(self.nCells, W)
        self.vertexCells = self.vertexCells.reshape(-1, 3)
        self.vertexNeighbors = self.vertexNeighbors.reshape(-1, 3)
        self.radius = float(np.sqrt(np.dot(pts[:3], pts[:3])))


def random_cell_centres(seed: int, n: int) -> np.ndarray:
    out = np.empty(3 * n)
    call("svm_random_cell_centres", int(seed), int(n), out)
    return out.reshape(n, 3)


def random_vertex_directors(seed: int, n_cells: int, vertex_positions: np.ndarray) -> np.ndarray:
    """Initial directors for these vertex positions: the construction of sphericalVertexModel.cpp:
    58-70 (a uniform random unit vector projected onto the tangent plane and normalised), drawn
    from the seeded stream after the cell centres and the cell model's directors.  The reference
    draws them from the model's own default noise source, which random_device seeds
    (noiseSource.h:21-30), so its directors do not repeat between runs; these do."""
    p = np.ascontiguousarray(vertex_positions, dtype=np.float64).reshape(-1)
    out = np.empty_like(p)
    call("svm_random_vertex_directors", int(seed), int(n_cells), p, p.size // 3, out)
    return out.reshape(-1, 3)


class noiseSource:
    """Seed holder mirroring src/utilities/noiseSource.h (reproducible mt19937 seed for the
    initial cell centres; the same seed keys the in-kernel Philox stream of the dynamics)."""

    def __init__(self, reproducible: bool = True):
        self.Reproducible = reproducible
        self.RNGSeed = -1

    def setReproducibleSeed(self, seed: int):
        self.RNGSeed = int(seed)
        self.Reproducible = True

    def setReproducible(self, rep: bool):
        self.Reproducible = rep


class sphericalVertexModel:
    """GPU spherical vertex model; N counts CELLS as in the reference constructor
    (sphericalVertexModel.cpp:5-82)."""

    def __init__(self, n: int, noise: noiseSource | None = None, a0: float = 1.0, p0: float = 3.8,
                 useGPU: bool = True, neverGPU: bool = False, ringCapacity: int = 16, stream=None,
                 topology: Topology | None = None, radius: float | None = None, ringHeadroom: int | None = None):
        """ringCapacity: the initial ring capacity (it grows on demand); ringHeadroom: free ring
        slots at or below which it grows before a T1 pass (svm_model_set_ring_headroom, default 2)."""
        if not useGPU or neverGPU:
            raise ValueError("this model runs on the GPU only")
        self.nCells = int(n)
        self.noise = noise or noiseSource(True)
        if topology is None:
            centres = random_cell_centres(self.noise.RNGSeed, self.nCells)
            topology = Topology(centres, device=True)
        self.topology = topology
        self.nVertices = topology.nVertices
        self.radius = math.sqrt(self.nCells / (4.0 * PI)) if radius is None else float(radius)
        cap = max(int(ringCapacity), topology.maxRing + 1)
        self.ringCapacity = cap
        h = C.c_void_p()
        call("svm_model_create", self.nCells, self.nVertices, cap, self.radius,
             C.c_void_p(stream) if stream else None, C.byref(h))
        self._h = h
        if ringHeadroom is not None:
            call("svm_model_set_ring_headroom", h, int(ringHeadroom))
        call("svm_model_set_topology", h, np.ascontiguousarray(topology.vertexPositions).reshape(-1),
             np.ascontiguousarray(topology.rings).reshape(-1), topology.rings.shape[1], topology.ringCounts,
             np.ascontiguousarray(topology.vertexCells).reshape(-1),
             np.ascontiguousarray(topology.vertexNeighbors).reshape(-1))
        self._restricted = False
        self.t1Threshold = 0.1
        call("svm_model_set_t1_threshold", h, 0.1)
        self.setPreferredParameters(a0, p0)
        self.setScalarModelParameter(1.0)
        self.setDirectors(random_vertex_directors(self.noise.RNGSeed, self.nCells, topology.vertexPositions))
        self.computeGeometry()

    def setDirectors(self, dirs: np.ndarray):
        """Directors, one per vertex (simpleModel.h:104-113), as used by the self-propelled updater."""
        call("svm_model_set_directors", self._h, np.ascontiguousarray(dirs, dtype=np.float64).reshape(-1))

    def returnDirectors(self) -> np.ndarray:
        out = np.empty(3 * self.nVertices)
        call("svm_model_get_directors", self._h, out)
        return out.reshape(-1, 3)

    # ---- lifetime ----
    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().svm_model_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    @property
    def handle(self):
        return self._h

    # ---- parameters (sphericalVertexModel.h:80-90, simpleModel.h:145) ----
    def setPreferredParameters(self, a0: float, p0: float):
        call("svm_model_set_preferred_parameters", self._h, float(a0), float(p0))

    def setPreferredParameterArray(self, a0p0: np.ndarray):
        call("svm_model_set_preferred_array", self._h, np.ascontiguousarray(a0p0, dtype=np.float64).reshape(-1))

    def setScalarModelParameter(self, kr: float):
        self.Kr = float(kr)
        call("svm_model_set_scalar_model_parameter", self._h, self.Kr)

    def setT1Threshold(self, t: float):
        self.t1Threshold = float(t)
        call("svm_model_set_t1_threshold", self._h, self.t1Threshold)

    @property
    def precision(self) -> str:
        """'fp64' (every quantity in FP64, the reference's formulas), 'mixed' (FP32 positions,
        forces and integration; FP64 included angles, areas, energy and renormalisation) or
        'fp64_vector' (FP64 with the forces as the exact gradient in vector form, for tight
        minimisation)."""
        return getattr(self, "_precision", "fp64")

    @precision.setter
    def precision(self, p: str):
        code = {"fp64": _lib.SVM_PRECISION_FP64, "mixed": _lib.SVM_PRECISION_MIXED,
                "fp64_vector": _lib.SVM_PRECISION_FP64_VECTOR}[p]
        call("svm_model_set_precision", self._h, code)
        self._precision = p

    @property
    def restrictedMotion(self) -> bool:
        return self._restricted

    @restrictedMotion.setter
    def restrictedMotion(self, r: bool):
        self._restricted = bool(r)
        call("svm_model_set_restricted_motion", self._h, int(self._restricted))

    def getNumberOfParticles(self) -> int:
        return self.nVertices

    # ---- the path ----
    def computeGeometry(self):
        call("svm_model_compute_geometry", self._h)

    def computeForces(self, zeroOutForces: bool = True):
        call("svm_model_compute_forces", self._h)

    def computeEnergy(self) -> float:
        e = C.c_double()
        call("svm_model_compute_energy", self._h, C.byref(e))
        return e.value

    def moveParticles(self, displacements: np.ndarray, scale: float = 1.0):
        call("svm_model_move_particles_host", self._h, np.ascontiguousarray(displacements, dtype=np.float64).reshape(-1),
             float(scale))

    def enforceTopology(self):
        call("svm_model_enforce_topology", self._h)

    # ---- state access ----
    def _vec(self, fn, n):
        out = np.empty(3 * n)
        call(fn, self._h, out)
        return out.reshape(n, 3)

    def returnPositions(self) -> np.ndarray:
        return self._vec("svm_model_get_positions", self.nVertices)

    def setPositions(self, p: np.ndarray):
        call("svm_model_set_positions", self._h, np.ascontiguousarray(p, dtype=np.float64).reshape(-1))

    def returnForces(self) -> np.ndarray:
        return self._vec("svm_model_get_forces", self.nVertices)

    def returnVelocities(self) -> np.ndarray:
        return self._vec("svm_model_get_velocities", self.nVertices)

    def setVelocities(self, v: np.ndarray):
        call("svm_model_set_velocities", self._h, np.ascontiguousarray(v, dtype=np.float64).reshape(-1))

    def cellPositions(self) -> np.ndarray:
        return self._vec("svm_model_get_cell_positions", self.nCells)

    def areaPerimeter(self) -> np.ndarray:
        out = np.empty(2 * self.nCells)
        call("svm_model_get_area_perimeter", self._h, out)
        return out.reshape(self.nCells, 2)

    def ringInfo(self) -> dict:
        """Ring capacity (it grows as the reference's growCellVerticesList widens its rings), the
        largest ring count seen and the number of growths."""
        out = np.zeros(3, dtype=np.int32)
        call("svm_model_ring_info", self._h, out)
        return dict(capacity=int(out[0]), max_ring=int(out[1]), growths=int(out[2]))

    def setRingHeadroom(self, slots: int):
        """The ring capacity grows before a T1 pass when this many slots or fewer are free in the
        largest ring (default 2)."""
        call("svm_model_set_ring_headroom", self._h, int(slots))

    def rings(self, stride: int | None = None):
        W = stride or self.ringInfo()["capacity"]
        out = np.empty(self.nCells * W, dtype=np.int32)
        cnt = np.empty(self.nCells, dtype=np.uint32)
        call("svm_model_get_rings", self._h, out, W, cnt)
        return out.reshape(self.nCells, W), cnt

    def vertexCellNeighbors(self) -> np.ndarray:
        out = np.empty(3 * self.nVertices, dtype=np.int32)
        call("svm_model_get_vertex_cells", self._h, out)
        return out.reshape(-1, 3)

    def vertexNeighbors(self) -> np.ndarray:
        out = np.empty(3 * self.nVertices, dtype=np.int32)
        call("svm_model_get_vertex_neighbors", self._h, out)
        return out.reshape(-1, 3)

    def areaCheck(self):
        """(total area, excess over 4 pi R^2, fallback taken) of the last geometry pass."""
        t, e, f = C.c_double(), C.c_double(), C.c_int()
        call("svm_model_area_check", self._h, C.byref(t), C.byref(e), C.byref(f))
        return t.value, e.value, bool(f.value)

    def deviceStatus(self) -> int:
        st = C.c_int()
        call("svm_model_status", self._h, C.byref(st))
        return st.value

    def takeFlips(self, capacity: int = 1 << 16) -> np.ndarray:
        out = np.empty(2 * capacity, dtype=np.int32)
        n = C.c_int()
        call("svm_model_take_flips", self._h, out, capacity, C.byref(n))
        return out[: 2 * min(n.value, capacity)].reshape(-1, 2)

    def streamHandle(self) -> int:
        """The cudaStream_t the model's work runs on (e.g. for torch.cuda.ExternalStream)."""
        s = C.c_void_p()
        call("svm_model_stream", self._h, C.byref(s))
        return s.value or 0

    def t1Stats(self) -> dict:
        """T1 counters since the last call: passes, flagged edges, edges run in parallel rounds,
        flips, rounds, passes replayed sequentially after a rollback."""
        out = np.zeros(6, dtype=np.int32)
        call("svm_model_t1_stats", self._h, out)
        return dict(passes=int(out[0]), flagged=int(out[1]), executed=int(out[2]), flips=int(out[3]),
                    rounds=int(out[4]), rollbacks=int(out[5]))

    def synchronize(self):
        call("svm_model_synchronize", self._h)

    def fallbackCount(self) -> int:
        """Geometry passes that took the triangle-fan area fallback since the last call."""
        n = C.c_int()
        call("svm_model_fallback_count", self._h, C.byref(n))
        return n.value

    def setT1Blocks(self, blocks: int = 0):
        """Blocks of the parallel T1 pass (0 automatic, 1 one block, n a cooperative grid of n);
        performance only, the results do not depend on it."""
        call("svm_model_set_t1_blocks", self._h, int(blocks))

    def setT1WaitLimit(self, polls: int = 1 << 20):
        """Polls of a cooperative T1 pass's grid-barrier wait before it gives up and reports
        SVM_DEV_T1_TIMEOUT (a diagnostic hook; a model whose pass gave up is to be recreated)."""
        call("svm_model_set_t1_wait_limit", self._h, int(polls))

    def t1Clocks(self, enable: bool = True):
        """SM cycles of the parallel T1 pass's phases since the last call (extraction, reserve,
        flips, release, end) and re-arms the counters (or turns them off)."""
        out = np.zeros(5, dtype=np.uint64)
        call("svm_model_t1_clocks", self._h, int(enable), out)
        return dict(zip(("extract", "reserve", "flip", "release", "end"), map(int, out)))

    def saveState(self) -> dict:
        """Positions and connectivity (host copies) for loadState."""
        rings, counts = self.rings()
        return dict(pos=self.returnPositions(), rings=rings, counts=counts, vcells=self.vertexCellNeighbors(),
                    vnbrs=self.vertexNeighbors())

    def loadState(self, st: dict):
        rings = np.ascontiguousarray(st["rings"], dtype=np.int32)
        call("svm_model_set_topology", self._h, np.ascontiguousarray(st["pos"], dtype=np.float64).reshape(-1),
             rings.reshape(-1), rings.shape[1], np.ascontiguousarray(st["counts"], dtype=np.uint32),
             np.ascontiguousarray(st["vcells"], dtype=np.int32).reshape(-1),
             np.ascontiguousarray(st["vnbrs"], dtype=np.int32).reshape(-1))


class sphericalVertexModelBatch(sphericalVertexModel):
    """Independent spheres (replicas) of uneven size in one model (svm_batch_* in include/svm.h):
    every step of the batch is one set of launches over all replicas.  Replica r has nCells[r]
    cells whose centres come from seeds[r] (random_cell_centres, the reference's recipe), radius
    sqrt(nCells[r] / 4 pi), and its own P0 and temperature.  Runs the mixed-precision form.
    State accessors of the base class return the concatenated arrays; `cellSlice(r)` and
    `vertexSlice(r)` cut replica r out of them."""

    def __init__(self, nCells, seeds, a0: float = 1.0, p0=3.8, ringCapacity: int = 16, stream=None,
                 topologies=None):
        nCells = [int(n) for n in nCells]
        R = len(nCells)
        if topologies is None:
            topologies = [Topology(random_cell_centres(int(sd), n), device=True) for n, sd in zip(nCells, seeds)]
        self.topologies = topologies
        self.nReplicas = R
        self.radii = np.array([math.sqrt(n / (4.0 * PI)) for n in nCells])
        self.radius = self.radii
        self.replicaCells = np.array(nCells, dtype=np.int32)
        self.replicaVertices = np.array([t.nVertices for t in topologies], dtype=np.int32)
        self.cellOffsets = np.concatenate([[0], np.cumsum(self.replicaCells)]).astype(np.int64)
        self.vertexOffsets = np.concatenate([[0], np.cumsum(self.replicaVertices)]).astype(np.int64)
        self.nCells = int(self.cellOffsets[-1])
        self.nVertices = int(self.vertexOffsets[-1])
        cap = max(int(ringCapacity), max(t.maxRing for t in topologies) + 1)
        self.ringCapacity = cap
        h = C.c_void_p()
        call("svm_batch_create", R, self.replicaCells, self.replicaVertices, cap, self.radii,
             C.c_void_p(stream) if stream else None, C.byref(h))
        self._h = h
        self._precision = "mixed"
        rings = np.full((self.nCells, cap), -1, dtype=np.int32)
        pos = np.empty((self.nVertices, 3))
        counts = np.empty(self.nCells, dtype=np.uint32)
        vc = np.empty((self.nVertices, 3), dtype=np.int32)
        vn = np.empty((self.nVertices, 3), dtype=np.int32)
        for r, t in enumerate(topologies):
            c0, c1 = self.cellOffsets[r], self.cellOffsets[r + 1]
            v0, v1 = self.vertexOffsets[r], self.vertexOffsets[r + 1]
            w = t.rings.shape[1]
            rings[c0:c1, :w] = np.where(t.rings >= 0, t.rings + v0, -1)
            counts[c0:c1] = t.ringCounts
            pos[v0:v1] = t.vertexPositions
            vc[v0:v1] = t.vertexCells + c0
            vn[v0:v1] = t.vertexNeighbors + v0
        call("svm_model_set_topology", h, pos.reshape(-1), rings.reshape(-1), cap, counts, vc.reshape(-1),
             vn.reshape(-1))
        self._restricted = False
        self.t1Threshold = 0.1
        call("svm_model_set_t1_threshold", h, 0.1)
        self.setPreferredParameters(a0, p0)
        self.setScalarModelParameter(1.0)
        self.temperatures = np.zeros(R)
        self.computeGeometry()

    def cellSlice(self, r: int) -> slice:
        return slice(int(self.cellOffsets[r]), int(self.cellOffsets[r + 1]))

    def vertexSlice(self, r: int) -> slice:
        return slice(int(self.vertexOffsets[r]), int(self.vertexOffsets[r + 1]))

    def setPreferredParameters(self, a0, p0):
        """A0 and P0: scalars, or one value per replica."""
        a = np.broadcast_to(np.asarray(a0, dtype=np.float64), (self.nReplicas,))
        p = np.broadcast_to(np.asarray(p0, dtype=np.float64), (self.nReplicas,))
        pref = np.empty((self.nCells, 2))
        pref[:, 0] = np.repeat(a, self.replicaCells)
        pref[:, 1] = np.repeat(p, self.replicaCells)
        self.setPreferredParameterArray(pref)

    def setTemperatures(self, T):
        self.temperatures = np.ascontiguousarray(np.broadcast_to(np.asarray(T, dtype=np.float64),
                                                                 (self.nReplicas,)))
        call("svm_batch_set_temperatures", self._h, self.temperatures)

    def replicaEnergies(self) -> np.ndarray:
        out = np.empty(self.nReplicas)
        call("svm_batch_energies", self._h, out)
        return out

    def replicaAreaCheck(self):
        """Per replica: total area, excess over 4 pi R^2, fallback taken (last geometry pass)."""
        t, e, f = np.empty(self.nReplicas), np.empty(self.nReplicas), np.empty(self.nReplicas, dtype=np.int32)
        call("svm_batch_area_check", self._h, t, e, f)
        return t, e, f.astype(bool)

    def autotune(self, lo: int = 64, hi: int = 1024, step: int = 64, nSamples: int = 3, period: int = 1000):
        """Block sizes of the batch kernels picked by kernelTuner-style sampling (lo <= 0: off)."""
        call("svm_batch_autotune", self._h, int(lo), int(hi), int(step), int(nSamples), int(period))

    def blockSizes(self):
        out = np.zeros(3, dtype=np.int32)
        done = C.c_int()
        call("svm_batch_block_sizes", self._h, out, C.byref(done))
        return dict(corners=int(out[0]), cells=int(out[1]), force=int(out[2]), samplingComplete=bool(done.value))

    @property
    def precision(self) -> str:
        return "mixed"

    @precision.setter
    def precision(self, p: str):
        if p != "mixed":
            raise ValueError("batches run the mixed-precision form")


class sphericalSelfPropelledParticle:
    """Self-propelled vertices on the sphere (src/updaters/sphericalSelfPropelledParticle.{h,cpp}):
    disp = dt (v0 n + mu F), then each director is re-projected and rotated by a uniform angle of
    half-width sqrt(2 dt tau) / 2 about its vertex.  The reference's GPU branch is empty; here the
    step runs on the device, with in-kernel Philox draws or injected uniforms."""

    def __init__(self, reproducible: bool = True):
        self.noise = noiseSource(reproducible)
        self.model = None
        self.deltaT = 0.01
        self.mu = 1.0
        self.v0 = 0.0
        self.tau = 1.0
        self._injected = None

    def setModel(self, model: sphericalVertexModel):
        self.model = model

    def setDeltaT(self, dt: float):
        self.deltaT = float(dt)

    def setMu(self, mu: float):
        self.mu = float(mu)

    def setV0(self, v0: float):
        self.v0 = float(v0)

    def setTau(self, tau: float):
        self.tau = float(tau)

    def injectNoise(self, r: np.ndarray | None):
        """Uniform draws in [-1/2, 1/2), one per vertex, for the next step only."""
        self._injected = None if r is None else np.ascontiguousarray(r, dtype=np.float64).reshape(-1)

    def integrateEquationOfMotion(self):
        m = self.model
        seed = self.noise.RNGSeed if self.noise.RNGSeed >= 0 else 1337
        if self._injected is not None:
            call("svm_spp_step", m.handle, self.deltaT, self.mu, self.v0, self.tau, _lib.SVM_NOISE_BUFFER,
                 self._injected, seed)
            self._injected = None
        else:
            call("svm_spp_step", m.handle, self.deltaT, self.mu, self.v0, self.tau, _lib.SVM_NOISE_PHILOX, None, seed)

    def performUpdate(self):
        self.integrateEquationOfMotion()

    def run(self, nSteps: int):
        for _ in range(int(nSteps)):
            self.integrateEquationOfMotion()


class sphericalVectorialVicsek(sphericalSelfPropelledParticle):
    """Vicsek alignment of the vertices' directors (src/updaters/sphericalVectorialVicsek.{h,cpp},
    parameters of vectorialVicsek.h:11-44, defaults mu 1, Eta 1, tau 1, v0 0.01): the self-propelled
    move, then each director relaxes at rate dt / tau towards the normalised tangent average of
    itself and its three vertex neighbours plus Eta times a random tangent unit vector.  The
    reference runs it on the CPU only; here the step runs on the device."""

    def __init__(self, reproducible: bool = True):
        super().__init__(reproducible)
        self.v0 = 0.01
        self.Eta = 1.0

    def setEta(self, eta: float):
        self.Eta = float(eta)

    def injectNoise(self, uw: np.ndarray | None):
        """Uniform draws in [0, 1), (u, w) for each vertex in vertex order, for the next step only."""
        self._injected = None if uw is None else np.ascontiguousarray(uw, dtype=np.float64).reshape(-1)

    def integrateEquationOfMotion(self):
        m = self.model
        seed = self.noise.RNGSeed if self.noise.RNGSeed >= 0 else 1337
        if self._injected is not None:
            call("svm_vicsek_step", m.handle, self.deltaT, self.mu, self.v0, self.Eta, self.tau,
                 _lib.SVM_NOISE_BUFFER, self._injected, seed)
            self._injected = None
        else:
            call("svm_vicsek_step", m.handle, self.deltaT, self.mu, self.v0, self.Eta, self.tau,
                 _lib.SVM_NOISE_PHILOX, None, seed)


class brownianDynamics:
    """Overdamped Brownian updater (brownianDynamics.h:11-29)."""

    def __init__(self, reproducible: bool = True):
        self.temperature = 0.0
        self.deltaT = 0.01
        self.mu = 1.0
        self.reproducible = reproducible
        self.noise = noiseSource(reproducible)
        self.model: sphericalVertexModel | None = None
        self._injected = None

    def setModel(self, model: sphericalVertexModel):
        self.model = model

    def setT(self, T: float):
        self.temperature = float(T)

    def setDeltaT(self, dt: float):
        self.deltaT = float(dt)

    def injectNoise(self, xi: np.ndarray | None):
        """Standard normals for the next step ([Nv,3], vertex-major), e.g. the reference's stream."""
        self._injected = None if xi is None else np.ascontiguousarray(xi, dtype=np.float64).reshape(-1)

    def _seed(self) -> int:
        return self.noise.RNGSeed if self.noise.RNGSeed >= 0 else 1337

    def integrateEquationOfMotion(self):
        m = self.model
        if self._injected is not None:
            call("svm_brownian_step_host_noise", m.handle, self.temperature, self.deltaT, self.mu, self._injected)
            self._injected = None
        else:
            call("svm_brownian_step", m.handle, self.temperature, self.deltaT, self.mu, _lib.SVM_NOISE_PHILOX, None,
                 self._seed())

    performUpdate = integrateEquationOfMotion

    def run(self, nSteps: int):
        """nSteps timesteps as one graph-captured launch sequence (Philox noise)."""
        call("svm_brownian_run", self.model.handle, self.temperature, self.deltaT, self.mu, self._seed(), int(nSteps))


class velocityVerlet:
    """Velocity-Verlet updater (src/updaters/velocityVerlet.{h,cpp}) with unit masses: per step,
    disp = dt v + dt^2/2 F and v += dt/2 F, the move (with T1 flips unless motion is restricted),
    geometry and forces, v += dt/2 F.  Forces must be current before the first step, as in the
    reference (computeForces)."""

    def __init__(self):
        self.deltaT = 0.01
        self.model: sphericalVertexModel | None = None

    def setModel(self, model: sphericalVertexModel):
        self.model = model

    def setDeltaT(self, dt: float):
        self.deltaT = float(dt)

    def integrateEquationOfMotion(self):
        call("svm_velocity_verlet_step", self.model.handle, self.deltaT, 1)

    performUpdate = integrateEquationOfMotion

    def run(self, nSteps: int):
        call("svm_velocity_verlet_step", self.model.handle, self.deltaT, int(nSteps))

    def halfKick(self):
        """gpu_update_velocity (velocityVerlet.cuh:14-19): v += dt/2 F."""
        call("svm_vv_half", self.model.handle, self.deltaT)


def dotProducts(model: sphericalVertexModel) -> dict:
    """gpu_dVec_dot_products (utilities.cuh:74) over the model's forces and velocities: sum F.v,
    sum F.F, sum v.v and max |F|."""
    out = np.empty(4)
    call("svm_reduce_dots", model.handle, out)
    return dict(power=out[0], force_norm2=out[1], velocity_norm2=out[2], max_force=out[3])


class energyMinimizerFIRE:
    """FIRE minimiser (energyMinimizerFIRE.h:27-68) with device-side control."""

    def __init__(self, model: sphericalVertexModel):
        self.model = model
        self._h = None
        self.params = dict(dt=0.01, alphaStart=0.99, dtMax=0.1, dtInc=1.05, dtDec=0.95, alphaDec=0.9, nMin=5,
                           forceCutoff=1e-7, alphaMin=0.0)
        self.maxIterations = 1000
        self.criterion = _lib.SVM_FIRE_RMS_OVER_N
        self._last = (0, 100.0)

    def setFIREParameters(self, deltaT, alphaStart, deltaTMax, deltaTInc, deltaTDec, alphaDec, nMin, forceCutoff,
                          alphaMin=0.75):
        self.params = dict(dt=deltaT, alphaStart=alphaStart, dtMax=deltaTMax, dtInc=deltaTInc, dtDec=deltaTDec,
                           alphaDec=alphaDec, nMin=nMin, forceCutoff=forceCutoff, alphaMin=alphaMin)
        self._reset()

    def setMaximumIterations(self, n: int):
        """Cap on the total iteration count; an existing minimizer keeps its dt, alpha and counters."""
        self.maxIterations = int(n)
        if self._h:
            call("svm_fire_set_max_iterations", self._h, self.maxIterations)

    def setForceCutoff(self, fc: float):
        self.params["forceCutoff"] = float(fc)
        self._reset()

    def setCriterion(self, criterion: int):
        self.criterion = int(criterion)

    def _reset(self):
        if self._h:
            _lib.lib().svm_fire_destroy(self._h)
            self._h = None

    def _ensure(self):
        if self._h is None:
            p = self.params
            h = C.c_void_p()
            call("svm_fire_create", self.model.handle, p["dt"], p["alphaStart"], p["dtMax"], p["dtInc"], p["dtDec"],
                 p["alphaDec"], int(p["nMin"]), p["forceCutoff"], p["alphaMin"], self.maxIterations, C.byref(h))
            self._h = h

    def minimize(self) -> int:
        self._ensure()
        it, val = C.c_int(), C.c_double()
        call("svm_fire_minimize", self._h, self.criterion, C.byref(it), C.byref(val))
        self._last = (it.value, val.value)
        return it.value

    performUpdate = minimize

    def state(self) -> dict:
        self._ensure()
        out = np.empty(7)
        call("svm_fire_state", self._h, out)
        return dict(dt=out[0], alpha=out[1], power=out[2], force_rms_over_n=out[3], max_force=out[4],
                    n_since=int(out[5]), iterations=int(out[6]))

    def fireStep(self):
        """fireStep (energyMinimizerFIRE.h:56): the sums, velocity update and dt/alpha control on
        the model's current forces and velocities (no integration; minimize pairs it with a
        velocity-Verlet step at the current dt)."""
        self._ensure()
        call("svm_fire_step", self._h)

    def integrateEquationOfMotion(self):
        """One velocity-Verlet step at the minimizer's current dt (energyMinimizerFIRE inherits
        velocityVerlet::integrateEquationOfMotion)."""
        call("svm_velocity_verlet_step", self.model.handle, self.state()["dt"], 1)

    def getMaxForce(self) -> float:
        return self.state()["force_rms_over_n"]

    def getCurrentIterations(self) -> int:
        return self.state()["iterations"]

    def __del__(self):
        self._reset()


class warmStartNetwork:
    """The per-vertex MLP of the learned FIRE warm start (svm_mlp_* in include/svm.h).  Device
    arrays are torch CUDA tensors (used for their memory only); every computation runs in libsvm's
    kernels."""

    def __init__(self, seed: int = 1, stream=None):
        h = C.c_void_p()
        call("svm_mlp_create", int(seed), C.c_void_p(stream) if stream else None, C.byref(h))
        self._h = h
        n = C.c_int()
        call("svm_mlp_parameter_count", C.byref(n))
        self.parameterCount = n.value
        self.outputScale = 1.0

    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().svm_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def weights(self) -> np.ndarray:
        w = np.empty(self.parameterCount, dtype=np.float32)
        call("svm_mlp_get_weights", self._h, w)
        return w

    def setWeights(self, w: np.ndarray):
        call("svm_mlp_set_weights", self._h, np.ascontiguousarray(w, dtype=np.float32))

    def setOutputScale(self, scale: float):
        self.outputScale = float(scale)
        call("svm_mlp_set_output_scale", self._h, self.outputScale)

    @staticmethod
    def features(model: sphericalVertexModel, frames: bool = False):
        """Features [nV, 24] (and frames [nV, 6]) of an FP64 model's current state after
        computeForces."""
        import torch
        X = torch.empty((model.nVertices, 24), dtype=torch.float32, device="cuda")
        F = torch.empty((model.nVertices, 6), dtype=torch.float64, device="cuda") if frames else None
        torch.cuda.synchronize()
        call("svm_mlp_features", model.handle, C.c_void_p(X.data_ptr()),
             C.c_void_p(F.data_ptr()) if F is not None else None)
        return (X, F) if frames else X

    def gradient(self, X, T):
        """(mean squared error, gradient) over the samples X [n, 24], T [n, 2] (CUDA tensors)."""
        import torch
        torch.cuda.synchronize()
        g = np.empty(self.parameterCount, dtype=np.float32)
        loss = C.c_double()
        call("svm_mlp_gradient", self._h, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()), int(X.shape[0]), g,
             C.byref(loss))
        return loss.value, g

    def train(self, X, T, epochs: int, batch: int = 4096, lr: float = 1e-3, seed: int = 0):
        """Adam epochs over (X, T) in a fresh seeded permutation each epoch; mean losses."""
        import torch
        rng = np.random.default_rng(seed)
        n = int(X.shape[0])
        losses = []
        for _ in range(epochs):
            order = torch.from_numpy(rng.permutation(n).astype(np.int32)).cuda()
            torch.cuda.synchronize()
            loss = C.c_double()
            call("svm_mlp_train", self._h, C.c_void_p(X.data_ptr()), C.c_void_p(T.data_ptr()),
                 C.c_void_p(order.data_ptr()), n, int(batch), C.c_float(lr), C.byref(loss))
            losses.append(loss.value)
        return losses

    def predict(self, X):
        import torch
        Y = torch.empty((X.shape[0], 2), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        call("svm_mlp_predict", self._h, C.c_void_p(X.data_ptr()), int(X.shape[0]), C.c_void_p(Y.data_ptr()))
        return Y

    def warmStart(self, model: sphericalVertexModel):
        """Moves every vertex of an FP64 model by the network's predicted displacement."""
        call("svm_mlp_warm_start", self._h, model.handle)


class neighborList:
    """Metric neighbour lists of points on the device (src/utilities/neighborList.{h,cpp}): every
    other point within `range` (minimum image in a periodic box of side 2 sphereRadius), through a
    cell list of grid size range / subGridReduction.  The spherical model's own is
    neighborList(1.0, R + 2.5) (sphericalModel.cpp:21)."""

    def __init__(self, range_: float, sphereRadius: float, subGridReduction: int = 1, slotCapacity: int = 16):
        self.maxRange = float(range_)
        self.radius = float(sphereRadius)
        self.subGridReduction = int(subGridReduction)
        self.slotCapacity = int(slotCapacity)
        self._h = None
        self._n = 0

    def _ensure(self, n: int):
        if self._h is not None and self._n == n:
            return
        self.close()
        h = C.c_void_p()
        call("svm_neighbor_list_create", self.maxRange, self.radius, self.subGridReduction, int(n),
             self.slotCapacity, None, C.byref(h))
        self._h, self._n = h, int(n)

    def computeNeighborLists(self, points, fetch: bool = True):
        """`points`: a sphericalVertexModel (its vertex positions) or a torch CUDA tensor of shape
        (n, 3), float64.  fetch=False leaves the lists on the device (Nmax is still read)."""
        if isinstance(points, sphericalVertexModel):
            self._ensure(points.nVertices)
            call("svm_neighbor_list_compute_model", self._h, points.handle)
        else:
            if (not getattr(points, "is_cuda", False) or str(points.dtype) != "torch.float64"
                    or points.dim() != 2 or points.shape[1] != 3 or not points.is_contiguous()):
                raise ValueError("points: a contiguous float64 CUDA tensor of shape (n, 3), or a model")
            n = int(points.shape[0])
            self._ensure(n)
            call("svm_neighbor_list_compute", self._h, C.c_void_p(points.data_ptr()), n)
        nm = C.c_int()
        if not fetch:
            call("svm_neighbor_list_get", self._h, C.byref(nm), None, None, None, None, 0)
            self.Nmax = nm.value
            return
        npp = np.empty(self._n, dtype=np.uint32)
        call("svm_neighbor_list_get", self._h, C.byref(nm), npp, None, None, None, 0)
        e = self._n * nm.value
        idx = np.empty(e, dtype=np.int32)
        vec = np.empty(3 * e)
        dist = np.empty(e)
        call("svm_neighbor_list_get", self._h, C.byref(nm), npp, idx, vec, dist, e)
        self.Nmax = nm.value
        self.neighborsPerParticle = npp
        self.particleIndices = idx.reshape(self._n, self.Nmax)
        self.neighborVectors = vec.reshape(self._n, self.Nmax, 3)
        self.neighborDistances = dist.reshape(self._n, self.Nmax)

    def close(self):
        if self._h is not None:
            _lib.lib().svm_neighbor_list_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()


class Simulation:
    """Ordered updaters over one configuration (src/simulation/simulation.{h,cpp})."""

    def __init__(self):
        self.configuration: sphericalVertexModel | None = None
        self.updaters = []
        self.integerTimestep = 0
        self.Time = 0.0
        self.integrationTimestep = 0.01

    def setConfiguration(self, config: sphericalVertexModel):
        self.configuration = config

    def addUpdater(self, upd, config=None):
        if config is not None and hasattr(upd, "setModel"):
            upd.setModel(config)
        self.updaters.append(upd)

    def setIntegrationTimestep(self, dt: float):
        self.integrationTimestep = float(dt)
        for u in self.updaters:
            if hasattr(u, "setDeltaT"):
                u.setDeltaT(dt)

    def setCPUOperation(self, setcpu: bool):
        if setcpu:
            raise ValueError("CPU operation is not available: this path runs on the GPU only")

    def setReproducible(self, reproducible: bool):
        for u in self.updaters:
            if hasattr(u, "reproducible"):
                u.reproducible = reproducible

    def computeForces(self):
        self.configuration.computeForces(True)

    def moveParticles(self, displacements, scale: float = 1.0):
        self.configuration.moveParticles(displacements, scale)

    def computeEnergy(self) -> float:
        return self.configuration.computeEnergy()

    def performTimestep(self):
        self.integerTimestep += 1
        self.Time += self.integrationTimestep
        for u in self.updaters:
            u.performUpdate()
