"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes wrappers for the CPU oracle (liborc.so, the restatement of the reference's CPU path in
svm_oracle.cpp) and, where it has been built, the reference itself compiled from its sources
(_ref/libsvmref.so).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs may
import this module; the product package never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIBORC = os.path.join(HERE, "liborc.so")
LIBREF = os.path.join(HERE, "_ref", "libsvmref.so")

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_up = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")


def build_oracle() -> str:
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIBORC


def _sig(lib, name, res, *args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = list(args)
    return f


_orc = None


def orc_lib():
    global _orc
    if _orc is None:
        if not os.path.exists(LIBORC):
            build_oracle()
        lib = C.CDLL(LIBORC)
        vp = C.c_void_p
        _sig(lib, "orc_create", vp, C.c_int, C.c_int, C.c_int, _dp, _ip, _up, _ip, _ip, C.c_double)
        _sig(lib, "orc_destroy", None, vp)
        _sig(lib, "orc_set_preferred", None, vp, C.c_double, C.c_double)
        _sig(lib, "orc_set_preferred_array", None, vp, _dp)
        _sig(lib, "orc_set_kr", None, vp, C.c_double)
        _sig(lib, "orc_set_t1_threshold", None, vp, C.c_double)
        _sig(lib, "orc_set_restricted", None, vp, C.c_int)
        _sig(lib, "orc_compute_geometry", None, vp)
        _sig(lib, "orc_compute_forces", None, vp)
        _sig(lib, "orc_energy", C.c_double, vp)
        _sig(lib, "orc_move", None, vp, _dp, C.c_double)
        _sig(lib, "orc_enforce_topology", None, vp)
        _sig(lib, "orc_num_vertices", C.c_int, vp)
        _sig(lib, "orc_ring_width", C.c_int, vp)
        for n in ("positions", "forces", "velocities", "cell_positions", "area_perimeter"):
            _sig(lib, "orc_get_" + n, None, vp, _dp)
        _sig(lib, "orc_set_positions", None, vp, _dp)
        _sig(lib, "orc_set_velocities", None, vp, _dp)
        _sig(lib, "orc_get_rings", C.c_int, vp, _ip, C.c_int, _up)
        _sig(lib, "orc_get_vertex_cells", None, vp, _ip)
        _sig(lib, "orc_get_vertex_neighbors", None, vp, _ip)
        _sig(lib, "orc_flip_count", C.c_int, vp)
        _sig(lib, "orc_get_flips", None, vp, _ip)
        _sig(lib, "orc_clear_flips", None, vp)
        _sig(lib, "orc_dynamics", None, _dp, _dp, C.c_int, C.c_double, C.c_double, C.c_double,
             C.POINTER(C.c_double), C.POINTER(C.c_double))
        _sig(lib, "orc_log_spaced", None, C.c_int, C.c_double, C.c_int, _ip)
        _sig(lib, "orc_neighbor_list", C.c_int, _dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, _up, _ip, _dp,
             _dp, C.c_long)
        _sig(lib, "orc_set_directors", None, vp, _dp)
        _sig(lib, "orc_get_directors", None, vp, _dp)
        _sig(lib, "orc_init_directors", None, vp, vp)
        _sig(lib, "orc_spp_step_noise", None, vp, _dp, C.c_double, C.c_double, C.c_double, C.c_double)
        _sig(lib, "orc_vicsek_step_noise", None, vp, _dp, C.c_double, C.c_double, C.c_double, C.c_double,
             C.c_double)
        _sig(lib, "orc_noise_uniforms", None, vp, C.c_double, C.c_double, _dp, C.c_long)
        _sig(lib, "orc_last_excess_area", C.c_double, vp)
        _sig(lib, "orc_fallback_count", C.c_int, vp)
        _sig(lib, "orc_noise_create", vp, C.c_int)
        _sig(lib, "orc_noise_destroy", None, vp)
        _sig(lib, "orc_noise_uniform", C.c_double, vp, C.c_double, C.c_double)
        _sig(lib, "orc_noise_normals", None, vp, _dp, C.c_long)
        _sig(lib, "orc_random_cell_centres", None, vp, C.c_int, _dp)
        _sig(lib, "orc_brownian_step", None, vp, vp, C.c_double, C.c_double, C.c_double, C.c_void_p)
        _sig(lib, "orc_brownian_step_noise", None, vp, _dp, C.c_double, C.c_double, C.c_double)
        _sig(lib, "orc_fire_create", vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
             C.c_double, C.c_int, C.c_double, C.c_double, C.c_int)
        _sig(lib, "orc_fire_destroy", None, vp)
        _sig(lib, "orc_fire_minimize", C.c_int, vp, vp, C.c_int)
        _sig(lib, "orc_fire_iterate", None, vp, vp, C.c_int)
        _sig(lib, "orc_fire_state", None, vp, _dp)
        _sig(lib, "orc_vv_step", None, vp, C.c_double)
        _sig(lib, "orc_fire_step", None, vp, vp)
        _sig(lib, "orc_cell_list_dims", C.c_int, C.c_double, C.c_double, C.POINTER(C.c_int), C.POINTER(C.c_double))
        _sig(lib, "orc_cell_list", C.c_int, _dp, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_int), _ip, _up, _ip, C.c_long)
        _sig(lib, "orc_set_portable_acos", None, C.c_int)
        _sig(lib, "orc_set_acos_mode", None, C.c_int, C.c_ulonglong)
        _sig(lib, "orc_acos_portable", None, _dp, _dp, C.c_long)
        _orc = lib
    return _orc


def set_portable_acos(on: bool) -> None:
    """Geometry arccosine of every oracle model in this process: the C library's (the reference's
    std::acos; the default) or the portable one shared with the device's portable build."""
    orc_lib().orc_set_portable_acos(1 if on else 0)


def set_acos_mode(mode: int, seed: int = 0) -> None:
    """0: the C library's acos; 1: the portable one; 2: the C library's with a seeded one-ulp
    perturbation of one result in four (another faithful arccosine)."""
    orc_lib().orc_set_acos_mode(int(mode), int(seed))


def acos_portable(x) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64).reshape(-1)
    out = np.empty_like(x)
    orc_lib().orc_acos_portable(x, out, x.size)
    return out


class OracleNoise:
    """std::mt19937 + libstdc++ distributions, seeded as noiseSource::setReproducibleSeed."""

    def __init__(self, seed: int = -1):
        self.lib = orc_lib()
        self.h = self.lib.orc_noise_create(int(seed))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_noise_destroy(self.h)
            self.h = None

    def normals(self, count: int) -> np.ndarray:
        out = np.empty(count, dtype=np.float64)
        self.lib.orc_noise_normals(self.h, out, count)
        return out

    def uniforms(self, count: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        out = np.empty(count, dtype=np.float64)
        self.lib.orc_noise_uniforms(self.h, lo, hi, out, count)
        return out

    def cell_centres(self, n: int) -> np.ndarray:
        out = np.empty(3 * n, dtype=np.float64)
        self.lib.orc_random_cell_centres(self.h, n, out)
        return out.reshape(n, 3)


class OracleModel:
    """The reference sphericalVertexModel restated on the CPU."""

    def __init__(self, pos, rings, counts, vcells, vnbrs, radius):
        self.lib = orc_lib()
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1)
        rings = np.ascontiguousarray(rings, dtype=np.int32)
        counts = np.ascontiguousarray(counts, dtype=np.uint32)
        self.nCells = rings.shape[0]
        self.nVertices = pos.size // 3
        W = rings.shape[1]
        self.h = self.lib.orc_create(self.nCells, self.nVertices, W, pos, rings.reshape(-1), counts,
                                     np.ascontiguousarray(vcells, dtype=np.int32).reshape(-1),
                                     np.ascontiguousarray(vnbrs, dtype=np.int32).reshape(-1), float(radius))

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_destroy(self.h)
            self.h = None

    def set_preferred(self, a0, p0):
        self.lib.orc_set_preferred(self.h, a0, p0)

    def set_preferred_array(self, a0p0):
        self.lib.orc_set_preferred_array(self.h, np.ascontiguousarray(a0p0, dtype=np.float64).reshape(-1))

    def set_kr(self, kr):
        self.lib.orc_set_kr(self.h, kr)

    def set_t1_threshold(self, t):
        self.lib.orc_set_t1_threshold(self.h, t)

    def set_restricted(self, r):
        self.lib.orc_set_restricted(self.h, int(bool(r)))

    def compute_geometry(self):
        self.lib.orc_compute_geometry(self.h)

    def compute_forces(self):
        self.lib.orc_compute_forces(self.h)

    def energy(self) -> float:
        return self.lib.orc_energy(self.h)

    def move(self, disp, scale=1.0):
        self.lib.orc_move(self.h, np.ascontiguousarray(disp, dtype=np.float64).reshape(-1), scale)

    def brownian_step(self, noise: OracleNoise, T, dt, mu=1.0):
        self.lib.orc_brownian_step(self.h, noise.h, T, dt, mu, None)

    def brownian_step_noise(self, xi, T, dt, mu=1.0):
        self.lib.orc_brownian_step_noise(self.h, np.ascontiguousarray(xi, dtype=np.float64).reshape(-1), T, dt, mu)

    def spp_step_noise(self, r, dt, mu, v0, tau):
        self.lib.orc_spp_step_noise(self.h, np.ascontiguousarray(r, dtype=np.float64).reshape(-1), dt, mu, v0, tau)

    def vicsek_step_noise(self, uw, dt, mu, v0, eta, tau):
        self.lib.orc_vicsek_step_noise(self.h, np.ascontiguousarray(uw, dtype=np.float64).reshape(-1), dt, mu, v0,
                                       eta, tau)

    def set_directors(self, d):
        self.lib.orc_set_directors(self.h, np.ascontiguousarray(d, dtype=np.float64).reshape(-1))

    def directors(self):
        out = np.empty(3 * self.lib.orc_num_vertices(self.h), dtype=np.float64)
        self.lib.orc_get_directors(self.h, out)
        return out.reshape(-1, 3)

    def init_directors(self, noise):
        self.lib.orc_init_directors(self.h, noise.h)

    def _vec(self, name, n):
        out = np.empty(3 * n, dtype=np.float64)
        getattr(self.lib, "orc_get_" + name)(self.h, out)
        return out.reshape(n, 3)

    def positions(self):
        return self._vec("positions", self.lib.orc_num_vertices(self.h))

    def set_positions(self, p):
        self.lib.orc_set_positions(self.h, np.ascontiguousarray(p, dtype=np.float64).reshape(-1))

    def forces(self):
        return self._vec("forces", self.nVertices)

    def velocities(self):
        return self._vec("velocities", self.nVertices)

    def set_velocities(self, v):
        self.lib.orc_set_velocities(self.h, np.ascontiguousarray(v, dtype=np.float64).reshape(-1))

    def cell_positions(self):
        return self._vec("cell_positions", self.nCells)

    def area_perimeter(self):
        out = np.empty(2 * self.nCells, dtype=np.float64)
        self.lib.orc_get_area_perimeter(self.h, out)
        return out.reshape(self.nCells, 2)

    def rings(self, W=32):
        out = np.empty(self.nCells * W, dtype=np.int32)
        cnt = np.empty(self.nCells, dtype=np.uint32)
        if self.lib.orc_get_rings(self.h, out, W, cnt) != 0:
            raise RuntimeError("ring wider than requested width")
        return out.reshape(self.nCells, W), cnt

    def vertex_cells(self):
        out = np.empty(3 * self.nVertices, dtype=np.int32)
        self.lib.orc_get_vertex_cells(self.h, out)
        return out.reshape(-1, 3)

    def vertex_neighbors(self):
        out = np.empty(3 * self.nVertices, dtype=np.int32)
        self.lib.orc_get_vertex_neighbors(self.h, out)
        return out.reshape(-1, 3)

    def flips(self, clear=True):
        n = self.lib.orc_flip_count(self.h)
        out = np.empty(2 * n, dtype=np.int32)
        if n:
            self.lib.orc_get_flips(self.h, out)
        if clear:
            self.lib.orc_clear_flips(self.h)
        return out.reshape(n, 2)

    def excess_area(self):
        return self.lib.orc_last_excess_area(self.h)

    def fallback_count(self):
        return self.lib.orc_fallback_count(self.h)


class OracleFire:
    def __init__(self, dt=0.01, alpha_start=0.99, dt_max=0.1, dt_inc=1.05, dt_dec=0.95, alpha_dec=0.9,
                 n_min=5, force_cutoff=1e-7, alpha_min=0.0, max_iterations=1000):
        self.lib = orc_lib()
        self.h = self.lib.orc_fire_create(dt, alpha_start, dt_max, dt_inc, dt_dec, alpha_dec, n_min,
                                          force_cutoff, alpha_min, max_iterations)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.orc_fire_destroy(self.h)
            self.h = None

    def minimize(self, model: OracleModel, criterion=0) -> int:
        return self.lib.orc_fire_minimize(model.h, self.h, criterion)

    def iterate(self, model: OracleModel, count: int):
        self.lib.orc_fire_iterate(model.h, self.h, count)

    def fire_step(self, model: OracleModel):
        """fireStepCPU alone (no integration, no iteration count)."""
        self.lib.orc_fire_step(model.h, self.h)

    def state(self):
        out = np.empty(7, dtype=np.float64)
        self.lib.orc_fire_state(self.h, out)
        return dict(dt=out[0], alpha=out[1], power=out[2], force_rms_over_n=out[3], max_force=out[4],
                    n_since=int(out[5]), iterations=int(out[6]))


def vv_step(model: OracleModel, dt: float) -> None:
    """velocityVerlet::integrateEOMCPU at dt (forces must be current)."""
    orc_lib().orc_vv_step(model.h, dt)


def oracle_cell_list(points, a, radius, nmax=2):
    lib = orc_lib()
    pts = np.ascontiguousarray(points, dtype=np.float64).reshape(-1)
    npnt = pts.size // 3
    nside = C.c_int()
    h = C.c_double()
    lib.orc_cell_list_dims(a, radius, C.byref(nside), C.byref(h))
    total = nside.value ** 3
    nm = C.c_int(nmax)
    bins = np.empty(npnt, dtype=np.int32)
    counts = np.empty(total, dtype=np.uint32)
    # first pass discovers Nmax; the slot table is then sized for it
    cap = total * max(nmax, 1)
    idx = np.empty(cap, dtype=np.int32)
    rc = lib.orc_cell_list(pts, npnt, a, radius, C.byref(nm), bins, counts, idx, cap)
    if rc != 0:
        cap = total * nm.value
        idx = np.empty(cap, dtype=np.int32)
        nm2 = C.c_int(nmax)
        rc = lib.orc_cell_list(pts, npnt, a, radius, C.byref(nm2), bins, counts, idx, cap)
        assert rc == 0
    return dict(nside=nside.value, h=h.value, nmax=nm.value, bins=bins, counts=counts,
                idx=idx[: total * nm.value].reshape(total, nm.value))


# ---- the reference compiled from its sources (only where oracle/ref has been built) -------------
_ref = None


def ref_available() -> bool:
    return os.path.exists(LIBREF)


def ref_lib():
    global _ref
    if _ref is None:
        lib = C.CDLL(LIBREF)
        vp = C.c_void_p
        _sig(lib, "ref_create", vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double)
        _sig(lib, "ref_destroy", None, vp)
        _sig(lib, "ref_bd_setup", None, vp, C.c_int, C.c_double, C.c_double, C.c_double)
        _sig(lib, "ref_fire_setup", None, vp, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
             C.c_double, C.c_int, C.c_double, C.c_double, C.c_int)
        _sig(lib, "ref_fire_iterations", C.c_int, vp)
        _sig(lib, "ref_fire_force", C.c_double, vp)
        _sig(lib, "ref_fire_set_max_iterations", None, vp, C.c_int)
        _sig(lib, "ref_steps", None, vp, C.c_int)
        _sig(lib, "ref_set_restricted", None, vp, C.c_int)
        _sig(lib, "ref_set_preferred", None, vp, C.c_double, C.c_double)
        _sig(lib, "ref_compute_forces", None, vp)
        _sig(lib, "ref_compute_geometry", None, vp)
        _sig(lib, "ref_energy", C.c_double, vp)
        _sig(lib, "ref_num_cells", C.c_int, vp)
        _sig(lib, "ref_num_vertices", C.c_int, vp)
        _sig(lib, "ref_ring_width", C.c_int, vp)
        _sig(lib, "ref_radius", C.c_double, vp)
        _sig(lib, "ref_active_setup", None, vp, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
             C.c_double)
        _sig(lib, "ref_dynamics", None, _dp, _dp, C.c_int, C.c_double, C.c_double, C.c_double,
             C.POINTER(C.c_double), C.POINTER(C.c_double))
        _sig(lib, "ref_log_spaced", None, C.c_int, C.c_double, C.c_int,
             np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS"))
        for n in ("positions", "forces", "velocities", "cell_positions", "area_perimeter", "directors"):
            _sig(lib, "ref_get_" + n, None, vp, _dp)
        _sig(lib, "ref_set_positions", None, vp, _dp)
        _sig(lib, "ref_get_rings", C.c_int, vp, _ip, C.c_int, _up)
        _sig(lib, "ref_get_vertex_cells", None, vp, _ip)
        _sig(lib, "ref_get_vertex_neighbors", None, vp, _ip)
        _sig(lib, "ref_cell_list", C.c_int, vp, C.POINTER(C.c_int), _up, _ip, C.c_long)
        _sig(lib, "ref_neighbor_list", C.c_int, _dp, C.c_int, C.c_double, C.c_double, C.c_int, _up, _ip, _dp, _dp,
             C.c_long)
        _ref = lib
    return _ref


class RefModel:
    """The unmodified reference sphericalVertexModel (CPU branch), built from its sources."""

    def __init__(self, n_cells, seed, a0=1.0, p0=3.8, kr=1.0, t1=0.1):
        self.lib = ref_lib()
        self.h = self.lib.ref_create(n_cells, seed, a0, p0, kr, t1)
        self.nCells = self.lib.ref_num_cells(self.h)
        self.nVertices = self.lib.ref_num_vertices(self.h)
        self.radius = self.lib.ref_radius(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            self.lib.ref_destroy(self.h)
            self.h = None

    def bd_setup(self, bd_seed, T, dt, mu=1.0):
        self.lib.ref_bd_setup(self.h, bd_seed, T, dt, mu)

    def fire_setup(self, dt=0.01, alpha_start=0.99, dt_max=0.1, dt_inc=1.05, dt_dec=0.95, alpha_dec=0.9,
                   n_min=5, force_cutoff=1e-7, alpha_min=0.0, max_iterations=1000):
        self.lib.ref_fire_setup(self.h, dt, alpha_start, dt_max, dt_inc, dt_dec, alpha_dec, n_min, force_cutoff,
                                alpha_min, max_iterations)

    def steps(self, n):
        self.lib.ref_steps(self.h, n)

    def active_setup(self, kind, seed, dt, mu, v0, eta, tau):
        """kind 0: sphericalSelfPropelledParticle, 1: sphericalVectorialVicsek (its noise seeded)."""
        self.lib.ref_active_setup(self.h, kind, seed, dt, mu, v0, eta, tau)

    def directors(self):
        return self._vec("directors", self.nVertices)

    def set_restricted(self, r):
        self.lib.ref_set_restricted(self.h, int(bool(r)))

    def set_preferred(self, a0, p0):
        self.lib.ref_set_preferred(self.h, a0, p0)

    def compute_forces(self):
        self.lib.ref_compute_forces(self.h)

    def compute_geometry(self):
        self.lib.ref_compute_geometry(self.h)

    def energy(self):
        return self.lib.ref_energy(self.h)

    def _vec(self, name, n):
        out = np.empty(3 * n, dtype=np.float64)
        getattr(self.lib, "ref_get_" + name)(self.h, out)
        return out.reshape(n, 3)

    def positions(self):
        return self._vec("positions", self.nVertices)

    def set_positions(self, p):
        self.lib.ref_set_positions(self.h, np.ascontiguousarray(p, dtype=np.float64).reshape(-1))

    def forces(self):
        return self._vec("forces", self.nVertices)

    def velocities(self):
        return self._vec("velocities", self.nVertices)

    def cell_positions(self):
        return self._vec("cell_positions", self.nCells)

    def area_perimeter(self):
        out = np.empty(2 * self.nCells, dtype=np.float64)
        self.lib.ref_get_area_perimeter(self.h, out)
        return out.reshape(self.nCells, 2)

    def rings(self, W=32):
        out = np.empty(self.nCells * W, dtype=np.int32)
        cnt = np.empty(self.nCells, dtype=np.uint32)
        if self.lib.ref_get_rings(self.h, out, W, cnt) != 0:
            raise RuntimeError("ring wider than requested width")
        return out.reshape(self.nCells, W), cnt

    def ring_width(self):
        return self.lib.ref_ring_width(self.h)

    def vertex_cells(self):
        out = np.empty(3 * self.nVertices, dtype=np.int32)
        self.lib.ref_get_vertex_cells(self.h, out)
        return out.reshape(-1, 3)

    def vertex_neighbors(self):
        out = np.empty(3 * self.nVertices, dtype=np.int32)
        self.lib.ref_get_vertex_neighbors(self.h, out)
        return out.reshape(-1, 3)

    def cell_list(self):
        nside = C.c_int()
        # bound the slot table generously: counts per bin are small on a sphere shell
        R = self.radius + 2.5
        n = int(np.floor(2 * R / 1.0))
        n -= n % 2
        total = n ** 3
        cap = total * 64
        counts = np.empty(total, dtype=np.uint32)
        idx = np.empty(cap, dtype=np.int32)
        nmax = self.lib.ref_cell_list(self.h, C.byref(nside), counts, idx, cap)
        assert nmax > 0 and nside.value == n
        return dict(nside=n, nmax=nmax, counts=counts, idx=idx[: total * nmax].reshape(total, nmax))

    def topology(self, W=None):
        """Arrays in the form OracleModel (and the GPU path) take them."""
        W = W or self.ring_width()
        rings, cnt = self.rings(W)
        return dict(pos=self.positions(), rings=rings, counts=cnt, vcells=self.vertex_cells(),
                    vnbrs=self.vertex_neighbors(), radius=self.radius)


def dynamics(initial, current, radius, fraction=1.0, cutoff=0.5, reference=False):
    """computeMSD and computeOverlapFunction (src/analysis/dynamicalFeatures.cpp:17-53);
    reference=True runs the reference's own class from oracle/_ref."""
    a = np.ascontiguousarray(initial, dtype=np.float64).reshape(-1)
    b = np.ascontiguousarray(current, dtype=np.float64).reshape(-1)
    msd, ov = C.c_double(), C.c_double()
    if reference:
        ref_lib().ref_dynamics(a, b, a.size // 3, fraction, radius, cutoff, C.byref(msd), C.byref(ov))
    else:
        orc_lib().orc_dynamics(a, b, a.size // 3, fraction, radius, cutoff, C.byref(msd), C.byref(ov))
    return msd.value, ov.value


def log_spaced(first_save, exponent, count, reference=False):
    """The first `count` save steps of logSpacedIntegers (inc/simpleUtilities.h:5-41);
    reference=True runs the reference's own class from oracle/_ref."""
    if reference:
        out = np.empty(count, dtype=np.int64)
        ref_lib().ref_log_spaced(int(first_save), float(exponent), int(count), out)
        return out
    out = np.empty(count, dtype=np.int32)
    orc_lib().orc_log_spaced(int(first_save), float(exponent), int(count), out)
    return out


def neighbor_list(points, range_, radius, sub_grid=1, reference=False):
    """neighborList::computeCPU (src/utilities/neighborList.cpp:96-151): (Nmax, counts, indices,
    displacements, distances) with the per-point arrays of width Nmax.  reference=True runs the
    reference's own class from oracle/_ref instead of the restatement."""
    p = np.ascontiguousarray(points, dtype=np.float64).reshape(-1)
    n = p.size // 3
    cap = n * 8
    while True:
        npp = np.empty(n, dtype=np.uint32)
        idx = np.empty(cap, dtype=np.int32)
        vec = np.empty(3 * cap)
        dist = np.empty(cap)
        if reference:
            nm = ref_lib().ref_neighbor_list(p, n, range_, radius, sub_grid, npp, idx, vec, dist, cap)
        else:
            nm = orc_lib().orc_neighbor_list(p, n, range_, radius, sub_grid, 4, npp, idx, vec, dist, cap)
        if nm > 0:
            e = n * nm
            return nm, npp, idx[:e].reshape(n, nm), vec[:3 * e].reshape(n, nm, 3), dist[:e].reshape(n, nm)
        cap = n * (-nm)
