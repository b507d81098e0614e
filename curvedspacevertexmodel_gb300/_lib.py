"""ctypes binding of libsvm.so (the C ABI in include/svm.h).

The library is built in-tree by curvedspacevertexmodel_gb300.build; there is no fallback: if the
library is missing, or no CUDA device is present when a model is created, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
# SVM_LIBRARY selects another build of the same library (e.g. one compiled with other flags).
LIBPATH = os.environ.get("SVM_LIBRARY") or os.path.join(PKG, "libsvm.so")

SVM_OK = 0
SVM_ERR_ARG = 1
SVM_ERR_CUDA = 2
SVM_ERR_HULL = 3
SVM_ERR_DEVICE = 4
SVM_ERR_NO_DEVICE = 5
SVM_DEV_RING_OVERFLOW = 0x1
SVM_DEV_T1_OVERFLOW = 0x2
SVM_DEV_CELLLIST_OVERFLOW = 0x4
SVM_DEV_BAD_TOPOLOGY = 0x8
SVM_DEV_T1_TIMEOUT = 0x10
SVM_NOISE_PHILOX = 0
SVM_NOISE_BUFFER = 1
PHASES = ("corners", "cells", "fallback", "force", "t1_apply", "move")
SVM_PROFILE_ONLY = 0x100
SVM_NOALLOC_MAX_CELLS = 2097152
SVM_FIRE_RMS_OVER_N = 0
SVM_FIRE_MAX_FORCE = 1
SVM_PRECISION_FP64 = 0
SVM_PRECISION_MIXED = 1
SVM_PRECISION_FP64_VECTOR = 2

def _nullable(ptr):
    """An ndpointer type that also accepts None (NULL) for optional outputs."""
    class Nullable(ptr):
        @classmethod
        def from_param(cls, obj):
            return None if obj is None else ptr.from_param(obj)
    return Nullable


dp = _nullable(np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS"))
ip = _nullable(np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS"))
up = _nullable(np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS"))
fp = _nullable(np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS"))
vp = C.c_void_p
i32 = C.c_int
f64 = C.c_double
u64 = C.c_uint64
pvp = C.POINTER(C.c_void_p)

# name -> (restype, argtypes); every entry point declared in include/svm.h
SIGNATURES = {
    "svm_status_string": (C.c_char_p, [i32]),
    "svm_device_count": (i32, [C.POINTER(i32)]),
    "svm_random_cell_centres": (i32, [i32, i32, dp]),
    "svm_random_vertex_directors": (i32, [i32, i32, dp, i32, dp]),
    "svm_topology_from_points": (i32, [dp, i32, pvp]),
    "svm_topology_from_points_gpu": (i32, [dp, i32, vp, pvp]),
    "svm_topology_from_triangles": (i32, [dp, i32, ip, i32, pvp]),
    "svm_topology_sizes": (i32, [vp, C.POINTER(i32), C.POINTER(i32), C.POINTER(i32)]),
    "svm_topology_get": (i32, [vp, dp, ip, i32, up, ip, ip]),
    "svm_topology_free": (None, [vp]),
    "svm_model_create": (i32, [i32, i32, i32, f64, vp, pvp]),
    "svm_model_destroy": (i32, [vp]),
    "svm_model_set_topology": (i32, [vp, dp, ip, i32, up, ip, ip]),
    "svm_model_set_preferred_parameters": (i32, [vp, f64, f64]),
    "svm_model_set_preferred_array": (i32, [vp, dp]),
    "svm_model_set_scalar_model_parameter": (i32, [vp, f64]),
    "svm_model_set_t1_threshold": (i32, [vp, f64]),
    "svm_model_set_restricted_motion": (i32, [vp, i32]),
    "svm_model_set_precision": (i32, [vp, i32]),
    "svm_model_compute_geometry": (i32, [vp]),
    "svm_model_compute_forces": (i32, [vp]),
    "svm_model_compute_energy": (i32, [vp, C.POINTER(f64)]),
    "svm_model_move_particles": (i32, [vp, vp, f64]),
    "svm_model_move_particles_host": (i32, [vp, dp, f64]),
    "svm_model_enforce_topology": (i32, [vp]),
    "svm_model_get_positions": (i32, [vp, dp]),
    "svm_model_set_positions": (i32, [vp, dp]),
    "svm_model_get_forces": (i32, [vp, dp]),
    "svm_model_get_velocities": (i32, [vp, dp]),
    "svm_model_set_velocities": (i32, [vp, dp]),
    "svm_model_get_area_perimeter": (i32, [vp, dp]),
    "svm_model_get_cell_positions": (i32, [vp, dp]),
    "svm_model_get_rings": (i32, [vp, ip, i32, up]),
    "svm_model_set_ring_headroom": (i32, [vp, i32]),
    "svm_model_ring_info": (i32, [vp, ip]),
    "svm_model_get_vertex_cells": (i32, [vp, ip]),
    "svm_model_get_vertex_neighbors": (i32, [vp, ip]),
    "svm_model_status": (i32, [vp, C.POINTER(i32)]),
    "svm_model_area_check": (i32, [vp, C.POINTER(f64), C.POINTER(f64), C.POINTER(i32)]),
    "svm_model_take_flips": (i32, [vp, ip, i32, C.POINTER(i32)]),
    "svm_model_synchronize": (i32, [vp]),
    "svm_model_t1_clocks": (i32, [vp, i32, _nullable(np.ctypeslib.ndpointer(dtype=np.uint64, flags="C_CONTIGUOUS"))]),
    "svm_model_fallback_count": (i32, [vp, C.POINTER(i32)]),
    "svm_model_set_t1_blocks": (i32, [vp, i32]),
    "svm_model_set_t1_wait_limit": (i32, [vp, i32]),
    "svm_model_t1_stats": (i32, [vp, ip]),
    "svm_model_profile": (i32, [vp, i32]),
    "svm_model_profile_read": (i32, [vp, dp, ip]),
    "svm_model_device_positions": (i32, [vp, pvp]),
    "svm_model_stream": (i32, [vp, pvp]),
    "svm_energy_noalloc": (i32, [vp, vp, f64, i32, vp, vp]),
    "svm_brownian_step": (i32, [vp, f64, f64, f64, i32, vp, u64]),
    "svm_brownian_step_host_noise": (i32, [vp, f64, f64, f64, dp]),
    "svm_model_set_dynamics_reference": (i32, [vp]),
    "svm_model_dynamics": (i32, [vp, f64, f64, C.POINTER(f64), C.POINTER(f64)]),
    "svm_neighbor_list_create": (i32, [f64, f64, i32, i32, i32, vp, pvp]),
    "svm_neighbor_list_destroy": (i32, [vp]),
    "svm_neighbor_list_compute": (i32, [vp, vp, i32]),
    "svm_neighbor_list_compute_model": (i32, [vp, vp]),
    "svm_neighbor_list_get": (i32, [vp, C.POINTER(i32), _nullable(np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")),
                                     _nullable(np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")), dp, dp,
                                     C.c_long]),
    "svm_model_set_directors": (i32, [vp, dp]),
    "svm_model_get_directors": (i32, [vp, dp]),
    "svm_spp_step": (i32, [vp, f64, f64, f64, f64, i32, dp, u64]),
    "svm_vicsek_step": (i32, [vp, f64, f64, f64, f64, f64, i32, dp, u64]),
    "svm_brownian_step_io": (i32, [vp, f64, f64, f64, u64, dp, dp, C.POINTER(f64)]),
    "svm_brownian_run": (i32, [vp, f64, f64, f64, u64, i32]),
    "svm_fire_create": (i32, [vp, f64, f64, f64, f64, f64, f64, i32, f64, f64, i32, pvp]),
    "svm_fire_destroy": (i32, [vp]),
    "svm_fire_minimize": (i32, [vp, i32, C.POINTER(i32), C.POINTER(f64)]),
    "svm_fire_state": (i32, [vp, dp]),
    "svm_fire_step": (i32, [vp]),
    "svm_softf64_check": (i32, [C.c_longlong, C.c_ulonglong, vp]),
    "svm_velocity_verlet_step": (i32, [vp, f64, i32]),
    "svm_vv_half": (i32, [vp, f64]),
    "svm_reduce_dots": (i32, [vp, dp]),
    "svm_fire_set_max_iterations": (i32, [vp, i32]),
    "svm_cell_list_create": (i32, [f64, f64, i32, i32, vp, pvp]),
    "svm_cell_list_destroy": (i32, [vp]),
    "svm_cell_list_compute_model": (i32, [vp, vp]),
    "svm_cell_list_compute": (i32, [vp, vp, i32]),
    "svm_cell_list_get": (i32, [vp, C.POINTER(i32), C.POINTER(i32), up, ip, C.c_long]),
    "svm_cell_list_bins": (i32, [vp, ip]),
    "svm_batch_create": (i32, [i32, ip, ip, i32, dp, vp, pvp]),
    "svm_batch_replicas": (i32, [vp, C.POINTER(i32)]),
    "svm_batch_offsets": (i32, [vp, ip, ip]),
    "svm_batch_set_temperatures": (i32, [vp, dp]),
    "svm_batch_energies": (i32, [vp, dp]),
    "svm_batch_area_check": (i32, [vp, dp, dp, ip]),
    "svm_batch_autotune": (i32, [vp, i32, i32, i32, i32, i32]),
    "svm_batch_block_sizes": (i32, [vp, ip, C.POINTER(i32)]),
    "svm_tuner_create": (i32, [i32, i32, i32, i32, i32, vp, pvp]),
    "svm_tuner_destroy": (i32, [vp]),
    "svm_tuner_begin": (i32, [vp]),
    "svm_tuner_end": (i32, [vp]),
    "svm_tuner_record": (i32, [vp, C.c_float]),
    "svm_tuner_parameter": (i32, [vp, C.POINTER(i32)]),
    "svm_tuner_sampling_complete": (i32, [vp, C.POINTER(i32)]),
    "svm_tuner_timing_data": (i32, [vp, ip, fp, i32, C.POINTER(i32)]),
    "svm_mlp_create": (i32, [C.c_uint, vp, pvp]),
    "svm_mlp_destroy": (i32, [vp]),
    "svm_mlp_parameter_count": (i32, [C.POINTER(i32)]),
    "svm_mlp_set_weights": (i32, [vp, fp]),
    "svm_mlp_get_weights": (i32, [vp, fp]),
    "svm_mlp_set_output_scale": (i32, [vp, f64]),
    "svm_mlp_features": (i32, [vp, vp, vp]),
    "svm_mlp_gradient": (i32, [vp, vp, vp, i32, fp, C.POINTER(f64)]),
    "svm_mlp_train": (i32, [vp, vp, vp, vp, i32, i32, C.c_float, C.POINTER(f64)]),
    "svm_mlp_predict": (i32, [vp, vp, i32, vp]),
    "svm_mlp_warm_start": (i32, [vp, vp]),
}


class SVMError(RuntimeError):
    def __init__(self, fn: str, code: int):
        super().__init__(f"{fn} failed with status {code}")
        self.code = code


_lib = None


def lib():
    """Loads libsvm.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIBPATH):
            raise RuntimeError(f"{LIBPATH} is missing: build it with `python -m curvedspacevertexmodel_gb300.build`")
        L = C.CDLL(LIBPATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def call(name: str, *args) -> None:
    rc = getattr(lib(), name)(*args)
    if rc != SVM_OK:
        raise SVMError(name, rc)


def device_count() -> int:
    n = C.c_int(0)
    lib().svm_device_count(C.byref(n))
    return n.value
