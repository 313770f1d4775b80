"""ctypes binding of libmerzgpu.so (include/merzgpu.h).

The library is loaded from merzgpu/lib/libmerzgpu.so only; there is no CPU
fallback.  Loading fails loudly if the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libmerzgpu.so")

MZ_MAX_SPECIES = 4
MZ_OK, MZ_E_ARG, MZ_E_CUDA, MZ_E_CAPACITY, MZ_E_TIMEOUT, MZ_E_STATE, MZ_E_NOMEM = range(7)
NTC_EQUAL_WEIGHT = 1
CONVECT_COMPUTE_CELL = 1
PROPS_ALL, PROPS_MOMENTS, PROPS_SORTED = 0, 1, 2

d, i32, i64, u64, vp = C.c_double, C.c_int32, C.c_int64, C.c_uint64, C.c_void_p
P = C.POINTER


class Interaction(C.Structure):
    _fields_ = [(n, d) for n in ("m_r", "mu1", "mu2", "vhs_d", "vhs_o", "vhs_Tref", "vhs_muref", "vhs_factor")]


class ParticleIndexer(C.Structure):
    _fields_ = [(n, i64) for n in ("n_local", "start1", "end1", "n_group1", "start2", "end2", "n_group2")]


class CollisionFactors(C.Structure):
    _fields_ = [("n1", i64), ("n2", i64), ("sigma_g_w_max", d), ("n_coll", i64), ("n_coll_performed", i64),
                ("n_eq_w_coll_performed", i64)]


class Grid1D(C.Structure):
    _fields_ = [("L", d), ("n_cells", i64), ("dx", d), ("inv_dx", d), ("min_x", d), ("max_x", d)]


class Walls1D(C.Structure):
    _fields_ = [("T", d * 2), ("v", (d * 3) * 2), ("accommodation", d * 2),
                ("reflection_v_sq", (d * MZ_MAX_SPECIES) * 2)]


class OctreeParams(C.Structure):
    _fields_ = [("split", i32), ("init_bin_bounds", i32), ("bin_bounds_compute", i32), ("max_Nbins", i32),
                ("max_depth", i32)]


class Counters(C.Structure):
    _fields_ = [(n, C.c_ulonglong) for n in ("candidates", "accepted", "splits", "merges", "wall_hits")]


class NcAttribute(C.Structure):
    _fields_ = [("name", C.c_char_p), ("type", i32), ("count", i32), ("values", vp)]


class Request(C.Structure):
    _fields_ = [("count", i64 * MZ_MAX_SPECIES), ("T", d * MZ_MAX_SPECIES), ("Fnum", d), ("V", d), ("n_steps", i64),
                ("seed", u64)]


class RequestResult(C.Structure):
    _fields_ = [("id", i64), ("state", i32), ("reserved", i32), ("steps_done", i64), ("np", i64 * MZ_MAX_SPECIES),
                ("n", d * MZ_MAX_SPECIES), ("v", (d * 3) * MZ_MAX_SPECIES), ("T", d * MZ_MAX_SPECIES)]


MZ_REQ_QUEUED, MZ_REQ_RUNNING, MZ_REQ_DONE = 0, 1, 2


class StepPlan(C.Structure):
    _fields_ = [("dims", i32), ("collide", i32), ("equal_weight", i32), ("props", i32), ("avg_start", i64),
                ("n_avg", i64), ("dt", d), ("dw_tol", d), ("step0", u64), ("use_graph", i32), ("big_cell", i32),
                ("grid", Grid1D), ("walls", Walls1D), ("launches", i32), ("hit_queue_capacity", i64),
                ("merge_threshold", i64), ("merge_target", i64), ("octree", OctreeParams), ("split_lanes", i32)]


_SIGS = {
    "mz_version": (i32, []),
    "mz_ctx_create": (i32, [i32, P(vp)]),
    "mz_ctx_destroy": (i32, [vp]),
    "mz_ctx_synchronize": (i32, [vp]),
    "mz_last_error": (i32, [vp, C.c_char_p, C.c_size_t]),
    "mz_ctx_stream": (i32, [vp, P(vp)]),
    "mz_timer_start": (i32, [vp]),
    "mz_timer_stop": (i32, [vp, P(d)]),
    "mz_ctx_flush_l2": (i32, [vp]),
    "mz_ctx_set_kernel_timing": (i32, [vp, i32]),
    "mz_kernel_timing": (i32, [vp, i32, C.c_char_p, C.c_size_t, P(d), P(i64), P(i32)]),
    "mz_launch_count": (i32, [vp, P(i64)]),
    "mz_domain_create": (i32, [vp, i64, i32, P(i64), P(vp)]),
    "mz_domain_destroy": (i32, [vp]),
    "mz_domain_reserve": (i32, [vp, i32, i64]),
    "mz_domain_info": (i32, [vp, i32, P(i64), P(i64), P(i64)]),
    "mz_set_species": (i32, [vp, P(d)]),
    "mz_set_interactions": (i32, [vp, P(Interaction)]),
    "mz_set_cell_volumes": (i32, [vp, P(d)]),
    "mz_set_seed": (i32, [vp, u64]),
    "mz_set_cell_rng": (i32, [vp, P(u64), P(C.c_uint32), P(C.c_uint32)]),
    "mz_upload_particles": (i32, [vp, i32, i64, P(d), P(d), P(d), P(i32)]),
    "mz_upload_particles_indexed": (i32, [vp, i32, i64, P(d), P(d), P(d), P(ParticleIndexer)]),
    "mz_download_particles": (i32, [vp, i32, i64, P(d), P(d), P(d), P(i32), P(i64)]),
    "mz_get_indexer": (i32, [vp, i32, P(ParticleIndexer), P(i64)]),
    "mz_set_collision_factors": (i32, [vp, i32, i32, P(d)]),
    "mz_get_collision_factors": (i32, [vp, i32, i32, P(CollisionFactors)]),
    "mz_ntc": (i32, [vp, i32, i32, d, i64, i64, u64, i32, d]),
    "mz_props_create": (i32, [vp, i32, P(i32), d, i32, P(vp)]),
    "mz_props_destroy": (i32, [vp]),
    "mz_compute_props": (i32, [vp, vp, i32]),
    "mz_avg_props": (i32, [vp, vp, d]),
    "mz_clear_props": (i32, [vp]),
    "mz_props_download": (i32, [vp, P(d), P(d), P(d), P(d), P(d), P(d)]),
    "mz_convect_1d": (i32, [vp, i32, P(Grid1D), P(Walls1D), d, u64, i32]),
    "mz_sort": (i32, [vp, i32, P(Grid1D), P(i64)]),
    "mz_squash": (i32, [vp, i32]),
    "mz_merge_octree_n2": (i32, [vp, i32, i64, i64, i64, i64, P(OctreeParams), P(Grid1D), u64, P(i64)]),
    "mz_sample_cells": (i32, [vp, i32, P(i64), P(d), P(d), P(d), d, P(d), i32, u64, P(d), P(d)]),
    "mz_sample_grid_ndens": (i32, [vp, i32, P(Grid1D), d, d, d, u64, P(d)]),
    "mz_step": (i32, [vp, P(StepPlan), i64, vp, vp]),
    "mz_get_counters": (i32, [vp, P(Counters), i32]),
    "mz_step_autotune": (i32, [vp, P(StepPlan), i64, P(i32), P(i32)]),
    "mz_surf_props_create": (i32, [vp, P(vp)]),
    "mz_surf_props_destroy": (i32, [vp]),
    "mz_surf_props_clear": (i32, [vp]),
    "mz_surf_avg_props": (i32, [vp, vp, d]),
    "mz_surf_props_download": (i32, [vp, P(d), P(d), P(d), P(d), P(d), P(d), P(d)]),
    "mz_convect_1d_surf": (i32, [vp, i32, P(Grid1D), P(Walls1D), d, u64, i32, vp]),
    "mz_step_set_surface": (i32, [vp, vp, vp]),
    "mz_sort_keys_noalloc": (i32, [vp, vp, i64, i32, vp, vp]),
    "mz_sincos_2pi": (i32, [vp, i64, P(u64), P(d), P(d)]),
    "mz_server_create": (i32, [vp, i32, P(d), P(Interaction), d, i64, P(i64), P(vp)]),
    "mz_server_destroy": (i32, [vp]),
    "mz_server_submit": (i32, [vp, P(Request), P(i64)]),
    "mz_server_step": (i32, [vp, P(i64), P(i64), P(i64)]),
    "mz_server_step_many": (i32, [vp, i64, P(i64), P(i64), P(i64), P(i64)]),
    "mz_server_result": (i32, [vp, i64, P(RequestResult)]),
    "mz_server_retired": (i32, [vp, i64, P(i64), P(i64)]),
    "mz_server_info": (i32, [vp, P(i64), P(i64)]),
    "mz_server_set_lane_split": (i32, [vp, i64]),
    "mz_server_set_hbm_headroom": (i32, [vp, i64]),
    "mz_check_indexing": (i32, [vp, i32, i32, P(i32), P(i64)]),
    "mz_slab_extract": (i32, [vp, i32, P(Grid1D), i64, P(i64), P(i64)]),
    "mz_slab_fetch": (i32, [vp, i32, P(d), P(d)]),
    "mz_slab_insert": (i32, [vp, i32, P(Grid1D), i64, P(d), i64, P(d), i64]),
    "mz_set_indexer": (i32, [vp, i32, P(ParticleIndexer), i64]),
    "mz_swpm": (i32, [vp, i32, d, d, i64, i64, u64]),
    "mz_props_snapshot": (i32, [vp, i32, P(d)]),
    "mz_props_snapshot_wait": (i32, [vp, i32]),
    "mz_host_alloc": (i32, [vp, C.c_size_t, P(vp)]),
    "mz_host_free": (i32, [vp]),
    "mz_nc_props_create": (i32, [C.c_char_p, P(C.c_char_p), i32, P(C.c_char_p), i32, i32, i32, i32, P(i32), i32,
                                 P(NcAttribute), i32, vp, P(vp)]),
    "mz_nc_surf_create": (i32, [C.c_char_p, P(C.c_char_p), i32, P(C.c_char_p), i32, i32, i32, P(NcAttribute), i32, vp,
                                P(vp)]),
    "mz_nc_props_write": (i32, [vp, vp, d, i32]),
    "mz_nc_props_write_host": (i32, [vp, P(d), P(d), P(d), P(d), P(d), P(d), i32, d, i32]),
    "mz_nc_surf_write": (i32, [vp, vp, d, i32]),
    "mz_nc_surf_write_host": (i32, [vp, P(d), P(d), P(d), P(d), P(d), P(d), P(d), d, i32]),
    "mz_nc_flush": (i32, [vp]),
    "mz_nc_records": (i32, [vp, P(i64)]),
    "mz_nc_close": (i32, [vp]),
    "mz_nc_last_error": (i32, [vp, C.c_char_p, C.c_size_t]),
}
NOALLOC_MAX_CELLS = 262144

_lib = None


class MerzError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"merzgpu error {code}: {msg}")
        self.code = code


def lib():
    """Load libmerzgpu.so; raises if it was not built (no fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"libmerzgpu.so not built at {LIB_PATH}; run merzgpu.build.build()")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def exported_symbols():
    return list(_SIGS)


def ptr(a, ctype=d):
    if a is None:
        return None
    return a.ctypes.data_as(P(ctype))


def check(rc, ctx_handle=None):
    if rc != MZ_OK:
        msg = ""
        if ctx_handle:
            buf = C.create_string_buffer(1024)
            lib().mz_last_error(ctx_handle, buf, 1024)
            msg = buf.value.decode(errors="replace")
        raise MerzError(rc, msg)


def f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None:
        a = a.reshape(shape)
    return a
