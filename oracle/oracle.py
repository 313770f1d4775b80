"""ORACLE wrapper -- test infrastructure only.

ctypes bindings for ``oracle/_build/liboracle.so`` (the C++ restatement of
Merzbild.jl's hot path in ``oracle.cpp``).  Only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may import
this module.  The product package never does.

Indices exposed here follow the reference: ``ParticleIndexer`` fields and the
``index`` / ``buffer`` entries are 1-based, empty groups are ``(0, -1)``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

K_B = 1.380649e-23

SPLIT_MID, SPLIT_MEAN = 1, 2
INIT_MINMAX, INIT_MINMAX_SYM, INIT_C = 1, 2, 3
BOUNDS_INHERIT, BOUNDS_RECOMPUTE = 1, 2

TAG_NCOLL, TAG_CAND, TAG_CONVECT, TAG_MERGE, TAG_SAMPLE, TAG_SAMPLE_CELL = 0, 1, 2, 3, 4, 5

_lib = None


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (idempotent)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        d, i32, i64, u64, vp = C.c_double, C.c_int32, C.c_int64, C.c_uint64, C.c_void_p
        P = C.POINTER
        sig = {
            "orc_create": (vp, [i64, i32]),
            "orc_destroy": (None, [vp]),
            "orc_set_mass": (None, [vp, P(d)]),
            "orc_load_interactions": (None, [vp, P(d), P(d), P(d)]),
            "orc_get_interaction": (None, [vp, i32, i32, P(d)]),
            "orc_pv_create": (None, [vp, i32, i64]),
            "orc_set_cell_offset": (None, [vp, i64]),
            "orc_pv_resize": (None, [vp, i32, i64]),
            "orc_pv_length": (i64, [vp, i32]),
            "orc_pv_get": (None, [vp, i32, P(d), P(i64), P(i64), P(i64), P(i64)]),
            "orc_pv_set": (None, [vp, i32, i64, P(d), P(i64), P(i64), P(i64), i64]),
            "orc_pia_get": (None, [vp, P(i64), P(i64), P(C.c_uint8)]),
            "orc_pia_set": (None, [vp, P(i64), P(i64), P(C.c_uint8)]),
            "orc_cf_get": (None, [vp, i32, i32, P(d), P(i64)]),
            "orc_cf_set_smax": (None, [vp, i32, i32, P(d)]),
            "orc_estimate_sigma_g_w_max": (None, [vp, P(d), P(d), i32, d]),
            "orc_estimate_sigma_g_w_max_single": (d, [vp, i32, i32, d, d, d, d]),
            "orc_ntc": (None, [vp, i32, i32, i64, d, d, u64, u64, d, i32]),
            "orc_ntc_cells": (None, [vp, i32, i32, d, P(d), u64, u64, d, i32, i32]),
            "orc_swpm": (None, [vp, i32, i64, d, d, d, u64, u64]),
            "orc_swpm_cells": (None, [vp, i32, d, d, P(d), u64, u64]),
            "orc_compute_props": (None, [vp, i32, P(i32), i32, d, P(d), P(d), P(d), P(d), P(d), P(d), P(d), i32]),
            "orc_avg_props": (None, [i64, P(d), P(d), d]),
            "orc_convect": (None, [vp, i32, d, i64, d, P(d), d, u64, u64, i32, i32]),
            "orc_convect_surf": (None, [vp, i32, d, i64, d, P(d), d, u64, u64, P(d)]),
            "orc_surf_update": (None, [P(d), i32, d, P(d), i32]),
            "orc_surf_scale": (None, [P(d), d, d, P(d)]),
            "orc_grid": (None, [d, i64, d, P(d)]),
            "orc_sort": (None, [vp, i32, d, i64, d]),
            "orc_squash": (None, [vp, i32]),
            "orc_restore_ordering": (None, [vp, i32]),
            "orc_delete_particle_end": (None, [vp, i32, i64]),
            "orc_delete_particle_end_group": (None, [vp, i32, i64, i32]),
            "orc_map_cont_index": (i64, [vp, i32, i64, i64]),
            "orc_indexer_new_particle": (None, [vp, i32, i64]),
            "orc_octree_create": (vp, [i32, i32, i32, i64, i64]),
            "orc_octree_destroy": (None, [vp]),
            "orc_octree_init": (None, [vp, vp, i32, i64]),
            "orc_octree_split": (None, [vp, vp, i32, i64]),
            "orc_octree_bin_props": (None, [vp, vp, i32, i64]),
            "orc_octree_compute_v_mean": (None, [vp, vp, i32, i64, i64]),
            "orc_octree_bounds_recompute": (None, [vp, vp, i32, i64, i64, i64]),
            "orc_octree_summary": (None, [vp, P(d)]),
            "orc_octree_pis": (None, [vp, i64, P(i64)]),
            "orc_octree_bins": (None, [vp, i64, P(d)]),
            "orc_merge_octree": (None, [vp, vp, i32, i64, i64, d, i64, d, u64, u64]),
            "orc_check_pia": (i32, [vp, i32, P(i64)]),
            "orc_check_unique_index": (i64, [vp, i32]),
            "orc_check_unique_buffer": (i64, [vp, i32]),
            "orc_sample_particles_equal_weight": (None, [vp, i32, i64, i64, d, d, P(d), u64, u64, i32, P(d)]),
            "orc_sample_grid_ndens": (None, [vp, i32, d, i64, d, d, d, d, u64, u64, P(d)]),
            "orc_stream_draws": (None, [u64, C.c_uint32, C.c_uint32, u64, C.c_uint32, C.c_uint32, i64, P(d)]),
            "orc_philox": (None, [P(C.c_uint32), P(C.c_uint32), P(C.c_uint32)]),
            "orc_tgamma": (d, [d]),
            "orc_com_g_scatter": (None, [vp, i32, i32, P(d), P(d), u64, i32, P(d)]),
            "orc_collide_vhs": (None, [vp, i32, i32, i64, i64, i64, d, u64, i32]),
            "orc_compute_octant": (i32, [P(d), P(d)]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _p(a, ctype=C.c_double):
    return a.ctypes.data_as(C.POINTER(ctype))


def surf_update(q, element, w, v, reflected):
    """update_surface_incident! / update_surface_reflected! (surface_props.jl:78-134)
    on q (2 x 11, see Oracle.convect_surf)."""
    v = np.ascontiguousarray(v, float)
    lib().orc_surf_update(_p(q), element, w, _p(v), 1 if reflected else 0)


def surf_scale(q, mass, dt, inv_areas):
    """surface_props_scale! (surface_props.jl:149-166) on q (2 x 11)."""
    ia = np.ascontiguousarray(inv_areas, float)
    lib().orc_surf_scale(_p(q), mass, dt, _p(ia))


def stream_draws(seed, tag, sub, step, a, b, n):
    out = np.zeros(n)
    lib().orc_stream_draws(seed, tag, sub, step, a, b, n, _p(out))
    return out


def philox(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().orc_philox(_p(c, C.c_uint32), _p(k, C.c_uint32), _p(o, C.c_uint32))
    return o


def grid(L, nx, wall_offset=1e-12):
    """Grid1DUniform(L, nx) fields (dx, inv_dx, min_x, max_x, L)."""
    out = np.zeros(5)
    lib().orc_grid(L, nx, wall_offset, _p(out))
    return dict(dx=out[0], inv_dx=out[1], min_x=out[2], max_x=out[3], L=out[4], n_cells=nx)


class Oracle:
    """One simulation state: ParticleVectors, ParticleIndexerArray,
    interactions and collision factors for n_cells x n_species."""

    def __init__(self, n_cells: int, n_species: int, mass):
        self.L = lib()
        self.n_cells = int(n_cells)
        self.n_species = int(n_species)
        self.h = self.L.orc_create(self.n_cells, self.n_species)
        self.mass = np.asarray(mass, dtype=np.float64).reshape(self.n_species)
        self.L.orc_set_mass(self.h, _p(self.mass))

    def __del__(self):
        try:
            if self.h:
                self.L.orc_destroy(self.h)
                self.h = None
        except Exception:
            pass

    # --- setup -------------------------------------------------------------
    def load_interactions(self, vhs_d, vhs_o, vhs_Tref):
        ns = self.n_species
        arr = [np.ascontiguousarray(np.broadcast_to(np.asarray(a, float), (ns, ns))) for a in (vhs_d, vhs_o, vhs_Tref)]
        self.L.orc_load_interactions(self.h, _p(arr[0]), _p(arr[1]), _p(arr[2]))

    def interaction(self, s1, s2):
        r = np.zeros(8)
        self.L.orc_get_interaction(self.h, s1, s2, _p(r))
        keys = ["m_r", "mu1", "mu2", "vhs_d", "vhs_o", "vhs_Tref", "vhs_muref", "vhs_factor"]
        return dict(zip(keys, r))

    def set_cell_offset(self, offset):
        """Global id of cell 1 minus one, for a slab of a larger grid: the
        collision, convection and merge streams of cell c are keyed on the
        global cell c - 1 + offset."""
        self.L.orc_set_cell_offset(self.h, int(offset))

    def pv_create(self, s, np_):
        self.L.orc_pv_create(self.h, s, np_)

    def pv_resize(self, s, np_):
        self.L.orc_pv_resize(self.h, s, np_)

    def pv_get(self, s):
        n = self.L.orc_pv_length(self.h, s)
        parts = np.zeros((n, 7))
        index = np.zeros(n, np.int64)
        cell = np.zeros(n, np.int64)
        buf = np.zeros(n, np.int64)
        nb = np.zeros(1, np.int64)
        if n:
            self.L.orc_pv_get(self.h, s, _p(parts), _p(index, C.c_int64), _p(cell, C.c_int64), _p(buf, C.c_int64),
                              _p(nb, C.c_int64))
        return dict(particles=parts, index=index, cell=cell, buffer=buf, nbuffer=int(nb[0]))

    def pv_set(self, s, particles, index=None, cell=None, buffer=None, nbuffer=None):
        particles = np.ascontiguousarray(particles, dtype=np.float64).reshape(-1, 7)
        n = particles.shape[0]
        index = np.arange(1, n + 1, dtype=np.int64) if index is None else np.ascontiguousarray(index, np.int64)
        cell = np.zeros(n, np.int64) if cell is None else np.ascontiguousarray(cell, np.int64)
        buffer = np.arange(n, 0, -1, dtype=np.int64) if buffer is None else np.ascontiguousarray(buffer, np.int64)
        nbuffer = 0 if nbuffer is None else nbuffer
        self.L.orc_pv_set(self.h, s, n, _p(particles), _p(index, C.c_int64), _p(cell, C.c_int64),
                          _p(buffer, C.c_int64), nbuffer)

    def pia_get(self):
        ind = np.zeros((self.n_species, self.n_cells, 7), np.int64)
        nt = np.zeros(self.n_species, np.int64)
        cg = np.zeros(self.n_species, np.uint8)
        self.L.orc_pia_get(self.h, _p(ind, C.c_int64), _p(nt, C.c_int64), _p(cg, C.c_uint8))
        return ind, nt, cg

    def pia_set(self, indexer, n_total, contiguous=None):
        ind = np.ascontiguousarray(indexer, np.int64).reshape(self.n_species, self.n_cells, 7)
        nt = np.ascontiguousarray(n_total, np.int64).reshape(self.n_species)
        cg = np.ones(self.n_species, np.uint8) if contiguous is None else np.ascontiguousarray(contiguous, np.uint8)
        self.L.orc_pia_set(self.h, _p(ind, C.c_int64), _p(nt, C.c_int64), _p(cg, C.c_uint8))

    def set_particles_simple(self, s, cells, particles):
        """Place particles (n x 7) for one species, cell ids 1-based, grouped
        by cell in the given order; builds a ParticleVector with identity index
        and a contiguous group1-only indexer (like sample_particles_equal_weight!)."""
        particles = np.asarray(particles, float).reshape(-1, 7)
        cells = np.asarray(cells, np.int64)
        order = np.argsort(cells, kind="stable")
        particles = particles[order]
        cells = cells[order]
        n = particles.shape[0]
        self.pv_set(s, particles, cell=cells, nbuffer=0)
        ind, nt, cg = self.pia_get()
        cnt = np.bincount(cells - 1, minlength=self.n_cells)[: self.n_cells].astype(np.int64)
        pos = 1 + np.concatenate(([0], np.cumsum(cnt)[:-1]))
        ind[s] = np.array([0, 0, -1, 0, 0, -1, 0])
        nz = cnt > 0
        ind[s, nz, 0] = cnt[nz]
        ind[s, nz, 1] = pos[nz]
        ind[s, nz, 2] = pos[nz] + cnt[nz] - 1
        ind[s, nz, 3] = cnt[nz]
        nt[s] = n
        cg[s] = 1
        self.pia_set(ind, nt, cg)
        return order

    def logical(self, s):
        """Particles of species s in logical order: cells in order, group1
        then group2 (what pv[i] returns for i over the indexer)."""
        pv = self.pv_get(s)
        ind, _, _ = self.pia_get()
        p = ind[s]
        # per cell: positions start1..end1 (those >= 1), then start2..end2 when
        # n_group2 > 0, cells in order
        len1 = np.maximum(p[:, 2] - p[:, 1] + 1, 0)
        len2 = np.where(p[:, 6] > 0, np.maximum(p[:, 5] - p[:, 4] + 1, 0), 0)
        lens = np.column_stack([len1, len2]).reshape(-1)
        starts = np.column_stack([p[:, 1], p[:, 4]]).reshape(-1)
        total = int(lens.sum())
        seg = np.repeat(np.arange(lens.size), lens)
        first = np.concatenate(([0], np.cumsum(lens)[:-1]))
        pos = starts[seg] + (np.arange(total) - first[seg])
        cells = seg // 2 + 1
        keep = pos >= 1
        pos, cells = pos[keep], cells[keep]
        rows = pv["particles"][pv["index"][pos - 1] - 1]
        return rows.reshape(-1, 7), cells.astype(np.int64)

    def cf_get(self, s1, s2):
        smax = np.zeros(self.n_cells)
        cnt = np.zeros((self.n_cells, 5), np.int64)
        self.L.orc_cf_get(self.h, s1, s2, _p(smax), _p(cnt, C.c_int64))
        return smax, cnt

    def cf_set_smax(self, s1, s2, smax):
        sm = np.ascontiguousarray(np.broadcast_to(np.asarray(smax, float), (self.n_cells,)))
        self.L.orc_cf_set_smax(self.h, s1, s2, _p(sm))

    def estimate_sigma_g_w_max(self, T_list, Fnum, mult=1.0):
        T = np.ascontiguousarray(np.broadcast_to(np.asarray(T_list, float), (self.n_species,)))
        F = np.atleast_1d(np.asarray(Fnum, float))
        per = 1 if F.size > 1 else 0
        F = np.ascontiguousarray(np.broadcast_to(F, (self.n_species,)) if per else F)
        self.L.orc_estimate_sigma_g_w_max(self.h, _p(T), _p(F), per, mult)

    def estimate_single(self, s1, s2, T1, T2, Fnum, mult=1.0):
        return self.L.orc_estimate_sigma_g_w_max_single(self.h, s1, s2, T1, T2, Fnum, mult)

    # --- hot path ------------------------------------------------------------
    def ntc(self, s1, s2, cell, dt, V, seed, step, dw_tol=1e-16, equal_weight=False):
        self.L.orc_ntc(self.h, s1, s2, cell, dt, V, seed, step, dw_tol, 1 if equal_weight else 0)

    def ntc_cells(self, s1, s2, dt, V, seed, step, dw_tol=1e-16, equal_weight=False, nthreads=1):
        Va = None
        if V is not None:
            Va = np.ascontiguousarray(np.broadcast_to(np.asarray(V, float), (self.n_cells,)))
        self.L.orc_ntc_cells(self.h, s1, s2, dt, _p(Va) if Va is not None else None, seed, step, dw_tol,
                             1 if equal_weight else 0, nthreads)

    def swpm(self, s, cell, G, dt, V, seed, step):
        """swpm! of one cell (1-based), collision_swpm.jl:201-288."""
        self.L.orc_swpm(self.h, s, cell, G, dt, V, seed, step)

    def swpm_cells(self, s, G, dt, V, seed, step):
        Va = None
        if V is not None:
            Va = np.ascontiguousarray(np.broadcast_to(np.asarray(V, float), (self.n_cells,)))
        self.L.orc_swpm_cells(self.h, s, G, dt, _p(Va) if Va is not None else None, seed, step)

    def compute_props(self, mode=0, powers=(), Tref=300.0, inv_V=None, nthreads=1):
        ns, nc = self.n_species, self.n_cells
        pw = np.ascontiguousarray(powers, np.int32)
        nm = len(pw)
        lpa = np.zeros(ns)
        npa = np.zeros((ns, nc))
        n = np.zeros((ns, nc))
        v = np.zeros((ns, nc, 3))
        T = np.zeros((ns, nc))
        mom = np.zeros((ns, nc, max(nm, 1)))
        iv = None if inv_V is None else np.ascontiguousarray(np.broadcast_to(np.asarray(inv_V, float), (nc,)))
        self.L.orc_compute_props(self.h, mode, _p(pw, C.c_int32) if nm else None, nm, Tref,
                                 _p(iv) if iv is not None else None, _p(lpa), _p(npa), _p(n), _p(v), _p(T),
                                 _p(mom), nthreads)
        return dict(lpa=lpa, np=npa, n=n, v=v, T=T, moments=mom[:, :, :nm])

    def convect(self, s, L, nx, walls, dt, seed, step, compute_cell=False, wall_offset=1e-12, nthreads=1):
        w = np.ascontiguousarray(walls, float).reshape(10)
        self.L.orc_convect(self.h, s, L, nx, wall_offset, _p(w), dt, seed, step, 1 if compute_cell else 0, nthreads)

    def sort(self, s, L=None, nx=None, wall_offset=1e-12):
        if L is None:
            self.L.orc_sort(self.h, s, -1.0, 0, wall_offset)
        else:
            self.L.orc_sort(self.h, s, float(L), int(nx), wall_offset)

    def squash(self, s):
        self.L.orc_squash(self.h, s)

    def restore_ordering(self, s):
        self.L.orc_restore_ordering(self.h, s)

    def delete_particle_end(self, s, cell):
        self.L.orc_delete_particle_end(self.h, s, cell)

    def map_cont_index(self, s, cell, i):
        """map_cont_index (particles.jl:364-366), cell 1-based, i 0-based"""
        return self.L.orc_map_cont_index(self.h, s, cell, i)

    def indexer_new_particle(self, s, cell):
        """update_particle_indexer_new_particle! (particles.jl:426-433)"""
        self.L.orc_indexer_new_particle(self.h, s, cell)

    def delete_particle_end_group(self, s, cell, group):
        """delete_particle_end_group1! / _group2! (particles.jl:501-566)"""
        self.L.orc_delete_particle_end_group(self.h, s, cell, group)

    def convect_surf(self, s, L, nx, walls, dt, seed, step, wall_offset=1e-12):
        """convect_particles! with SurfProps (convection_1D.jl:176-206): returns
        the scaled surface sums of this call as (2 elements, 11 quantities):
        np, flux_incident, flux_reflected, force xyz, normal_pressure, shear
        xyz, kinetic_energy_flux."""
        w = np.ascontiguousarray(walls, float)
        out = np.zeros(22)
        self.L.orc_convect_surf(self.h, s, L, nx, wall_offset, _p(w), dt, seed, step, _p(out))
        return out.reshape(2, 11)

    def merge_octree(self, octree, s, cell, target, L=None, nx=0, seed=0, step=0, wall_offset=1e-12):
        self.L.orc_merge_octree(self.h, octree.h, s, cell, target, -1.0 if L is None else float(L), nx, wall_offset,
                                seed, step)

    def check_pia(self, s):
        bad = np.zeros(1, np.int64)
        ok = self.L.orc_check_pia(self.h, s, _p(bad, C.c_int64))
        return bool(ok), int(bad[0])

    def check_unique_index(self, s):
        r = self.L.orc_check_unique_index(self.h, s)
        return (r == 0), int(r)

    def check_unique_buffer(self, s):
        r = self.L.orc_check_unique_buffer(self.h, s)
        return (r == 0), int(r)

    def sample_equal_weight(self, s, cell, n, T, Fnum, box=(0, 1, 0, 1, 0, 1), seed=0, step=0, distribution=0,
                            v0=(0, 0, 0)):
        b = np.ascontiguousarray(box, float)
        v = np.ascontiguousarray(v0, float)
        self.L.orc_sample_particles_equal_weight(self.h, s, cell, n, T, Fnum, _p(b), seed, step, distribution, _p(v))

    def sample_grid_ndens(self, s, L, nx, ndens, T, Fnum, seed=0, step=0, wall_offset=1e-12, v0=(0.0, 0.0, 0.0)):
        v = np.ascontiguousarray(v0, float).reshape(3)
        self.L.orc_sample_grid_ndens(self.h, s, L, nx, wall_offset, ndens, T, Fnum, seed, step, _p(v))

    def com_g_scatter(self, s1, s2, p1, p2, seed=0, scatter=True):
        a = np.ascontiguousarray(p1, float).copy()
        b = np.ascontiguousarray(p2, float).copy()
        out = np.zeros(4)
        self.L.orc_com_g_scatter(self.h, s1, s2, _p(a), _p(b), seed, 1 if scatter else 0, _p(out))
        return a, b, out[:3].copy(), float(out[3])

    def collide_vhs(self, s1, s2, cell, pos_i, pos_k, dw_tol=1e-16, seed=0, equal_weight=False):
        self.L.orc_collide_vhs(self.h, s1, s2, cell, pos_i, pos_k, dw_tol, seed, 1 if equal_weight else 0)


def compute_octant(v, mid):
    a = np.ascontiguousarray(v, float)
    b = np.ascontiguousarray(mid, float)
    return int(lib().orc_compute_octant(_p(a), _p(b)))


class Octree:
    """OctreeN2Merge (merging_octree_N2.jl:235-246)."""

    def __init__(self, split=SPLIT_MID, init_bin_bounds=INIT_MINMAX, bin_bounds_compute=BOUNDS_INHERIT,
                 max_Nbins=4096, max_depth=10):
        self.L = lib()
        self.h = self.L.orc_octree_create(split, init_bin_bounds, bin_bounds_compute, max_Nbins, max_depth)

    def __del__(self):
        try:
            if self.h:
                self.L.orc_octree_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def init(self, orc, s, cell):
        self.L.orc_octree_init(orc.h, self.h, s, cell)

    def split_bin(self, orc, s, bin_id):
        self.L.orc_octree_split(orc.h, self.h, s, bin_id)

    def compute_bin_props(self, orc, s, bin_id):
        self.L.orc_octree_bin_props(orc.h, self.h, s, bin_id)

    def compute_v_mean(self, orc, s, bs, be):
        self.L.orc_octree_compute_v_mean(orc.h, self.h, s, bs, be)

    def bin_bounds_recompute(self, orc, s, bin_id, bs, be):
        self.L.orc_octree_bounds_recompute(orc.h, self.h, s, bin_id, bs, be)

    def summary(self):
        r = np.zeros(6)
        self.L.orc_octree_summary(self.h, _p(r))
        return dict(Nbins=int(r[0]), n_particles=int(r[1]), total_post_merge_np=int(r[2]), vel_middle=r[3:6].copy())

    def pis(self, n):
        out = np.zeros(n, np.int64)
        self.L.orc_octree_pis(self.h, n, _p(out, C.c_int64))
        return out

    def bins(self, nbins):
        out = np.zeros((nbins, 18))
        self.L.orc_octree_bins(self.h, nbins, _p(out))
        return dict(np=out[:, 0].astype(np.int64), w=out[:, 1], depth=out[:, 2].astype(np.int64),
                    can_be_refined=out[:, 3] > 0, bin_start=out[:, 4].astype(np.int64),
                    bin_end=out[:, 5].astype(np.int64), vmin=out[:, 6:9], vmax=out[:, 9:12], v_mean=out[:, 12:15],
                    x_mean=out[:, 15:18])
