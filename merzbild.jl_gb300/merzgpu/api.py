"""Host-side mirror of Merzbild.jl's hot-path interface on top of libmerzgpu.

Names follow the reference (``ntc``, ``ntc_equal_weight``, ``convect_particles``,
``sort_particles``, ``compute_props``, ``merge_octree_N2_based``, ...).  Device
state lives in a :class:`Domain` (the ParticleVector of every species, the
ParticleIndexerArray and the CollisionFactors array of one simulation).
Cells and slots are 0-based here.

Randomness: :class:`PhiloxRNG` replaces the reference's ``rng`` argument.  It
holds a seed and a step counter; every call draws from streams keyed on
(seed, step, cell, particle), so the time loop advances ``rng.step`` once per
time step (``rng.next_step()``).
"""
from __future__ import annotations

import ctypes as C
import math
import time
import tomllib
import weakref
from dataclasses import dataclass
from fractions import Fraction

import numpy as np

from . import _lib as L
from ._lib import check, f64, lib, ptr

K_B = 1.380649e-23  # constants.jl:4
Q_E = 1.602176634e-19


def _fma(a, b, c):
    """Correctly rounded a*b + c (math.fma is not in Python 3.12)."""
    return float(Fraction(a) * Fraction(b) + Fraction(c))


# --------------------------------------------------------------------- data
@dataclass
class Species:  # Species, particles.jl:31-36
    name: str
    mass: float
    charge: float = 0.0

    @property
    def charge_div_mass(self):
        return Q_E * self.charge / self.mass


def load_species_data(species_filename, species_names):
    """load_species_data (particles.jl:580-608)."""
    if isinstance(species_names, str):
        species_names = [species_names]
    with open(species_filename, "rb") as f:
        data = tomllib.load(f)
    return [Species(n, float(data[n]["mass"]), float(data[n]["charge"])) for n in species_names]


@dataclass
class Interaction:  # Interaction, collision_utils.jl:73-82
    m_r: float
    mu1: float
    mu2: float
    vhs_d: float
    vhs_o: float
    vhs_Tref: float
    vhs_muref: float
    vhs_factor: float

    def c_struct(self):
        return L.Interaction(self.m_r, self.mu1, self.mu2, self.vhs_d, self.vhs_o, self.vhs_Tref, self.vhs_muref,
                             self.vhs_factor)


def compute_vhs_factor(vhs_Tref, vhs_d, vhs_o, m_r):
    """compute_vhs_factor (collision_utils.jl:98-101)."""
    return math.pi * vhs_d ** 2 * (2 * K_B * vhs_Tref / m_r) ** (vhs_o - 0.5) / math.gamma(2.5 - vhs_o)


def compute_mu_ref(m_r, vhs_o, vhs_Tref, vhs_d):
    """compute_mu_ref (collision_utils.jl:218-223)."""
    num = 30.0 * math.sqrt(m_r * K_B * vhs_Tref)
    den = 4.0 * math.sqrt(math.pi) * (5.0 - 2.0 * vhs_o) * (7.0 - 2.0 * vhs_o) * vhs_d * vhs_d
    return num / den


def interactions_from_vhs(species_data, vhs_table):
    """Build the n_species x n_species Interaction table like
    load_interaction_data (collision_utils.jl:159-202) from a mapping
    ``{"A,B": (vhs_d, vhs_o, vhs_Tref)}``."""
    names = [s.name for s in species_data]
    ns = len(names)
    out = [[None] * ns for _ in range(ns)]
    for i, a in enumerate(names):
        for k, b in enumerate(names):
            if i < k:
                continue
            rec = vhs_table.get(f"{a},{b}") or vhs_table[f"{b},{a}"]
            d_, o_, tr = (rec["vhs_d"], rec["vhs_o"], rec["vhs_Tref"]) if isinstance(rec, dict) else rec
            mi, mk = species_data[i].mass, species_data[k].mass
            m_r = mi * mk / (mi + mk)
            mu1, mu2 = mi / (mi + mk), mk / (mi + mk)
            muref = compute_mu_ref(0.5 * (mi + mk), o_, tr, d_)
            fac = compute_vhs_factor(tr, d_, o_, m_r)
            out[i][k] = Interaction(m_r, mu1, mu2, d_, o_, tr, muref, fac)
            out[k][i] = Interaction(m_r, mu2, mu1, d_, o_, tr, muref, fac)
    return out


def load_interaction_data(interactions_filename, species_data):
    """load_interaction_data (collision_utils.jl:159-202)."""
    with open(interactions_filename, "rb") as f:
        data = tomllib.load(f)
    return interactions_from_vhs(species_data, data)


def estimate_sigma_g_w_max(interaction, species1, species2, T1, T2, Fnum, mult_factor=1.0):
    """estimate_sigma_g_w_max (collision_utils.jl:418-423)."""
    g1 = math.sqrt(2 * T1 * K_B / species1.mass)
    g2 = math.sqrt(2 * T2 * K_B / species2.mass)
    g = 0.5 * (g1 + g2)
    sigma = interaction.vhs_factor * g ** _fma(-2.0, interaction.vhs_o, 1.0)
    return mult_factor * sigma * g * Fnum


def mean_collision_frequency(interaction, species_data, species, n, T):
    """mean_collision_frequency (collisional_props.jl:42-47)."""
    I = interaction[species][species]
    nu = 4.0 * I.vhs_d ** 2 * n
    nu *= math.sqrt(math.pi * K_B * I.vhs_Tref / species_data[species].mass)
    nu *= (T / I.vhs_Tref) ** (1.0 - I.vhs_o)
    return nu


def mean_free_path(interaction, species, n, T):
    """mean_free_path (collisional_props.jl:18-22)."""
    I = interaction[species][species]
    lam = math.sqrt(2.0) * math.pi * I.vhs_d ** 2 * n
    lam *= (I.vhs_Tref / T) ** (I.vhs_o - 0.5)
    return 1.0 / lam


class Grid1DUniform:
    """Grid1DUniform(L, nx; wall_offset=1e-12) (grid_uniform1D.jl:49-86)."""

    def __init__(self, L_, nx, wall_offset=1e-12):
        self.L = float(L_)
        self.n_cells = int(nx)
        self.dx = self.L / self.n_cells
        self.inv_dx = 1.0 / self.dx
        self.min_x = self.dx * wall_offset
        self.max_x = _fma(-self.dx, wall_offset, self.L)
        self.V = np.full(self.n_cells, self.dx)

    def c_struct(self):
        return L.Grid1D(self.L, self.n_cells, self.dx, self.inv_dx, self.min_x, self.max_x)

    def get_cell(self, x):
        return int(math.floor(x * self.inv_dx))


class MaxwellWalls1D:
    """MaxwellWalls1D(species_data, T_l, T_r, vy_l, vy_r, acc_l, acc_r) (boundary_conditions.jl:49-53)."""

    def __init__(self, species_data, T_l, T_r, vy_l, vy_r, accommodation_l, accommodation_r):
        self.T = (float(T_l), float(T_r))
        self.v = ((0.0, float(vy_l), 0.0), (0.0, float(vy_r), 0.0))
        self.accommodation = (float(accommodation_l), float(accommodation_r))
        self.reflection_velocities_sq = [[2 * K_B * T / sd.mass for sd in species_data] for T in self.T]

    def c_struct(self):
        w = L.Walls1D()
        for b in range(2):
            w.T[b] = self.T[b]
            w.accommodation[b] = self.accommodation[b]
            for k in range(3):
                w.v[b][k] = self.v[b][k]
            for s, v in enumerate(self.reflection_velocities_sq[b]):
                w.reflection_v_sq[b][s] = v
        return w

    def as_flat_array(self):
        return [self.T[0], self.T[1], *self.v[0], *self.v[1], self.accommodation[0], self.accommodation[1]]


OctreeBinMidSplit = 1
OctreeInitBinMinMaxVel, OctreeInitBinMinMaxVelSym, OctreeInitBinC = 1, 2, 3
OctreeBinBoundsInherit, OctreeBinBoundsRecompute = 1, 2


class OctreeN2Merge:
    """OctreeN2Merge(split; init_bin_bounds, bin_bounds_compute, max_Nbins, max_depth)
    (merging_octree_N2.jl:235-246)."""

    def __init__(self, split=OctreeBinMidSplit, init_bin_bounds=OctreeInitBinMinMaxVel,
                 bin_bounds_compute=OctreeBinBoundsInherit, max_Nbins=4096, max_depth=10):
        if split != OctreeBinMidSplit:
            raise ValueError("only OctreeBinMidSplit is implemented on the device")
        self.params = L.OctreeParams(split, init_bin_bounds, bin_bounds_compute, max_Nbins, max_depth)


class PhiloxRNG:
    """Counter-based RNG handle: seed + step.  Replaces the reference's rng."""

    def __init__(self, seed=1234, step=0):
        self.seed = int(seed)
        self.step = int(step)

    def next_step(self):
        self.step += 1
        return self.step


# --------------------------------------------------------------------- device objects
class Context:
    """One device and one CUDA stream.  Closing it closes its domains first."""

    def __init__(self, device=0):
        self.h = C.c_void_p()
        self._children = weakref.WeakSet()
        check(lib().mz_ctx_create(device, C.byref(self.h)))

    def close(self):
        if self.h:
            for child in list(self._children):
                child.close()
            lib().mz_ctx_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def synchronize(self):
        check(lib().mz_ctx_synchronize(self.h), self.h)

    def timer_start(self):
        check(lib().mz_timer_start(self.h), self.h)

    def timer_stop(self):
        ms = C.c_double()
        check(lib().mz_timer_stop(self.h, C.byref(ms)), self.h)
        return ms.value

    def flush_l2(self):
        check(lib().mz_ctx_flush_l2(self.h), self.h)

    def set_kernel_timing(self, on):
        check(lib().mz_ctx_set_kernel_timing(self.h, 1 if on else 0), self.h)

    def kernel_timings(self):
        n = C.c_int32()
        check(lib().mz_kernel_timing(self.h, -1, None, 0, None, None, C.byref(n)), self.h)
        out = {}
        for k in range(n.value):
            name = C.create_string_buffer(64)
            ms = C.c_double()
            cnt = C.c_int64()
            check(lib().mz_kernel_timing(self.h, k, name, 64, C.byref(ms), C.byref(cnt), None), self.h)
            out[name.value.decode()] = (ms.value, cnt.value)
        return out

    def launch_count(self):
        n = C.c_int64()
        check(lib().mz_launch_count(self.h, C.byref(n)))
        return n.value


class Domain:
    """ParticleVector per species + ParticleIndexerArray + CollisionFactors
    for n_cells cells, resident on one GPU."""

    def __init__(self, ctx: Context, n_cells, species_data, capacity, interactions=None, seed=1234):
        self.ctx = ctx
        self._children = weakref.WeakSet()
        self.n_cells = int(n_cells)
        self.species_data = list(species_data)
        self.n_species = len(self.species_data)
        cap = np.ascontiguousarray(np.broadcast_to(np.asarray(capacity, np.int64), (self.n_species,)))
        self.h = C.c_void_p()
        check(lib().mz_domain_create(ctx.h, self.n_cells, self.n_species, ptr(cap, C.c_int64), C.byref(self.h)),
              ctx.h)
        ctx._children.add(self)
        m = f64([s.mass for s in self.species_data])
        self._ck(lib().mz_set_species(self.h, ptr(m)))
        if interactions is not None:
            self.set_interactions(interactions)
        self.set_seed(seed)

    def _ck(self, rc):
        check(rc, self.ctx.h)

    def close(self):
        """Destroy the device state; property sets of this domain close first."""
        if self.h:
            for child in list(self._children):
                child.close()
            if self.ctx.h:
                lib().mz_domain_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # setup ---------------------------------------------------------------
    def set_interactions(self, interactions):
        ns = self.n_species
        arr = (L.Interaction * (ns * ns))()
        for s2 in range(ns):
            for s1 in range(ns):
                arr[s1 + ns * s2] = interactions[s1][s2].c_struct()
        self.interactions = interactions
        self._ck(lib().mz_set_interactions(self.h, arr))

    def set_cell_volumes(self, V):
        v = None if V is None else f64(np.broadcast_to(np.asarray(V, float), (self.n_cells,)))
        self._ck(lib().mz_set_cell_volumes(self.h, ptr(v)))

    def set_seed(self, seed):
        self._ck(lib().mz_set_seed(self.h, int(seed)))

    def set_cell_rng(self, seeds=None, rids=None, step_offsets=None):
        s = None if seeds is None else np.ascontiguousarray(seeds, np.uint64)
        r = None if rids is None else np.ascontiguousarray(rids, np.uint32)
        o = None if step_offsets is None else np.ascontiguousarray(step_offsets, np.uint32)
        self._ck(lib().mz_set_cell_rng(self.h, ptr(s, C.c_uint64), ptr(r, C.c_uint32), ptr(o, C.c_uint32)))

    def reserve(self, species, capacity):
        self._ck(lib().mz_domain_reserve(self.h, species, int(capacity)))

    def info(self, species=0):
        cap, nt, hw = C.c_int64(), C.c_int64(), C.c_int64()
        self._ck(lib().mz_domain_info(self.h, species, C.byref(cap), C.byref(nt), C.byref(hw)))
        return dict(capacity=cap.value, n_total=nt.value, high_water=hw.value)

    # particles -----------------------------------------------------------
    def upload(self, species, w, v, x, cell):
        w = f64(w)
        n = w.shape[0]
        v = f64(v, (n, 3))
        x = f64(x, (n, 3))
        cell = np.ascontiguousarray(cell, np.int32)
        self._ck(lib().mz_upload_particles(self.h, species, n, ptr(w), ptr(v), ptr(x), ptr(cell, C.c_int32)))

    def upload_indexed(self, species, w, v, x, indexer):
        """Raw slots + explicit indexer rows (n_local, start1, end1, n_group1,
        start2, end2, n_group2), 0-based."""
        w = f64(w)
        n = w.shape[0]
        v = f64(v, (n, 3))
        x = f64(x, (n, 3))
        ind = (L.ParticleIndexer * self.n_cells)()
        for c in range(self.n_cells):
            ind[c] = L.ParticleIndexer(*[int(a) for a in indexer[c]])
        self._ck(lib().mz_upload_particles_indexed(self.h, species, n, ptr(w), ptr(v), ptr(x), ind))

    def download(self, species):
        """Particles in logical order: (w, v, x, cell)."""
        nt = C.c_int64()
        self._ck(lib().mz_get_indexer(self.h, species, None, C.byref(nt)))
        n = nt.value
        w = np.zeros(n)
        v = np.zeros((n, 3))
        x = np.zeros((n, 3))
        cell = np.zeros(n, np.int32)
        self._ck(lib().mz_download_particles(self.h, species, n, ptr(w), ptr(v), ptr(x), ptr(cell, C.c_int32),
                                             C.byref(nt)))
        return w, v, x, cell

    def indexer(self, species):
        arr = (L.ParticleIndexer * self.n_cells)()
        nt = C.c_int64()
        self._ck(lib().mz_get_indexer(self.h, species, arr, C.byref(nt)))
        out = np.array([[getattr(arr[c], f) for f, _ in L.ParticleIndexer._fields_] for c in range(self.n_cells)],
                       np.int64)
        return out, nt.value

    # validators (particles.jl:805-1025) -----------------------------------
    def _check(self, species, mode):
        ok, detail = C.c_int32(), C.c_int64()
        self._ck(lib().mz_check_indexing(self.h, int(species), int(mode), C.byref(ok), C.byref(detail)))
        return bool(ok.value), int(detail.value)

    def check_pia_is_correct(self, species):
        """(True, 0), or (False, first bad cell 1-based), or (False, 0) for a wrong n_total."""
        return self._check(species, 0)

    def check_unique_index(self, species):
        """(True, 0), or (False, n_index / -n_index / -1) as the reference returns."""
        return self._check(species, 1)

    def check_unique_buffer(self, species):
        return self._check(species, 2)

    def count_disordered_particles(self, species, use_offset=True):
        return self._check(species, 3 if use_offset else 4)[1]

    def set_indexer(self, species, indexer, n_total):
        """Write indexer rows (n_local, start1, end1, n_group1, start2, end2,
        n_group2), 0-based, as given (mz_set_indexer)."""
        ind = (L.ParticleIndexer * self.n_cells)()
        for c in range(self.n_cells):
            ind[c] = L.ParticleIndexer(*[int(a) for a in indexer[c]])
        self._ck(lib().mz_set_indexer(self.h, int(species), ind, int(n_total)))

    # collisions ----------------------------------------------------------
    def set_sigma_g_w_max(self, s1, s2, values):
        v = f64(np.broadcast_to(np.asarray(values, float), (self.n_cells,)))
        self._ck(lib().mz_set_collision_factors(self.h, s1, s2, ptr(v)))

    def collision_factors(self, s1, s2):
        arr = (L.CollisionFactors * self.n_cells)()
        self._ck(lib().mz_get_collision_factors(self.h, s1, s2, arr))
        return dict(
            sigma_g_w_max=np.array([arr[c].sigma_g_w_max for c in range(self.n_cells)]),
            n1=np.array([arr[c].n1 for c in range(self.n_cells)]),
            n2=np.array([arr[c].n2 for c in range(self.n_cells)]),
            n_coll=np.array([arr[c].n_coll for c in range(self.n_cells)]),
            n_coll_performed=np.array([arr[c].n_coll_performed for c in range(self.n_cells)]),
            n_eq_w_coll_performed=np.array([arr[c].n_eq_w_coll_performed for c in range(self.n_cells)]),
        )

    def ntc(self, s1, s2, dt, step, cells=None, equal_weight=False, dw_tol=1e-16):
        cb, ce = (0, self.n_cells) if cells is None else cells
        flags = L.NTC_EQUAL_WEIGHT if equal_weight else 0
        self._ck(lib().mz_ntc(self.h, s1, s2, float(dt), int(cb), int(ce), int(step), flags, float(dw_tol)))

    def swpm(self, species, G, dt, step, cells=None):
        cb, ce = (0, self.n_cells) if cells is None else cells
        self._ck(lib().mz_swpm(self.h, species, float(G), float(dt), int(cb), int(ce), int(step)))

    # convection / sorting / merging ----------------------------------------
    def convect(self, species, grid, walls, dt, step, compute_cell=False):
        g = grid.c_struct()
        w = walls.c_struct()
        self._ck(lib().mz_convect_1d(self.h, species, C.byref(g), C.byref(w), float(dt), int(step),
                                     L.CONVECT_COMPUTE_CELL if compute_cell else 0))

    # slabs of a larger grid (mz_slab_*) ---------------------------------------
    def slab_extract(self, species, grid, c0):
        """Free the particles that left the slab [c0, c0 + n_cells) of the
        global grid and stage them; returns (to the left, to the right)."""
        g = grid.c_struct()
        nl, nr = C.c_int64(), C.c_int64()
        self._ck(lib().mz_slab_extract(self.h, species, C.byref(g), int(c0), C.byref(nl), C.byref(nr)))
        self._slab_pending = (nl.value, nr.value)
        return nl.value, nr.value

    def slab_fetch(self, species):
        """The staged particles as two (n, 7) arrays of w, vx, vy, vz, x, y, z."""
        nl, nr = self._slab_pending
        left, right = np.empty((nl, 7)), np.empty((nr, 7))
        self._ck(lib().mz_slab_fetch(self.h, species, ptr(left) if nl else None, ptr(right) if nr else None))
        return left, right

    def slab_insert(self, species, grid, c0, from_left, from_right):
        """Add the arrivals from the neighbours and sort the slab by cell."""
        g = grid.c_struct()
        a = np.ascontiguousarray(from_left, np.float64).reshape(-1, 7)
        b = np.ascontiguousarray(from_right, np.float64).reshape(-1, 7)
        self._ck(lib().mz_slab_insert(self.h, species, C.byref(g), int(c0), ptr(a) if a.shape[0] else None,
                                      a.shape[0], ptr(b) if b.shape[0] else None, b.shape[0]))

    def sort(self, species, grid=None, return_index=False):
        out = None
        if return_index:
            nt = C.c_int64()
            self._ck(lib().mz_get_indexer(self.h, species, None, C.byref(nt)))
            out = np.zeros(nt.value, np.int64)
        g = grid.c_struct() if grid is not None else None
        self._ck(lib().mz_sort(self.h, species, C.byref(g) if g is not None else None, ptr(out, C.c_int64)))
        return out

    def squash(self, species):
        self._ck(lib().mz_squash(self.h, species))

    def merge_octree(self, species, octree, target_np, threshold=-1, cells=None, grid=None, step=0):
        cb, ce = (0, self.n_cells) if cells is None else cells
        g = grid.c_struct() if grid is not None else None
        n = C.c_int64()
        self._ck(lib().mz_merge_octree_n2(self.h, species, int(cb), int(ce), int(threshold), int(target_np),
                                          C.byref(octree.params), C.byref(g) if g is not None else None, int(step),
                                          C.byref(n)))
        return n.value

    # sampling --------------------------------------------------------------
    def sample_cells(self, species, counts, T, Fnum, step=0, log10_weight_span=0.0, box=None, distribution=0,
                     v0=None):
        """sample_particles_equal_weight! for every cell at once; v0: the
        velocity offset (vx0, vy0, vz0) of every cell, or one per cell
        (n_cells x 3)."""
        counts = np.ascontiguousarray(np.broadcast_to(np.asarray(counts, np.int64), (self.n_cells,)))
        T = np.asarray(T, float)
        T3 = T3_all = None
        if T.ndim == 0:
            T3_all = f64([T, T, T])
        elif T.shape == (3,):
            T3_all = f64(T)
        else:
            T3 = f64(np.broadcast_to(T.reshape(self.n_cells, -1), (self.n_cells, 3)))
        F = f64(np.broadcast_to(np.asarray(Fnum, float), (self.n_cells,)))
        b = None if box is None else f64(np.broadcast_to(np.asarray(box, float), (self.n_cells, 6)))
        v0c = v0a = None
        if v0 is not None:
            v = np.asarray(v0, float)
            if v.shape == (3,):
                v0a = f64(v)
            else:
                v0c = f64(np.broadcast_to(v.reshape(self.n_cells, 3), (self.n_cells, 3)))
        self._ck(lib().mz_sample_cells(self.h, species, ptr(counts, C.c_int64), ptr(T3), ptr(T3_all), ptr(F),
                                       float(log10_weight_span), ptr(b), int(distribution), int(step), ptr(v0c),
                                       ptr(v0a)))

    def sample_grid_ndens(self, species, grid, ndens, T, Fnum, step=0, v0=None):
        g = grid.c_struct()
        v = None if v0 is None else f64(np.asarray(v0, float).reshape(3))
        self._ck(lib().mz_sample_grid_ndens(self.h, species, C.byref(g), float(ndens), float(T), float(Fnum),
                                            int(step), ptr(v)))

    # fused -----------------------------------------------------------------
    def step(self, plan, n_steps, inst=None, avg=None):
        self._ck(lib().mz_step(self.h, C.byref(plan), int(n_steps), inst.h if inst else None,
                               avg.h if avg else None))

    def set_step_surface(self, inst=None, avg=None):
        """mz_step_set_surface: fused 1-D steps sample the walls into inst (and
        average into avg from plan.avg_start on)."""
        self._ck(lib().mz_step_set_surface(self.h, inst.h if inst else None, avg.h if avg else None))

    def autotune(self, plan, trial_steps=2):
        """mz_step_autotune: time each fused-step mapping on real steps (the
        state advances) and keep the fastest; returns (lanes, big_cell)."""
        lanes, big = C.c_int32(), C.c_int32()
        self._ck(lib().mz_step_autotune(self.h, C.byref(plan), int(trial_steps), C.byref(lanes), C.byref(big)))
        return lanes.value, big.value

    def counters(self, reset=False):
        c = L.Counters()
        self._ck(lib().mz_get_counters(self.h, C.byref(c), 1 if reset else 0))
        return {f: getattr(c, f) for f, _ in L.Counters._fields_}


class PhysProps:
    """PhysProps(n_cells, n_species, moments_list; ndens_not_Np, Tref), device resident
    (physical_props.jl:24-58).  Arrays come back in the reference's shapes
    (np/n/T: cells x species; v: 3 x cells x species)."""

    def __init__(self, domain: Domain, moments_list=(), ndens_not_Np=False, Tref=300.0):
        self.domain = domain
        self.moment_powers = list(moments_list)
        p = np.ascontiguousarray(self.moment_powers, np.int32)
        self.h = C.c_void_p()
        domain._ck(lib().mz_props_create(domain.h, len(p), ptr(p, C.c_int32) if len(p) else None, float(Tref),
                                         1 if ndens_not_Np else 0, C.byref(self.h)))
        domain._children.add(self)
        self.ndens_not_Np = ndens_not_Np
        self.Tref = Tref

    def close(self):
        if self.h:
            if self.domain.h:
                lib().mz_props_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def snapshot(self, slot, dst: PinnedArray):
        """mz_props_snapshot: start copying np, n, v, T into dst (6 x cells x
        species doubles) without waiting; see snapshot_wait and unpack."""
        self.domain._ck(lib().mz_props_snapshot(self.h, int(slot), ptr(dst.array)))

    def snapshot_wait(self, slot):
        self.domain._ck(lib().mz_props_snapshot_wait(self.h, int(slot)))

    def unpack(self, flat):
        """np, n, v, T of a snapshot in the shapes fetch() returns."""
        nc, ns = self.domain.n_cells, self.domain.n_species
        m = nc * ns
        return dict(np=flat[:m].reshape(ns, nc).T, n=flat[m:2 * m].reshape(ns, nc).T,
                    v=flat[2 * m:5 * m].reshape(ns, nc, 3).transpose(2, 1, 0), T=flat[5 * m:6 * m].reshape(ns, nc).T)

    def fetch(self):
        nc, ns, nm = self.domain.n_cells, self.domain.n_species, len(self.moment_powers)
        lpa = np.zeros(ns)
        np_ = np.zeros(nc * ns)
        n = np.zeros(nc * ns)
        v = np.zeros(3 * nc * ns)
        T = np.zeros(nc * ns)
        mom = np.zeros(max(1, nm * nc * ns))
        self.domain._ck(lib().mz_props_download(self.h, ptr(lpa), ptr(np_), ptr(n), ptr(v), ptr(T), ptr(mom)))
        # column-major (Julia) -> numpy [..., cell, species] views
        return dict(lpa=lpa, np=np_.reshape(ns, nc).T, n=n.reshape(ns, nc).T, v=v.reshape(ns, nc, 3).transpose(2, 1, 0),
                    T=T.reshape(ns, nc).T, moments=mom[: nm * nc * ns].reshape(ns, nc, nm).transpose(2, 1, 0))


class PinnedArray:
    """A numpy array in page-locked host memory (mz_host_alloc), for
    asynchronous copies such as PhysProps.snapshot and fast uploads."""

    def __init__(self, ctx: Context, shape, dtype=np.float64):
        shape = (int(shape),) if np.ndim(shape) == 0 else tuple(int(k) for k in shape)
        dt = np.dtype(dtype)
        nbytes = max(1, int(np.prod(shape)) * dt.itemsize)
        self.ptr = C.c_void_p()
        check(lib().mz_host_alloc(ctx.h, nbytes, C.byref(self.ptr)), ctx.h)
        raw = np.ctypeslib.as_array(C.cast(self.ptr, C.POINTER(C.c_uint8)), shape=(nbytes,))
        self.array = raw[: int(np.prod(shape)) * dt.itemsize].view(dt).reshape(shape)

    def close(self):
        if self.ptr:
            self.array = None
            lib().mz_host_free(self.ptr)
            self.ptr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SurfProps:
    """SurfProps(pia, grid) of a 1-D domain (surface_props.jl:22-67): element
    0 = left wall (normal +x), element 1 = right wall (normal -x), unit areas.
    fetch() returns the reference's arrays (elements x species; force and
    shear_pressure 3 x elements x species)."""

    def __init__(self, domain: Domain):
        self.domain = domain
        self.h = C.c_void_p()
        domain._ck(lib().mz_surf_props_create(domain.h, C.byref(self.h)))
        domain._children.add(self)

    def close(self):
        if self.h:
            if self.domain.h:
                lib().mz_surf_props_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def fetch(self):
        ns = self.domain.n_species
        a = {k: np.zeros(m * 2 * ns) for k, m in (("np", 1), ("flux_incident", 1), ("flux_reflected", 1), ("force", 3),
                                                   ("normal_pressure", 1), ("shear_pressure", 3),
                                                   ("kinetic_energy_flux", 1))}
        self.domain._ck(lib().mz_surf_props_download(self.h, ptr(a["np"]), ptr(a["flux_incident"]),
                                                     ptr(a["flux_reflected"]), ptr(a["force"]),
                                                     ptr(a["normal_pressure"]), ptr(a["shear_pressure"]),
                                                     ptr(a["kinetic_energy_flux"])))
        out = {}
        for k, v in a.items():
            if k in ("force", "shear_pressure"):
                out[k] = v.reshape(ns, 2, 3).transpose(2, 1, 0)
            else:
                out[k] = v.reshape(ns, 2).T
        return out


# --------------------------------------------------------------------- serving
class Server:
    """Continuous-batching server of independent 0-D solves (mz_server_*).

    Each request is the README relaxation problem for given particle counts
    and temperatures per species; requests run side by side, one cell each,
    and advance together in fused steps.  Requests of at least 4,096
    particles (`set_lane_split`) run in a second lane (domain and stream) while the smaller ones
    take several steps per step of the large ones.  A request's result
    depends only on the request itself (its seed)."""

    def __init__(self, ctx: Context, species_data, interactions, dt, max_requests, capacity):
        self.ctx = ctx
        self.ns = len(species_data)
        mass = f64([sp.mass for sp in species_data])
        tab = (L.Interaction * (self.ns * self.ns))()
        for s1 in range(self.ns):
            for s2 in range(self.ns):
                tab[s1 + self.ns * s2] = interactions[s1][s2].c_struct()
        cap = np.ascontiguousarray(np.broadcast_to(np.asarray(capacity, np.int64), (self.ns,)))
        self.h = C.c_void_p()
        check(lib().mz_server_create(ctx.h, self.ns, ptr(mass), tab, float(dt), int(max_requests),
                                     ptr(cap, C.c_int64), C.byref(self.h)), ctx.h)
        ctx._children.add(self)

    def close(self):
        if self.h:
            if self.ctx.h:
                lib().mz_server_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _ck(self, rc):
        check(rc, self.ctx.h)

    def set_lane_split(self, particles):
        """mz_server_set_lane_split: requests of at least `particles` particles
        go to the lane of large requests (0: one lane for all)."""
        self._ck(lib().mz_server_set_lane_split(self.h, int(particles)))

    def set_hbm_headroom(self, nbytes):
        """mz_server_set_hbm_headroom: device memory that admission by free
        memory (a server created with capacity 0) leaves free."""
        self._ck(lib().mz_server_set_hbm_headroom(self.h, int(nbytes)))

    def submit(self, counts, T, Fnum, n_steps, seed, V=1.0):
        r = L.Request()
        for s in range(self.ns):
            r.count[s] = int(counts[s]) if s < len(counts) else 0
            r.T[s] = float(T[s]) if s < len(T) else 0.0
        r.Fnum, r.V, r.n_steps, r.seed = float(Fnum), float(V), int(n_steps), int(seed)
        rid = C.c_int64()
        self._ck(lib().mz_server_submit(self.h, C.byref(r), C.byref(rid)))
        return rid.value

    def step(self, max_steps=1):
        """mz_server_step_many: admit, then up to max_steps steps of every running
        request (no request past its end); returns (running, queued, retired)."""
        k, run, que, ret = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        self._ck(lib().mz_server_step_many(self.h, int(max_steps), C.byref(k), C.byref(run), C.byref(que),
                                           C.byref(ret)))
        return run.value, que.value, ret.value

    def result(self, rid):
        out = L.RequestResult()
        self._ck(lib().mz_server_result(self.h, int(rid), C.byref(out)))
        ns = self.ns
        return dict(state=out.state, steps_done=out.steps_done, np=[out.np[s] for s in range(ns)],
                    n=[out.n[s] for s in range(ns)], v=[[out.v[s][k] for k in range(3)] for s in range(ns)],
                    T=[out.T[s] for s in range(ns)])

    def retired(self):
        """ids of the requests the last step() retired"""
        n = C.c_int64()
        self._ck(lib().mz_server_retired(self.h, 0, None, C.byref(n)))
        ids = np.zeros(max(1, n.value), np.int64)
        self._ck(lib().mz_server_retired(self.h, n.value, ptr(ids, C.c_int64), C.byref(n)))
        return ids[: n.value].tolist()

    def info(self):
        steps, ps = C.c_int64(), C.c_int64()
        self._ck(lib().mz_server_info(self.h, C.byref(steps), C.byref(ps)))
        return dict(steps=steps.value, particle_steps=ps.value)

    def serve(self, requests, clock=time.perf_counter, max_steps=16):
        """Request loop: `requests` are (arrival_s, kwargs of submit) sorted by
        arrival.  Requests are submitted when their arrival time has passed
        (relative to the start), the server steps while work remains (up to
        max_steps steps per call, fewer when a running request finishes
        sooner), and the latency of each request (completion - arrival) is
        recorded.  Returns (latencies in s, ids, elapsed s)."""
        t0 = clock()
        i, n = 0, len(requests)
        ids, arrival = [], {}
        pending = set()
        lat = {}
        while i < n or pending:
            now = clock() - t0
            while i < n and requests[i][0] <= now:
                rid = self.submit(**requests[i][1])
                ids.append(rid)
                arrival[rid] = requests[i][0]
                pending.add(rid)
                i += 1
            if not pending:
                # idle until the next arrival
                time.sleep(max(0.0, min(requests[i][0] - now, 0.002)))
                continue
            _, _, retired = self.step(max_steps)
            if retired:
                t = clock() - t0
                for rid in self.retired():
                    lat[rid] = t - arrival[rid]
                    pending.discard(rid)
        return [lat[r] for r in ids], ids, clock() - t0


# --------------------------------------------------------------------- reference-named functions
def ntc(rng, domain, cell, species, dt, species2=None, dw_tol=1e-16):
    """ntc! for one cell (collision_ntc.jl:338, :412); cell may be a (begin, end) range."""
    s2 = species if species2 is None else species2
    cells = cell if isinstance(cell, tuple) else (cell, cell + 1)
    domain.ntc(species, s2, dt, rng.step, cells=cells, equal_weight=False, dw_tol=dw_tol)


def ntc_equal_weight(rng, domain, cell, species, dt, species2=None):
    """ntc_equal_weight! (collision_ntc.jl:479, :554)."""
    s2 = species if species2 is None else species2
    cells = cell if isinstance(cell, tuple) else (cell, cell + 1)
    domain.ntc(species, s2, dt, rng.step, cells=cells, equal_weight=True)


def swpm(rng, domain, cell, species, G, dt):
    """swpm! (collision_swpm.jl:201-288) for one cell or a (begin, end) range;
    (sigma g)_max comes from the pair's collision factors
    (create_collision_factors_swpm_array)."""
    cells = cell if isinstance(cell, tuple) else (cell, cell + 1)
    domain.swpm(species, G, dt, rng.step, cells=cells)


def convect_particles(rng, grid, boundaries, domain, species, dt, surf_props=None):
    """convect_particles! (convection_1D.jl:130-157); with surf_props, the
    surface-sampling form (convection_1D.jl:176-206)."""
    if surf_props is not None:
        g, w = grid.c_struct(), boundaries.c_struct()
        domain._ck(lib().mz_convect_1d_surf(domain.h, species, C.byref(g), C.byref(w), float(dt), int(rng.step), 0,
                                            surf_props.h))
        return
    domain.convect(species, grid, boundaries, dt, rng.step, compute_cell=False)


def convect_particles_and_compute_cell(rng, grid, boundaries, domain, species, dt):
    """convect_particles_and_compute_cell! (convection_1D.jl:225-255)."""
    domain.convect(species, grid, boundaries, dt, rng.step, compute_cell=True)


def sort_particles(domain, species, grid=None):
    """sort_particles! (grid_sorting.jl:58-113 with grid, :128-182 without)."""
    domain.sort(species, grid)


def squash_pia(domain, species=None):
    """squash_pia! (particles.jl:622-701)."""
    for s in range(domain.n_species) if species is None else [species]:
        domain.squash(s)


def compute_props(domain, phys_props):
    """compute_props! (physical_props.jl:104-154)."""
    domain._ck(lib().mz_compute_props(domain.h, phys_props.h, L.PROPS_ALL))


def compute_props_with_total_moments(domain, phys_props):
    """compute_props_with_total_moments! (physical_props.jl:168-245)."""
    domain._ck(lib().mz_compute_props(domain.h, phys_props.h, L.PROPS_MOMENTS))


def compute_props_sorted(domain, phys_props):
    """compute_props_sorted! (physical_props.jl:317-372, :393-454 when ndens_not_Np)."""
    domain._ck(lib().mz_compute_props(domain.h, phys_props.h, L.PROPS_SORTED))


def avg_props(phys_props_avg, phys_props, n_avg_timesteps):
    """avg_props! (physical_props.jl:281-299)."""
    phys_props.domain._ck(lib().mz_avg_props(phys_props_avg.h, phys_props.h, float(n_avg_timesteps)))


def clear_surf_props(surf_props):
    """clear_props!(surf_props::SurfProps) (surface_props.jl:176-196)."""
    surf_props.domain._ck(lib().mz_surf_props_clear(surf_props.h))


def avg_surf_props(surf_props_avg, surf_props, n_avg_timesteps):
    """avg_props!(surf_props_avg::SurfProps, surf_props, n) (surface_props.jl:205-226)."""
    surf_props.domain._ck(lib().mz_surf_avg_props(surf_props_avg.h, surf_props.h, float(n_avg_timesteps)))


def clear_props(phys_props):
    """clear_props! (physical_props.jl:256-262)."""
    phys_props.domain._ck(lib().mz_clear_props(phys_props.h))


def merge_octree_N2_based(rng, octree, domain, cell, species, target_np, grid=None):
    """merge_octree_N2_based! (merging_octree_N2.jl:1060, :1088); cell may be a range."""
    cells = cell if isinstance(cell, tuple) else (cell, cell + 1)
    return domain.merge_octree(species, octree, target_np, threshold=-1, cells=cells, grid=grid, step=rng.step)


def create_collision_factors_array(domain, interactions, species_data, T_list, Fnum, mult_factor=1.0):
    """create_collision_factors_array(pia, interactions, species_data, T, Fnum) +
    estimate_sigma_g_w_max! (collision_ntc.jl:120-155, collision_utils.jl:464-504)."""
    ns = len(species_data)
    T_list = [T_list] * ns if np.ndim(T_list) == 0 else list(T_list)
    per = np.ndim(Fnum) > 0
    for s2 in range(ns):
        for s1 in range(ns):
            F = max(Fnum[s1], Fnum[s2]) if per else Fnum
            v = estimate_sigma_g_w_max(interactions[s1][s2], species_data[s1], species_data[s2], T_list[s1],
                                       T_list[s2], F, mult_factor)
            domain.set_sigma_g_w_max(s1, s2, v)


def create_collision_factors_swpm_array(domain, interactions, species_data, T_list, mult_factor=1.0):
    """create_collision_factors_swpm_array(pia, interactions, species_data, T;
    mult_factor) (collision_swpm.jl:118-149): (sigma g)_max of every pair and
    cell from estimate_sigma_g_max! (collision_utils.jl:523-534), the NTC
    estimate with Fnum = 1; stored in the domain's collision factors."""
    create_collision_factors_array(domain, interactions, species_data, T_list, 1.0, mult_factor)
