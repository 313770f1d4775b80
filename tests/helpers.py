"""Shared helpers: build matched oracle / device states from the same arrays."""
import numpy as np

import merzgpu as mz

EPS = np.finfo(float).eps


def species(names):
    masses = {"Ar": mz.AR_MASS, "He": mz.HE_MASS}
    return [mz.Species(n, masses[n]) for n in names]


def interactions(sp, table=None):
    return mz.interactions_from_vhs(sp, table or mz.VHS)


def random_particles(rng, n, n_cells, T=300.0, mass=mz.AR_MASS, w=1e12, L=None, wspan=0.0, drift=(0, 0, 0)):
    """Arrays (w, v, x, cell) with cells in [0, n_cells), x inside its cell when L is given."""
    cell = rng.integers(0, n_cells, size=n).astype(np.int32)
    vs = np.sqrt(mz.K_B * T / mass)
    v = rng.normal(0.0, vs, size=(n, 3)) + np.asarray(drift)
    x = rng.random((n, 3))
    if L is not None:
        dx = L / n_cells
        x[:, 0] = (cell + rng.uniform(0.05, 0.95, size=n)) * dx
    ww = np.full(n, float(w))
    if wspan > 0:
        ww = w * 10.0 ** (wspan * (2 * rng.random(n) - 1))
    return ww, v, x, cell


def oracle_state(orc, n_cells, sp, inter_table, arrays_by_species, capacity=None):
    """Oracle with particles placed cell by cell in the given order (stable)."""
    o = orc.Oracle(n_cells, len(sp), [s.mass for s in sp])
    names = [s.name for s in sp]
    ns = len(sp)
    d = np.zeros((ns, ns))
    om = np.zeros((ns, ns))
    tr = np.zeros((ns, ns))
    for i in range(ns):
        for k in range(ns):
            rec = inter_table.get(f"{names[i]},{names[k]}") or inter_table[f"{names[k]},{names[i]}"]
            d[i, k], om[i, k], tr[i, k] = rec
    o.load_interactions(d, om, tr)
    for s, (w, v, x, cell) in enumerate(arrays_by_species):
        parts = np.column_stack([w, v, x])
        o.set_particles_simple(s, cell + 1, parts)
        if capacity:
            o.pv_resize(s, capacity)
    return o


def device_state(ctx, n_cells, sp, inter, arrays_by_species, capacity=None, seed=1234):
    cap = capacity or max(len(a[0]) for a in arrays_by_species) * 2 + 64
    dom = mz.Domain(ctx, n_cells, sp, cap, interactions=inter, seed=seed)
    for s, (w, v, x, cell) in enumerate(arrays_by_species):
        dom.upload(s, w, v, x, cell)
    return dom


def oracle_logical(o, s):
    rows, cells = o.logical(s)
    return rows, cells - 1


def device_logical(dom, s):
    w, v, x, cell = dom.download(s)
    return np.column_stack([w, v, x]), cell


def assert_close_rows(a, b, rtol=1e-12, what=""):
    """|a - b| <= rtol * (largest magnitude in that column): relative error on
    the scale of the quantity, so components that nearly cancel are judged
    against the velocity / position scale, not against their own size."""
    assert a.shape == b.shape, f"{what}: shape {a.shape} vs {b.shape}"
    if a.size == 0:
        return
    a2 = a.reshape(a.shape[0], -1)
    b2 = b.reshape(b.shape[0], -1)
    scale = np.maximum(np.max(np.abs(a2), axis=0), np.max(np.abs(b2), axis=0))
    err = np.abs(a2 - b2)
    bad = err > rtol * scale
    worst = np.max(err / np.maximum(scale, 1e-300))
    assert not np.any(bad), f"{what}: {np.count_nonzero(bad)} mismatches, worst relative {worst:.3e}"
