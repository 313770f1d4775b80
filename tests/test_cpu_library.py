"""CPU-only checks: the C-ABI library builds for sm_103a, loads without a GPU,
exports every entry point include/merzgpu.h declares, and the host-side
mirror computes the reference's setup quantities."""
import ctypes
import math
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "merzgpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*int\s+(mz_\w+)\s*\(", txt, flags=re.M)))


@pytest.fixture(scope="module")
def built():
    from merzgpu import build as b

    return b.build()


def test_library_exports_every_declared_symbol(built):
    lib = ctypes.CDLL(built)
    syms = declared_symbols()
    assert len(syms) > 30
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    import merzgpu

    assert sorted(merzgpu.exported_symbols()) == syms  # the Python binding covers the whole ABI
    assert merzgpu.lib().mz_version() == 3


def test_julia_binding_calls_only_declared_symbols():
    """Every ccall in the Julia binding names an entry point of the header
    (the binding cannot run here: no Julia toolchain)."""
    jl = open(os.path.join(ROOT, "merzbild.jl_gb300", "julia", "MerzbildGPU.jl")).read()
    called = set(re.findall(r"ccall\(\(:(mz_\w+),\s*libmz\)", jl))
    assert len(called) > 30
    assert not called - set(declared_symbols()), sorted(called - set(declared_symbols()))


def test_library_is_built_for_sm103a_only():
    from merzgpu import build as b

    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def test_interactions_match_oracle(orc):
    import merzgpu as mz

    sp = [mz.Species("Ar", mz.AR_MASS), mz.Species("He", mz.HE_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    o = orc.Oracle(1, 2, [mz.AR_MASS, mz.HE_MASS])
    t = mz.VHS
    d = [[t["Ar,Ar"][0], t["Ar,He"][0]], [t["Ar,He"][0], t["He,He"][0]]]
    om = [[t["Ar,Ar"][1], t["Ar,He"][1]], [t["Ar,He"][1], t["He,He"][1]]]
    o.load_interactions(d, om, 273.0)
    for s1 in range(2):
        for s2 in range(2):
            ref = o.interaction(s1, s2)
            got = inter[s1][s2]
            for k, v in ref.items():
                assert math.isclose(getattr(got, k), v, rel_tol=4e-15), (s1, s2, k)


def test_grid_and_estimates_match_oracle(orc):
    import merzgpu as mz

    g = mz.Grid1DUniform(5e-4, 2000)
    r = orc.grid(5e-4, 2000)
    assert g.dx == r["dx"] and g.inv_dx == r["inv_dx"] and g.min_x == r["min_x"] and g.max_x == r["max_x"]
    sp = [mz.Species("Ar", mz.AR_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    o = orc.Oracle(1, 1, [mz.AR_MASS])
    o.load_interactions(*mz.VHS["Ar,Ar"])
    a = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], 273.0, 273.0, 1.25e14)
    b = o.estimate_single(0, 0, 273.0, 273.0, 1.25e14)
    assert math.isclose(a, b, rel_tol=1e-15)
    # Couette config: dt = 0.2 / nu, nu = 2.86e7 1/s at n = 1e23, T = 273 K
    nu = mz.mean_collision_frequency(inter, sp, 0, 1e23, 273.0)
    assert 2.8e7 < nu < 2.9e7


def test_oracle_is_not_imported_by_the_product():
    pkg = os.path.join(ROOT, "merzbild.jl_gb300")
    for dirpath, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h", ".jl")):
                txt = open(os.path.join(dirpath, f)).read()
                assert "oracle" not in re.sub(r"#.*|//.*", "", txt).lower() or f == "build.py", f


def test_collisional_props_known_answers():
    """test/test_collisional_props_computes.jl: mean free path and collision
    frequency of VHS argon at 1e23 m^-3 and 300 K (bit-exact values), their
    monotonicity in T and linear scaling in n, and the temperature-independent
    mean free path of a hard-sphere gas (omega = 0.5)."""
    import merzgpu as mz

    sp = [mz.Species("Ar", mz.AR_MASS)]
    inter = mz.interactions_from_vhs(sp, mz.VHS)
    mfp1 = mz.mean_free_path(inter, 0, 1e23, 300.0)
    cf1 = mz.mean_collision_frequency(inter, sp, 0, 1e23, 300.0)
    assert abs(mfp1 - 1.371982759796177e-5) <= 2 * np.finfo(float).eps
    assert abs(cf1 - 2.907146431686186e7) <= 2 * np.finfo(float).eps
    assert mz.mean_free_path(inter, 0, 1e23, 500.0) > mfp1
    assert mz.mean_collision_frequency(inter, sp, 0, 1e23, 500.0) > cf1
    assert abs(mz.mean_free_path(inter, 0, 2e23, 300.0) / mfp1 - 0.5) <= 2 * np.finfo(float).eps
    assert abs(mz.mean_collision_frequency(inter, sp, 0, 2e23, 300.0) / cf1 - 2.0) <= 2 * np.finfo(float).eps
    hs = mz.interactions_from_vhs(sp, {"Ar,Ar": (4.11e-10, 0.5, 300.0)})
    assert abs(mz.mean_free_path(hs, 0, 1e23, 300.0) - mz.mean_free_path(hs, 0, 1e23, 5000.0)) <= 2 * np.finfo(float).eps
