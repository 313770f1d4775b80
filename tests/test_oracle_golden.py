"""Pin the oracle (C++ restatement of the reference path) against the
reference's own known-answer tests, transcribed into tests/golden/reference_kat.json.

Each test names the reference assertion it reproduces."""
import numpy as np
import pytest

from conftest import scenario

EPS = np.finfo(float).eps


def _indexer(o):
    ind, nt, cg = o.pia_get()
    return ind, nt, cg


def _tol(t):
    if t == "2eps":
        return 2 * EPS
    if t == "eps":
        return EPS
    return float(t)


def test_philox_known_answers(orc):
    # Random123 known-answer vectors for philox4x32-10
    assert list(orc.philox([0, 0, 0, 0], [0, 0])) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    f = 0xFFFFFFFF
    assert list(orc.philox([f, f, f, f], [f, f])) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert list(orc.philox([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0])) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_stream_uniforms_in_range(orc):
    u = orc.stream_draws(1234, orc.TAG_CAND, 0, 7, 3, 11, 20000)
    assert u.min() >= 0.0 and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01
    # multiples of 2^-52 (Julia rand(Float64) construction)
    assert np.all(np.floor(u * 2.0**52) == u * 2.0**52)


def test_grid_sorting_known_answers(orc, golden):
    sc = scenario(golden, "grid_sorting_coarse_fine_uneven")
    mass = [golden["species"]["Ar"]["mass"]]
    parts = np.array(sc["particles"])
    st = sc["steps"]

    # coarse grid (test_grid_sorting.jl:23-67)
    o = orc.Oracle(2, 1, mass)
    o.pv_set(0, parts, nbuffer=0)
    ind, nt, cg = _indexer(o)
    ind[0, 0] = [4, 1, 4, 4, 0, -1, 0]
    ind[0, 1] = [4, 5, 8, 4, 0, -1, 0]
    nt[0] = 8
    o.pia_set(ind, nt, cg)
    o.sort(0, L=8.0, nx=2)
    pv = o.pv_get(0)
    assert list(pv["index"]) == st[0]["expect_index"]
    ind, nt, cg = _indexer(o)
    assert ind[0].tolist() == st[0]["expect_indexer"]
    logical, _ = o.logical(0)
    for i in range(1, 5):
        assert logical[i - 1, 4] == 0.99 * 8.0 * (9.0 - i - 4) / 8
    for i in range(5, 9):
        assert logical[i - 1, 4] == 0.99 * 8.0 * (9.0 - i + 4) / 8

    # fine grid, continuing from the sorted ParticleVector (test_grid_sorting.jl:98-143)
    of = orc.Oracle(4, 1, mass)
    of.pv_set(0, pv["particles"], index=pv["index"], cell=pv["cell"], buffer=pv["buffer"], nbuffer=pv["nbuffer"])
    ind, nt, cg = _indexer(of)
    ind[0, 0] = [8, 1, 8, 8, 0, -1, 0]
    nt[0] = 8
    of.pia_set(ind, nt, cg)
    of.sort(0, L=8.0, nx=4)
    pvf = of.pv_get(0)
    assert list(pvf["index"]) == st[1]["expect_index"]
    ind, _, _ = _indexer(of)
    assert ind[0].tolist() == st[1]["expect_indexer"]

    # uneven split after resetting the index (test_grid_sorting.jl:145-187)
    p2 = pvf["particles"].copy()
    p2[:, 4] = st[2]["x"]
    of.pv_set(0, p2, index=np.arange(1, 9), cell=pvf["cell"], buffer=pvf["buffer"], nbuffer=pvf["nbuffer"])
    of.sort(0, L=8.0, nx=4)
    assert list(of.pv_get(0)["index"]) == st[2]["expect_index"]
    ind, _, _ = _indexer(of)
    assert ind[0, :, 3].tolist() == st[2]["expect_counts"]
    assert ind[0, :, 1].tolist() == st[2]["expect_starts"]
    assert ind[0, :, 2].tolist() == st[2]["expect_ends"]
    assert np.all(ind[0, :, 6] == 0) and np.all(ind[0, :, 4] == 0) and np.all(ind[0, :, 5] == -1)
    pr = of.compute_props(mode=0)
    assert np.all(np.abs(pr["n"][0] - np.array(st[2]["expect_n"])) < 2 * EPS)
    assert pr["np"][0].tolist() == st[2]["expect_counts"]

    # stored-cell variant (test_grid_sorting.jl:189-235)
    p3 = p2.copy()
    p3[:4, 4] = 0.05
    p3[4, 4] = 0.1
    p3[5:, 4] = 0.3
    of.pv_set(0, p3, index=np.arange(1, 9), cell=st[3]["cell"], buffer=pvf["buffer"], nbuffer=pvf["nbuffer"])
    of.sort(0)
    assert list(of.pv_get(0)["index"]) == st[3]["expect_index"]
    ind, _, _ = _indexer(of)
    assert ind[0, :, 3].tolist() == st[3]["expect_counts"]
    assert ind[0, :, 1].tolist() == st[3]["expect_starts"]
    assert ind[0, :, 2].tolist() == st[3]["expect_ends"]


def _convection_setup(orc, sc):
    o = orc.Oracle(sc["nx"], 1, [sc["mass"]])
    o.pv_set(0, np.array(sc["particles"]), nbuffer=0)
    ind, nt, cg = o.pia_get()
    ind[0, 0] = [4, 1, 4, 4, 0, -1, 0]
    nt[0] = 4
    o.pia_set(ind, nt, cg)
    return o


def test_convection_known_answers(orc, golden):
    sc = scenario(golden, "convection_specular_4particles")
    for variant in ("grid", "compute_cell"):
        o = _convection_setup(orc, sc)
        if variant == "grid":
            o.convect(0, sc["L"], sc["nx"], sc["walls"], sc["dt"], seed=1, step=0)
            o.sort(0, L=sc["L"], nx=sc["nx"])
        else:
            o.convect(0, sc["L"], sc["nx"], sc["walls"], sc["dt"], seed=1, step=0, compute_cell=True)
            assert o.pv_get(0)["cell"][:4].tolist() == sc["expect_cells_after_convect"]
            o.sort(0)
        assert o.pv_get(0)["index"].tolist() == sc["expect_index_after_sort"]
        logical, _ = o.logical(0)
        for k, e in enumerate(sc["expect_sorted"]):
            assert np.max(np.abs(logical[k, 4:7] - np.array(e["x"]))) < _tol(e["x_tol"])
            assert logical[k, 1:4].tolist() == e["v"]
            assert logical[k, 0] == e["w"]
        pr = o.compute_props(mode=0)
        expect = np.zeros(sc["nx"])
        for c, w in sc["expect_n_by_cell"].items():
            expect[int(c) - 1] = w
        assert np.all(np.abs(pr["n"][0] - expect) < EPS)


def test_convection_noncontiguous(orc, golden):
    sc = scenario(golden, "convection_noncontiguous")
    o = orc.Oracle(sc["nx"], 1, [sc["mass"]])
    o.pv_set(0, np.array(sc["particles"]), nbuffer=0)
    ind, nt, cg = o.pia_get()
    ind[0, 1] = sc["indexer_cell2"]
    nt[0] = sc["n_total"]
    cg[0] = 0
    o.pia_set(ind, nt, cg)
    pr = o.compute_props(mode=0)
    assert abs(pr["n"][0, 1] - 15.0) < EPS
    assert np.all(np.abs(np.delete(pr["n"][0], 1)) <= EPS)
    assert abs(pr["v"][0, 1, 0] - 1.0) < EPS
    o.convect(0, sc["L"], sc["nx"], sc["walls"], sc["dt"], seed=3, step=0)
    o.sort(0, L=sc["L"], nx=sc["nx"])
    pr = o.compute_props(mode=0)
    assert abs(pr["n"][0, 3] - 15.0) < EPS
    assert np.all(np.abs(np.delete(pr["n"][0], 3)) <= EPS)
    assert abs(pr["v"][0, 3, 0] - 1.0) < EPS


def test_collision_utils(orc, golden):
    sc = scenario(golden, "collision_utils_com_g")
    ar = golden["species"]["Ar"]["mass"]
    o = orc.Oracle(1, 1, [ar])
    d, om, tr = golden["vhs"]["Ar,Ar"]
    o.load_interactions(d, om, tr)
    I = o.interaction(0, 0)
    assert abs(I["mu1"] - 0.5) < EPS and abs(I["mu2"] - 0.5) < EPS
    a, b, vcom, g = o.com_g_scatter(0, 0, sc["p1"], sc["p2"], seed=1234, scatter=True)
    assert np.all(np.abs(vcom - np.array(sc["expect_v_com"])) < EPS)
    assert abs(g - sc["expect_g"]) < EPS
    _, _, vcom2, g2 = o.com_g_scatter(0, 0, a, b, scatter=False)
    assert np.all(np.abs(vcom2 - np.array(sc["expect_v_com"])) < EPS)
    assert abs(g2 - 3.0) < 2.1 * EPS
    # two-species mass ratios (test_collision_utils.jl:42-53)
    he = golden["species"]["He"]["mass"]
    o2 = orc.Oracle(1, 2, [ar, he])
    vhs = golden["vhs"]
    o2.load_interactions([[vhs["Ar,Ar"][0], vhs["Ar,He"][0]], [vhs["Ar,He"][0], vhs["He,He"][0]]],
                         [[vhs["Ar,Ar"][1], vhs["Ar,He"][1]], [vhs["Ar,He"][1], vhs["He,He"][1]]], 273.0)
    I11, I22, I12, I21 = (o2.interaction(0, 0), o2.interaction(1, 1), o2.interaction(0, 1), o2.interaction(1, 0))
    assert abs(I11["mu1"] - 0.5) < EPS and abs(I22["mu2"] - 0.5) < EPS
    assert abs(I12["mu1"] - I21["mu2"]) < EPS and abs(I12["mu2"] - I21["mu1"]) < EPS
    assert abs(I12["mu1"] + I12["mu2"] - 1.0) < EPS
    # estimate_sigma_g_w_max! scalar vs per-species T (test_collision_utils.jl:101-134)
    o2.estimate_sigma_g_w_max([300.0, 300.0], 1e10, mult=2.0)
    s_a, _ = o2.cf_get(0, 1)
    assert abs(s_a[0] - o2.estimate_single(0, 1, 300.0, 300.0, 1e10, 2.0)) <= 2 * EPS


def _kinetic(parts, m):
    return 0.5 * m * np.sum(parts[:, 0] * np.sum(parts[:, 1:4] ** 2, axis=1))


@pytest.mark.parametrize("w1,w2,dw_tol,expect_split", [(1.0, 1.0, 1e-16, None), (2.0, 1.0, 1e-16, 0),
                                                       (1.0, 2.0, 1e-16, 1), (1.0, 1.01, 0.1, None)])
def test_collide_vhs_split_semantics(orc, golden, w1, w2, dw_tol, expect_split):
    # test/test_collision_vhs.jl:35-218
    ar = golden["species"]["Ar"]["mass"]
    o = orc.Oracle(1, 1, [ar])
    o.load_interactions(*golden["vhs"]["Ar,Ar"])
    parts = np.array([[w1, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0], [w2, -1.0, 0.0, 0.0, 0.0, 0.0, 0.0]])
    o.pv_set(0, parts, nbuffer=0)
    ind, nt, cg = o.pia_get()
    nt[0] = 2
    ind[0, 0] = [2, 1, 2, 2, 0, -1, 0]
    o.pia_set(ind, nt, cg)
    o.cf_set_smax(0, 0, 0.0)
    ke0 = _kinetic(parts, ar)
    o.collide_vhs(0, 0, 1, 1, 2, dw_tol=dw_tol, seed=1234)
    _, cnt = o.cf_get(0, 0)
    assert cnt[0, 3] > 0  # n_coll_performed
    _, nt, _ = o.pia_get()
    logical, _ = o.logical(0)
    if expect_split is None:
        assert nt[0] == 2 and cnt[0, 4] > 0
    else:
        assert nt[0] == 3
        assert logical[2, 0] == 1.0
        assert logical[2, 1:4].tolist() == parts[expect_split, 1:4].tolist()
        assert logical[2, 4:7].tolist() == parts[expect_split, 4:7].tolist()
        assert logical[expect_split, 0] == 1.0
    assert abs(_kinetic(logical, ar) - ke0) <= 1e-14


@pytest.mark.parametrize("w1,w2", [(1.0, 1.0), (2.0, 1.0), (1.0, 2.0)])
def test_collide_vhs_equal_weight_known_answers(orc, golden, w1, w2):
    # test/test_collision_vhs_equal_weight.jl: the equal-weight collision
    # never splits, whatever the weights, and conserves the weighted energy
    ar = golden["species"]["Ar"]["mass"]
    o = orc.Oracle(1, 1, [ar])
    o.load_interactions(*golden["vhs"]["Ar,Ar"])
    parts = np.array([[w1, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0], [w2, -1.0, 0.0, 0.0, 0.0, 0.0, 0.0]])
    o.pv_set(0, parts, nbuffer=0)
    ind, nt, cg = o.pia_get()
    nt[0] = 2
    ind[0, 0] = [2, 1, 2, 2, 0, -1, 0]
    o.pia_set(ind, nt, cg)
    o.cf_set_smax(0, 0, 0.0)
    ke0 = _kinetic(parts, ar)
    o.collide_vhs(0, 0, 1, 1, 2, seed=1234, equal_weight=True)
    _, cnt = o.cf_get(0, 0)
    assert cnt[0, 3] > 0 and cnt[0, 4] == cnt[0, 3]
    _, nt, _ = o.pia_get()
    assert nt[0] == 2
    logical, _ = o.logical(0)
    assert logical[:, 0].tolist() == [w1, w2]
    assert abs(_kinetic(logical, ar) - ke0) <= 1e-14


def _merge_state(orc, parts, ar, indexer=None):
    parts = np.array(parts)
    n = parts.shape[0]
    o = orc.Oracle(1, 1, [ar])
    o.pv_set(0, parts, nbuffer=0)
    ind, nt, cg = o.pia_get()
    ind[0, 0] = indexer if indexer is not None else [n, 1, n, n, 0, -1, 0]
    nt[0] = n
    o.pia_set(ind, nt, cg)
    return o


def test_octree_merge_known_answers(orc, golden):
    sc = scenario(golden, "octree_merge_24")
    ar = sc["mass"]
    o = _merge_state(orc, sc["particles24"], ar)
    oc = orc.Octree(orc.SPLIT_MID, orc.INIT_C)
    oc.init(o, 0, 1)
    oc.split_bin(o, 0, 1)
    assert oc.summary()["Nbins"] == 8
    for b in range(1, 9):
        oc.compute_bin_props(o, 0, b)
    bins = oc.bins(8)
    e = sc["split_once"]
    assert bins["np"].tolist() == e["expect_np"]
    assert bins["w"].tolist() == e["expect_w"]
    assert np.max(np.abs(bins["v_mean"] - np.array(e["expect_v_mean"]))) < 1e-14
    assert np.max(np.abs(bins["x_mean"] - np.array(e["expect_x_mean"]))) < 1e-14

    pr0 = o.compute_props(mode=0)
    n0, T0, v0 = pr0["n"][0, 0], pr0["T"][0, 0], pr0["v"][0, 0].copy()
    assert n0 == 108.0
    oc2 = orc.Octree(orc.SPLIT_MID, orc.INIT_C)
    o.merge_octree(oc2, 0, 1, 16, seed=1234, step=0)
    s = oc2.summary()
    _, nt, _ = o.pia_get()
    assert s["Nbins"] == 8 and nt[0] == 16
    assert np.all(oc2.bins(8)["depth"] == 1)
    pr = o.compute_props(mode=0)
    assert pr["np"][0, 0] == 16
    assert abs(pr["n"][0, 0] - n0) < EPS
    assert abs(pr["T"][0, 0] - T0) < 1e-14
    assert np.max(np.abs(pr["v"][0, 0] - v0)) < 1e-14

    o.merge_octree(oc2, 0, 1, 2, seed=1234, step=1)
    assert oc2.summary()["Nbins"] == 1
    _, nt, _ = o.pia_get()
    assert nt[0] == 2
    logical, _ = o.logical(0)
    assert logical[0, 0] == 0.5 * 108.0 and logical[0, 0] == logical[1, 0]
    pr = o.compute_props(mode=0)
    assert abs(pr["n"][0, 0] - n0) < EPS
    assert abs(pr["T"][0, 0] - T0) < 1e-14
    assert np.max(np.abs(pr["v"][0, 0] - v0)) < 1e-14

    for key in ("zero_weight_last", "zero_weight_two_groups"):
        z = sc[key]
        o = _merge_state(orc, z["particles"], ar, indexer=z.get("indexer"))
        pr0 = o.compute_props(mode=0)
        o.merge_octree(oc2, 0, 1, z["target"], seed=99, step=0)
        _, nt, _ = o.pia_get()
        assert nt[0] == z["expect_n_total"]
        pr = o.compute_props(mode=0)
        assert pr["np"][0, 0] == nt[0]
        assert abs(pr["n"][0, 0] - pr0["n"][0, 0]) < EPS
        assert abs(pr["T"][0, 0] - pr0["T"][0, 0]) < 1e-14
        assert np.max(np.abs(pr["v"][0, 0] - pr0["v"][0, 0])) < 1e-14
        logical, _ = o.logical(0)
        assert np.all(logical[:, 0] > 0) and not np.any(np.isnan(logical[:, 4]))
        ind, _, _ = o.pia_get()
        if key == "zero_weight_last":
            assert ind[0, 0, 2] == nt[0] and ind[0, 0, 4] == 0 and ind[0, 0, 5] == -1
        else:
            assert ind[0, 0, 5] > 0 and ind[0, 0, 4] > 0

    t = sc["two_particles"]
    o = _merge_state(orc, t["particles"], ar)
    o.merge_octree(oc2, 0, 1, t["target"], seed=5, step=0)
    b = oc2.bins(1)
    assert b["np"][0] == 2 and oc2.summary()["n_particles"] == 2 and not b["can_be_refined"][0]


def test_octree_sorting_known_answers(orc, golden):
    sc = scenario(golden, "octree_sorting")
    ar = golden["species"]["Ar"]["mass"]
    for v, expect in sc["octants"]["cases"]:
        assert orc.compute_octant(v, sc["octants"]["vmid"]) == expect

    e = sc["nine_reverse"]
    o = _merge_state(orc, e["particles"], ar)
    oc = orc.Octree(orc.SPLIT_MID, orc.INIT_C)
    oc.init(o, 0, 1)
    assert sorted(oc.pis(9).tolist()) == list(range(1, 10))
    oc.split_bin(o, 0, 1)
    assert oc.summary()["Nbins"] == 8
    assert oc.pis(9).tolist() == e["expect_pis"]

    e = sc["nine_mixed"]
    for indexer in (None, e["two_group_indexer"]):
        o = _merge_state(orc, e["particles"], ar, indexer=indexer)
        oc.init(o, 0, 1)
        oc.split_bin(o, 0, 1)
        assert oc.summary()["Nbins"] == 8
        assert oc.pis(9).tolist() == e["expect_pis"]
        b = oc.bins(8)
        assert b["bin_start"].tolist() == e["expect_bin_start"]
        assert b["bin_end"].tolist() == e["expect_bin_end"]
        assert b["np"].tolist() == e["expect_np"]
        assert b["w"].tolist() == e["expect_w"]

    e = sc["seven"]
    o = _merge_state(orc, e["particles"], ar)
    oc.init(o, 0, 1)
    oc.split_bin(o, 0, 1)
    b = oc.bins(7)
    assert oc.summary()["Nbins"] == 7
    assert oc.pis(7).tolist() == e["expect_pis"]
    assert b["bin_start"].tolist() == e["expect_bin_start"] and b["bin_end"].tolist() == e["expect_bin_end"]
    assert b["np"].tolist() == e["expect_np"] and b["w"].tolist() == e["expect_w"]

    e = sc["nested15"]
    o = _merge_state(orc, e["particles"], ar)
    oc2 = orc.Octree(orc.SPLIT_MID, orc.INIT_MINMAX_SYM)
    oc2.init(o, 0, 1)
    b = oc2.bins(1)
    assert b["bin_start"][0] == 1 and b["bin_end"][0] == 15
    oc2.split_bin(o, 0, 1)
    f = e["first_split"]
    assert oc2.summary()["Nbins"] == 8
    pis = oc2.pis(15)
    assert pis[:2].tolist() == f["expect_pis_1_2"]
    b = oc2.bins(8)
    assert [b["bin_start"][2], b["bin_end"][2]] == f["expect_bin3"]
    assert sorted(pis[2:10].tolist()) == f["expect_sorted_3_10"]
    assert pis[10:15].tolist() == f["expect_pis_11_15"]
    assert b["np"].tolist() == f["expect_np"] and b["w"].tolist() == f["expect_w"]
    oc2.split_bin(o, 0, 3)
    sft = e["second_split"]
    assert oc2.summary()["Nbins"] == 15
    pis = oc2.pis(15)
    assert pis[:2].tolist() == f["expect_pis_1_2"]
    assert sorted(pis[2:10].tolist()) == f["expect_sorted_3_10"]
    assert pis[10:15].tolist() == f["expect_pis_11_15"]
    b = oc2.bins(15)
    assert b["bin_start"][:3].tolist() == sft["expect_bin_start_1_3"]
    assert b["bin_start"][3:8].tolist() == sft["expect_bin_start_4_8"]
    assert b["bin_start"][8:15].tolist() == sft["expect_bin_start_9_15"]
    assert b["np"].tolist() == sft["expect_np"] and b["w"].tolist() == sft["expect_w"]


def test_octree_bounds_known_answers(orc, golden):
    sc = scenario(golden, "octree_bounds")
    ar = golden["species"]["Ar"]["mass"]
    o = _merge_state(orc, sc["eight"], ar)
    oc = orc.Octree(orc.SPLIT_MID, orc.INIT_C)
    oc.init(o, 0, 1)
    b = oc.bins(1)
    c = sc["c_bounds"]
    assert np.max(np.abs(b["vmin"][0] + c)) < 1e-12 and np.max(np.abs(b["vmax"][0] - c)) < 1e-12
    oc.split_bin(o, 0, 1)
    assert np.max(np.abs(oc.summary()["vel_middle"])) < 1e-12

    o = _merge_state(orc, sc["fifteen"], ar)
    oc2 = orc.Octree(orc.SPLIT_MID, orc.INIT_MINMAX_SYM)
    oc2.init(o, 0, 1)
    b = oc2.bins(1)
    assert np.max(np.abs(b["vmin"][0] + b["vmax"][0])) < 1e-12
    assert np.max(np.abs(b["vmax"][0] - np.array(sc["sym_vmax"]))) < 1e-12
    oc3 = orc.Octree(orc.SPLIT_MID, orc.INIT_MINMAX)
    oc3.init(o, 0, 1)
    b = oc3.bins(1)
    assert np.max(np.abs(b["vmin"][0] - np.array(sc["minmax_vmin"]))) < 1e-11
    assert np.max(np.abs(b["vmax"][0] - np.array(sc["minmax_vmax"]))) < 1e-11

    oc4 = orc.Octree(orc.SPLIT_MEAN, orc.INIT_MINMAX)
    oc4.init(o, 0, 1)
    oc4.compute_v_mean(o, 0, 1, 15)
    parts = np.array(sc["fifteen"])
    assert np.max(np.abs(oc4.summary()["vel_middle"] - parts[:, 1:4].mean(axis=0))) < 1e-11
    prev = oc4.bins(1)
    parts[14, 1:4] = sc["outlier_v"]
    o2 = _merge_state(orc, parts, ar)
    oc4.bin_bounds_recompute(o2, 0, 1, 1, 15)
    b = oc4.bins(1)
    assert b["vmin"][0, 0] == prev["vmin"][0, 0] and b["vmax"][0, 0] == parts[14, 1]
    assert b["vmin"][0, 1] == parts[14, 2] and b["vmax"][0, 1] == prev["vmax"][0, 1]
    assert b["vmin"][0, 2] == prev["vmin"][0, 2] and b["vmax"][0, 2] == parts[14, 3]


def test_computes_known_answers(orc, golden):
    sc = scenario(golden, "computes_uniform")
    ar = golden["species"]["Ar"]["mass"]
    n = sc["n_particles"]
    Fnum = sc["n_dens"] / n
    parts = np.tile(np.array([Fnum] + sc["v0"] + sc["x0"]), (n, 1))
    o = _merge_state(orc, parts, ar)
    pr = o.compute_props(mode=0)
    assert abs(pr["np"][0, 0] - n) / n <= EPS
    assert abs(pr["n"][0, 0] - sc["n_dens"]) / sc["n_dens"] < sc["tol_small"]
    assert np.max(np.abs(pr["v"][0, 0] - np.array(sc["v0"]))) < sc["tol_small"]
    assert abs(pr["T"][0, 0]) < EPS
    ps = o.compute_props(mode=2)
    assert abs(ps["np"][0, 0] - pr["np"][0, 0]) < EPS and abs(ps["n"][0, 0] - pr["n"][0, 0]) < EPS
    assert abs(ps["T"][0, 0]) < EPS
    # avg_props! (test_computes.jl:83-106)
    import ctypes as C

    a = sc["avg"]
    avg = np.zeros(4)
    for k in range(2):
        inst = np.array([a["T"][k], a["n"][k], a["np"][k], a["v"][k]])
        orc.lib().orc_avg_props(4, avg.ctypes.data_as(C.POINTER(C.c_double)),
                                inst.ctypes.data_as(C.POINTER(C.c_double)), 2.0)
    ex = a["expect"]
    assert np.max(np.abs(avg - np.array([ex["T"], ex["n"], ex["np"], ex["v"]]))) < 2 * EPS


def test_collisions_1d_conservation(orc, golden):
    # test/test_collisions_1D.jl:1-83 with pseudo-Maxwell data
    ar = golden["species"]["Ar"]["mass"]
    np_, Fnum, T = 2000, 1e15, 750.0
    o = orc.Oracle(5, 1, [ar])
    o.load_interactions(*golden["pseudo_maxwell"]["Ar,Ar"])
    o.pv_create(0, np_)
    g = orc.grid(10.0, 5)
    o.sample_equal_weight(0, 2, np_, T, Fnum, box=(g["dx"], 2 * g["dx"], 0, 1, 0, 1), seed=1234, step=0)
    _, nt, _ = o.pia_get()
    ind, _, _ = o.pia_get()
    assert nt[0] == np_ and ind[0, 1, 1] == 1 and ind[0, 1, 2] == np_
    pr0 = o.compute_props(mode=0)
    assert pr0["n"][0].tolist() == [0.0, np_ * Fnum, 0.0, 0.0, 0.0]
    o.cf_set_smax(0, 0, o.estimate_single(0, 0, T, T, Fnum))
    for cell in range(1, 6):
        o.ntc(0, 0, cell, 1e-3, g["dx"], seed=1234, step=1)
    _, cnt = o.cf_get(0, 0)
    assert cnt[1, 2] > 0
    assert np.all(cnt[:, 0] == pr0["np"][0]) and np.all(cnt[:, 1] == pr0["np"][0])
    pr = o.compute_props(mode=0)
    assert pr["n"][0].tolist() == [0.0, np_ * Fnum, 0.0, 0.0, 0.0]
    # The reference asserts 5e-13 K and 2e-14 m/s for its own RNG realization.
    # Over 20 Philox seeds the round-off reaches 1.4e-12 K and 3.9e-14 m/s, so
    # the bounds here are FP64 round-off bounds with 2-3x headroom.
    assert abs(pr["T"][0, 1] - pr0["T"][0, 1]) < 4e-15 * T
    assert np.max(np.abs(pr["v"][0, 1] - pr0["v"][0, 1])) < 1e-13


def test_surface_props_known_answers(orc):
    """test/test_surface_props_1D_uniform.jl:74-178: incident and reflected
    updates of the two wall elements, then surface_props_scale! with areas 2
    and 4 and dt 1e-20 (values transcribed from the test's expressions)."""
    EPS2 = 2 * np.finfo(float).eps
    q = np.zeros((2, 11))
    orc.surf_update(q, 0, 3.5, [-9.0, 9.0, 0.0], False)
    orc.surf_update(q, 1, 10.5, [10.0, 0.0, 3.0], False)
    NP, FIN, FREF, FX, FY, FZ, PN, SX, SY, SZ, KE = range(11)
    assert q[:, NP].tolist() == [1.0, 1.0] and q[:, FIN].tolist() == [3.5, 10.5] and q[:, FREF].tolist() == [0, 0]
    assert abs(q[0, FX] - 3.5 * -9) < EPS2 and abs(q[1, FX] - 10.5 * 10) < EPS2
    assert abs(q[0, FY] - 3.5 * 9) < EPS2 and q[1, FY] == 0.0 and q[0, FZ] == 0.0
    assert abs(q[1, FZ] - 10.5 * 3) < EPS2
    assert abs(q[0, PN] - 9 * 3.5) < EPS2 and abs(q[1, PN] - 10 * 10.5) < EPS2
    assert abs(q[0, SY] - 9 * 3.5) < EPS2 and abs(q[1, SZ] - 3 * 10.5) < EPS2 and q[0, SX] == 0.0
    assert abs(q[0, KE] - 0.5 * 3.5 * (81 + 81)) < EPS2 and abs(q[1, KE] - 0.5 * 10.5 * (100 + 9)) < EPS2
    # reflections: left specular (-9, 9, 0) -> (9, 9, 0); right re-emitted at
    # (-1, -2, -4) with weight 10
    orc.surf_update(q, 0, 3.5, [9.0, 9.0, 0.0], True)
    orc.surf_update(q, 1, 10.0, [-1.0, -2.0, -4.0], True)
    assert q[:, FREF].tolist() == [-3.5, -10.0]
    assert abs(q[0, FX] - (3.5 * -9 - 3.5 * 9)) < EPS2 and abs(q[1, FX] - (10.5 * 10 - 10.0 * -1)) < EPS2
    assert abs(q[0, FY]) < EPS2 and abs(q[1, FY] - (-10.0 * -2)) < EPS2
    assert abs(q[1, FZ] - (10.5 * 3 - 10.0 * -4)) < EPS2
    assert abs(q[0, PN] - (9 * 3.5 + 9 * 3.5)) < EPS2 and abs(q[1, PN] - (10 * 10.5 + 1 * 10.0)) < EPS2
    assert abs(q[0, SY] - (9 * 3.5 - 9 * 3.5)) < EPS2 and abs(q[1, SY] - (0 * 10.5 - -2 * 10.0)) < EPS2
    assert abs(q[1, SZ] - (3 * 10.5 - -4 * 10.0)) < EPS2
    assert abs(q[0, KE]) < EPS2
    assert abs(q[1, KE] - (0.5 * 10.5 * 109 - 0.5 * 10.0 * 21)) < EPS2
    kept = q.copy()
    mass, dt = 6.633e-26, 1e-20
    orc.surf_scale(q, mass, dt, [0.5, 0.25])
    f = mass * np.array([0.5, 0.25]) / dt
    assert q[:, NP].tolist() == [1.0, 1.0]
    for k in range(1, 11):
        assert np.all(np.abs(q[:, k] - f * kept[:, k]) <= EPS2 * np.maximum(1.0, np.abs(f * kept[:, k])))


def _two_cells_spread(orc, ar):
    """test/test_octree_merging_1D.jl:4-44: 4 particles in each of 2 cells of a
    unit grid, placed so that mean(x) -/+ std(x) leaves the domain."""
    x1, x2 = [0.05, 0.05, 0.05, 0.45], [0.55, 0.95, 0.85, 0.99]
    parts = [[2.0, 0.5, -3.0, 4.0, x, 0.0, 0.0] for x in x1] + [[3.0, 0.5, -3.0, 4.0, x, 0.0, 0.0] for x in x2]
    o = orc.Oracle(2, 1, [ar])
    o.pv_set(0, parts, nbuffer=0)
    ind, nt, cg = o.pia_get()
    ind[0, 0] = [4, 1, 4, 4, 0, -1, 0]
    ind[0, 1] = [4, 5, 8, 4, 0, -1, 0]
    nt[0] = 8
    o.pia_set(ind, nt, cg)
    return o


def test_octree_merge_1d_keeps_particles_in_the_grid(orc, golden):
    # test/test_octree_merging_1D.jl:46-133
    ar = scenario(golden, "octree_merge_24")["mass"]
    for with_grid in (False, True):
        o = _two_cells_spread(orc, ar)
        oc = orc.Octree(orc.SPLIT_MID, orc.INIT_C)
        for cell in (1, 2):
            if with_grid:
                o.merge_octree(oc, 0, cell, 2, L=1.0, nx=2, seed=1234, step=0)
            else:
                o.merge_octree(oc, 0, cell, 2, seed=1234, step=0)
        ind, _, cg = o.pia_get()
        assert ind[0, 0, :4].tolist() == [2, 1, 2, 2]
        assert ind[0, 1, :4].tolist() == [2, 5, 6, 2]
        logical, cells = o.logical(0)
        for c in (1, 2):
            x = logical[cells == c, 4]
            outside = bool(np.any((x < 0.0) | (x > 1.0)))
            assert outside == (not with_grid), (with_grid, c, x)
        if with_grid:
            assert cg[0] == 0  # merging leaves the indexer non-contiguous
            o.sort(0, L=1.0, nx=2)
            pr = o.compute_props(mode=0)
            assert pr["np"][0].tolist() == [2, 2]
            assert pr["n"][0].tolist() == [8.0, 12.0]


def _pia_state(orc, ar, n_cells, x, indexer, cell=None):
    """ParticleVector(10) with particle i = (w i, v 0, x_i) and nbuffer set to
    0, plus a hand-built indexer (test/test_pia_contiguous.jl)."""
    n = len(x)
    parts = [[float(i + 1), 0.0, 0.0, 0.0, x[i], 0.0, 1.0] for i in range(n)]
    o = orc.Oracle(n_cells, 1, [ar])
    o.pv_set(0, parts, cell=cell, nbuffer=0)
    ind, nt, cg = o.pia_get()
    for c, row in enumerate(indexer):
        ind[0, c] = row
    nt[0] = n
    o.pia_set(ind, nt, cg)
    return o


def _mark_noncontiguous(o):
    ind, nt, cg = o.pia_get()
    cg[0] = 0
    o.pia_set(ind, nt, cg)


def test_squash_pia_known_answers(orc, golden):
    # test/test_pia_contiguous.jl:1-320
    ar = scenario(golden, "octree_merge_24")["mass"]
    cells = list(range(11, 21))

    # 1 cell, 1 group: delete the last particle of group 1
    o = _pia_state(orc, ar, 1, [10.0] * 10, [[10, 1, 10, 10, -1, -1, 0]], cell=cells)
    pr = o.compute_props(mode=0)
    assert pr["np"][0, 0] == 10 and abs(pr["n"][0, 0] - 55.0) / 55.0 < 1e-15
    o.delete_particle_end_group(0, 1, 1)
    _mark_noncontiguous(o)
    pv = o.pv_get(0)
    assert pv["nbuffer"] == 1
    freed = pv["buffer"][0]
    o.squash(0)
    ind, _, cg = o.pia_get()
    assert cg[0] == 1
    assert ind[0, 0, 3] == 9 and ind[0, 0, 2] == 9 and ind[0, 0, 6] == 0
    pv = o.pv_get(0)
    assert pv["cell"][:9].tolist() == cells[:9]
    pr = o.compute_props(mode=0)
    assert pr["np"][0, 0] == 9 and abs(pr["n"][0, 0] - 45.0) / 45.0 < 1e-15
    assert freed not in pv["index"][:9]

    # 1 cell, 2 groups: delete the last particle of each group
    o = _pia_state(orc, ar, 1, [10.0] * 10, [[10, 1, 5, 5, 6, 10, 5]], cell=cells)
    o.delete_particle_end_group(0, 1, 1)
    o.delete_particle_end_group(0, 1, 2)
    _mark_noncontiguous(o)
    pv = o.pv_get(0)
    assert pv["nbuffer"] == 2
    freed = pv["buffer"][:2].tolist()
    o.squash(0)
    pv = o.pv_get(0)
    assert pv["cell"][:8].tolist() == [11, 12, 13, 14, 16, 17, 18, 19]
    ind, _, cg = o.pia_get()
    assert cg[0] == 1 and ind[0, 0, 3] == 4 and ind[0, 0, 2] == 4 and ind[0, 0, 6] == 4
    pr = o.compute_props(mode=0)
    assert pr["np"][0, 0] == 8 and abs(pr["n"][0, 0] - 40.0) / 40.0 < 1e-15
    assert not any(f in pv["index"][:8] for f in freed)

    # 3 cells laid out 111 22 33 1 33; delete 3 from cell 1, 1 from cell 3's group 1
    x = [1.0, 1.0, 1.0, 2.0, 2.0, 3.0, 3.0, 1.0, 3.0, 3.0]
    o = _pia_state(orc, ar, 3, x, [[4, 1, 3, 3, 8, 8, 1], [2, 4, 5, 2, -1, -1, 0], [4, 6, 7, 2, 9, 10, 2]])
    pr = o.compute_props(mode=0)
    assert pr["np"][0].tolist() == [4, 2, 4] and pr["n"][0].tolist() == [14.0, 9.0, 32.0]
    for _ in range(3):
        o.delete_particle_end(0, 1)
    o.delete_particle_end_group(0, 3, 1)
    _mark_noncontiguous(o)
    o.squash(0)
    ind, _, _ = o.pia_get()
    assert ind[0, 0].tolist()[:4] == [1, 1, 1, 1] and ind[0, 0, 6] == 0
    assert ind[0, 1].tolist()[:4] == [2, 2, 3, 2] and ind[0, 1, 6] == 0
    assert ind[0, 2].tolist() == [3, 4, 4, 1, 5, 6, 2]
    pv = o.pv_get(0)
    assert not any(b in pv["index"][:6] for b in pv["buffer"][:pv["nbuffer"]])
    pr = o.compute_props(mode=0)
    assert pr["np"][0].tolist() == [1, 2, 3] and pr["n"][0].tolist() == [1.0, 9.0, 25.0]

    # 3 cells laid out 111 2 333 222; cell 2 ends with group 2 only
    x = [1.0, 1.0, 1.0, 2.0, 3.0, 3.0, 3.0, 2.0, 2.0, 2.0]
    o = _pia_state(orc, ar, 3, x, [[3, 1, 3, 3, -1, -1, 0], [4, 4, 4, 1, 8, 10, 3], [3, 5, 7, 3, -1, -1, 0]])
    pr = o.compute_props(mode=0)
    assert pr["np"][0].tolist() == [3, 4, 3] and pr["n"][0].tolist() == [6.0, 31.0, 18.0]
    o.delete_particle_end(0, 1)
    o.delete_particle_end(0, 3)
    o.delete_particle_end(0, 3)
    o.delete_particle_end_group(0, 2, 1)
    _mark_noncontiguous(o)
    o.squash(0)
    ind, _, _ = o.pia_get()
    assert ind[0, 0].tolist()[:4] == [2, 1, 2, 2] and ind[0, 0, 6] == 0
    assert ind[0, 1, 0] == 3 and ind[0, 1, 3] == 0 and ind[0, 1].tolist()[4:] == [4, 6, 3]
    assert ind[0, 2].tolist()[:4] == [1, 3, 3, 1] and ind[0, 2, 6] == 0
    pv = o.pv_get(0)
    assert not any(i in pv["buffer"][:pv["nbuffer"]] for i in pv["index"][:6])
    pr = o.compute_props(mode=0)
    assert pr["np"][0].tolist() == [2, 3, 1] and pr["n"][0].tolist() == [3.0, 27.0, 5.0]


RESTORE_CASES = [
    # (index, particles written through the index, buffer, nbuffer, expected buffer head)
    # test/test_particle_index_sorting.jl:13-168
    (list(range(1, 11)), 10, list(range(10, 0, -1)), 10, list(range(10, 0, -1))),
    ([5, 1, 7, 3, 2, 4, 10, 8, 6, 9], 2, [7, 3, 2, 4, 10, 8, 6, 9, 5, 1], 8, [10, 9, 8, 7, 6, 5, 4, 3]),
    ([10, 9, 5, 6, 1, 8, 3, 7, 2, 4], 7, [4, 7, 2, 10, 9, 5, 6, 1, 8, 3], 3, [10, 9, 8]),
    ([4, 10, 7, 3, 1, 2, 9, 8, 5, 6], 10, [4, 7, 2, 10, 9, 5, 6, 1, 8, 3], 0, []),
    ([10, 5, 7, 6, 2, 1, 3, 5, 4, 6], 5, [3, 7, 4, 1, 9, 10, 8, 2, 6, 5], 5, [10, 9, 8, 7, 6]),
]


@pytest.mark.parametrize("case", range(len(RESTORE_CASES)))
def test_restore_particle_ordering_known_answers(orc, golden, case):
    index, n_set, buffer, nbuffer, head = RESTORE_CASES[case]
    ar = scenario(golden, "octree_merge_24")["mass"]
    slots = np.zeros((10, 7))
    for i in range(1, n_set + 1):  # particles[i] = Particle(i, [i, 2i, 3i], [-i, -4i, -5i])
        slots[index[i - 1] - 1] = [i, i, 2 * i, 3 * i, -i, -4 * i, -5 * i]
    o = orc.Oracle(1, 1, [ar])
    o.pv_set(0, slots, index=index, buffer=buffer, nbuffer=nbuffer)
    o.restore_ordering(0)
    pv = o.pv_get(0)
    assert pv["index"].tolist() == list(range(1, 11))
    assert pv["nbuffer"] == nbuffer
    assert pv["buffer"][: len(head)].tolist() == head
    for i in range(1, n_set + 1 if nbuffer < 10 else 11):
        assert pv["particles"][i - 1].tolist() == [i, i, 2 * i, 3 * i, -i, -4 * i, -5 * i]


def _sampled_three_cells(orc, ar, nps, Ts, Fnum):
    o = orc.Oracle(3, 1, [ar])
    o.pv_create(0, 700)
    xcells = [0.0, 0.5, 1.0, 1.5]
    for c in range(3):
        o.sample_equal_weight(0, c + 1, nps[c], Ts[c], Fnum, box=(xcells[c], xcells[c + 1], 0, 1, 0, 1), seed=1234,
                              step=0)
    return o


def test_merge_and_squash_conserve_known_answers(orc, golden):
    # test/test_pia_contiguous.jl:324-439: cells of 100, 200 and 300 sampled
    # particles merged to 16 (N:2 octree, middle split, bounds from C), then
    # squashed; the temperatures are checked to 4.5 standard errors of the
    # sample (the reference's fixed bounds are met by its own stream)
    ar = scenario(golden, "octree_merge_24")["mass"]
    nps, Ts, Fnum = [100, 200, 300], [1000.0, 750.0, 600.0], 1e10
    for split_cell3 in (False, True):
        o = _sampled_three_cells(orc, ar, nps, Ts, Fnum)
        if split_cell3:
            ind, nt, cg = o.pia_get()
            ind[0, 2] = [300, 301, 304, 4, 305, 600, 296]
            o.pia_set(ind, nt, cg)
        pr = o.compute_props(mode=0)
        assert pr["np"][0].tolist() == nps
        for c in range(3):
            assert abs(pr["T"][0, c] - Ts[c]) / Ts[c] < 4.5 * np.sqrt(2.0 / (3.0 * nps[c]))
        T0 = pr["T"][0].copy()
        oc = orc.Octree(orc.SPLIT_MID, orc.INIT_C)
        order = (3, 2, 1) if split_cell3 else (1, 2, 3)
        expect_contiguous = (True, False, False) if split_cell3 else (False, False, False)
        for cell, contiguous in zip(order, expect_contiguous):
            o.merge_octree(oc, 0, cell, 16, seed=1234, step=1)
            assert bool(o.pia_get()[2][0]) == contiguous, (split_cell3, cell)
        o.squash(0)
        pr = o.compute_props(mode=0)
        assert np.all(pr["np"][0] < 30)
        for c in range(3):
            assert abs(pr["n"][0, c] - Fnum * nps[c]) / (Fnum * nps[c]) < 1e-15
            assert abs(pr["T"][0, c] - T0[c]) / T0[c] < 1e-14
        if not split_cell3:
            assert o.pv_get(0)["nbuffer"] == int(sum(nps) - pr["np"][0].sum()) + 700 - sum(nps)


def test_squash_pia_emptied_cells_known_answers(orc, golden):
    # test/test_pia_contiguous.jl:440-615: layout 111 2 333 222 with cell 1,
    # then cell 3, deleted to empty
    ar = scenario(golden, "octree_merge_24")["mass"]
    x = [1.0, 1.0, 1.0, 2.0, 3.0, 3.0, 3.0, 2.0, 2.0, 2.0]
    rows = [[3, 1, 3, 3, -1, -1, 0], [4, 4, 4, 1, 8, 10, 3], [3, 5, 7, 3, -1, -1, 0]]
    o = _pia_state(orc, ar, 3, x, rows)
    for _ in range(3):
        o.delete_particle_end(0, 1)
    _mark_noncontiguous(o)
    o.squash(0)
    ind, _, _ = o.pia_get()
    assert ind[0, 0].tolist()[:4] == [0, 0, -1, 0] and ind[0, 0, 6] == 0
    assert ind[0, 1].tolist() == [4, 1, 1, 1, 5, 7, 3]
    assert ind[0, 2].tolist()[:4] == [3, 2, 4, 3] and ind[0, 2, 6] == 0

    o = _pia_state(orc, ar, 3, x, rows)
    o.delete_particle_end(0, 1)
    for _ in range(3):
        o.delete_particle_end(0, 3)
    _mark_noncontiguous(o)
    pv = o.pv_get(0)
    assert pv["nbuffer"] == 4 and pv["buffer"][:4].tolist() == [3, 7, 6, 5]
    o.squash(0)
    ind, nt, _ = o.pia_get()
    assert ind[0, 0].tolist()[:4] == [2, 1, 2, 2] and ind[0, 0, 6] == 0
    assert ind[0, 1].tolist() == [4, 3, 3, 1, 4, 6, 3]
    assert ind[0, 2].tolist()[:4] == [0, 0, -1, 0] and ind[0, 2, 6] == 0
    pv = o.pv_get(0)
    assert not any(i in (3, 7, 6, 5) for i in pv["index"][: nt[0]])


def test_indexer_known_answers(orc, golden):
    # test/test_indexing.jl:1-63: appends go to group 2; map_cont_index walks
    # group 1, then group 2
    ar = scenario(golden, "octree_merge_24")["mass"]
    o = orc.Oracle(1, 1, [ar])
    o.pv_create(0, 64)
    ind, nt, cg = o.pia_get()
    ind[0, 0] = [20, 1, 20, 20, 0, -1, 0]
    nt[0] = 20
    o.pia_set(ind, nt, cg)
    o.indexer_new_particle(0, 1)
    o.indexer_new_particle(0, 1)
    ind, nt, _ = o.pia_get()
    assert nt[0] == 22 and ind[0, 0].tolist() == [22, 1, 20, 20, 21, 22, 2]

    ind[0, 0] = [15, 1, 10, 10, 31, 35, 5]
    nt[0] = 15
    o.pia_set(ind, nt, cg)
    assert [o.map_cont_index(0, 1, i0 - 1) for i0 in (1, 4, 10)] == [1, 4, 10]
    assert [o.map_cont_index(0, 1, i0 - 1) for i0 in (11, 12, 15)] == [31 + i0 - 10 - 1 for i0 in (11, 12, 15)]
    ind[0, 0] = [10, 24, 28, 5, 31, 35, 5]
    nt[0] = 10
    o.pia_set(ind, nt, cg)
    assert [o.map_cont_index(0, 1, i0 - 1) for i0 in (1, 4, 5)] == [24 + i0 - 1 for i0 in (1, 4, 5)]
    assert [o.map_cont_index(0, 1, i0 - 1) for i0 in (6, 8, 10)] == [31 + i0 - 5 - 1 for i0 in (6, 8, 10)]
