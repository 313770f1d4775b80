"""Device validators of the indexing (check_pia_is_correct, check_unique_index,
check_unique_buffer, count_disordered_particles; particles.jl:805-1025):
they hold on every state the device path produces, agree with the oracle's
checks of the reference's structures on the same states, and catch the
inconsistencies the reference's own checks catch when an indexer is edited by
hand (test_pia_contiguous.jl builds such indexers)."""
import numpy as np
import pytest

import merzgpu as mz
from helpers import interactions, oracle_state, random_particles, species

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import merzgpu.build as b

    b.build()
    c = mz.Context(0)
    yield c
    c.close()


def test_validators_hold_through_the_device_path_and_agree_with_the_oracle(ctx, orc):
    sp = species(["Ar"])
    inter = interactions(sp)
    rng = np.random.default_rng(8)
    n_cells, n = 40, 6000
    arrays = random_particles(rng, n, n_cells, L=5e-4, wspan=1.0)
    dom = mz.Domain(ctx, n_cells, sp, 4 * n, interactions=inter, seed=8)
    dom.upload(0, *arrays)
    o = oracle_state(orc, n_cells, sp, mz.VHS, [arrays], capacity=4 * n)
    smax = mz.estimate_sigma_g_w_max(inter[0][0], sp[0], sp[0], 300.0, 300.0, 1e12)
    dom.set_sigma_g_w_max(0, 0, smax)
    o.cf_set_smax(0, 0, smax)
    grid = mz.Grid1DUniform(5e-4, n_cells)
    octree = mz.OctreeN2Merge(max_Nbins=4096)
    oc = orc.Octree(orc.SPLIT_MID, mz.OctreeInitBinMinMaxVel, mz.OctreeBinBoundsInherit, 4096, 10)
    for stage in ("uploaded", "split", "merged", "sorted"):
        if stage == "split":
            # splits land in group 2 of each cell; unused reserved slots are free
            dom.ntc(0, 0, 2.0, 1, equal_weight=False)
            o.ntc_cells(0, 0, 2.0, None, 8, 1, equal_weight=False)
            assert dom.counters()["splits"] > 50
        elif stage == "merged":
            dom.merge_octree(0, octree, 60, threshold=160, grid=grid, step=1)
            ind, _, _ = o.pia_get()
            for c in np.nonzero(ind[0, :, 0] > 160)[0]:
                o.merge_octree(oc, 0, int(c) + 1, 60, L=grid.L, nx=n_cells, seed=8, step=1)
        elif stage == "sorted":
            dom.sort(0, grid)
            o.sort(0, L=grid.L, nx=n_cells)
        assert dom.check_pia_is_correct(0) == (True, 0), stage
        assert dom.check_unique_index(0) == (True, 0), stage
        assert dom.check_unique_buffer(0) == (True, 0), stage
        assert o.check_pia(0)[0] and o.check_unique_index(0)[0] and o.check_unique_buffer(0)[0], stage
        assert dom.count_disordered_particles(0, use_offset=True) == 0, stage
    # sorted: particles lie in index order, cell by cell
    assert dom.count_disordered_particles(0, use_offset=False) == 0
    dom.close()


def test_validators_catch_hand_edited_indexers(ctx):
    sp = species(["Ar"])
    inter = interactions(sp)
    rng = np.random.default_rng(3)
    n_cells = 4
    w, v, x, _ = random_particles(rng, 40, n_cells)
    cell = np.repeat(np.arange(n_cells, dtype=np.int32), 10)
    dom = mz.Domain(ctx, n_cells, sp, 200, interactions=inter, seed=3)
    dom.upload(0, w, v, x, cell)
    assert dom.check_pia_is_correct(0) == (True, 0)

    def row(s1, n1, s2=0, n2=0):
        return (n1 + n2, s1 if n1 else 0, s1 + n1 - 1 if n1 else -1, n1, s2 if n2 else 0, s2 + n2 - 1 if n2 else -1, n2)

    good = [row(10 * c, 10) for c in range(n_cells)]
    dom.set_indexer(0, good, 40)
    assert dom.check_pia_is_correct(0) == (True, 0)
    assert dom.check_unique_index(0) == (True, 0)
    # a wrong n_total: check_pia_is_correct returns (false, 0)
    dom.set_indexer(0, good, 41)
    assert dom.check_pia_is_correct(0) == (False, 0)
    # cell 3 (1-based) also lists cell 2's first five particles: two indices
    # point at the same particle
    bad = list(good)
    bad[2] = row(20, 10, 10, 5)
    dom.set_indexer(0, bad, 45)
    assert dom.check_pia_is_correct(0) == (True, 0)
    assert dom.check_unique_index(0) == (False, 2)
    # free slots: 50 slots of which the cells list 40 (slots 10-11, 22-24
    # and 35-39 are free, the reference's buffer)
    w50, v50, x50, _ = random_particles(rng, 50, n_cells)
    layout = [row(0, 10), row(12, 10), row(25, 10), row(40, 10)]
    dom.upload_indexed(0, w50, v50, x50, layout)
    assert dom.check_pia_is_correct(0) == (True, 0)
    assert dom.check_unique_index(0) == (True, 0)
    # cell 1 also lists free slot 10: (false, -1)
    edited = list(layout)
    edited[0] = row(0, 10, 10, 1)
    dom.set_indexer(0, edited, 41)
    assert dom.check_pia_is_correct(0) == (True, 0)
    assert dom.check_unique_index(0) == (False, -1)
    # cells 1 and 2 both list free slot 10: (false, -2)
    edited[1] = row(12, 10, 10, 1)
    dom.set_indexer(0, edited, 42)
    assert dom.check_unique_index(0) == (False, -2)
    # the groups sit where the index order puts them except cell 2's and
    # later ones (gaps): count_disordered_particles without offsets counts them
    dom.set_indexer(0, layout, 40)
    assert dom.count_disordered_particles(0, use_offset=False) == 30
    assert dom.count_disordered_particles(0, use_offset=True) == 0
    # groups outside the slots in use are refused at the boundary
    with pytest.raises(Exception):
        dom.set_indexer(0, [row(0, 10**6)] + good[1:], 40)
    dom.close()
