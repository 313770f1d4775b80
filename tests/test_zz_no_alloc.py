"""mz_sort_keys_noalloc -- the entry point that allocates nothing -- against the
regular sort entry point (mz_sort), through the C ABI, on calls in a row.

It exists for callers that cannot allocate device memory once running: a
process whose GPU memory already belongs to another framework's caching
allocator, or a loop that must not take the device-wide synchronisation of
cudaMalloc / cudaFree.  Such a caller passes its own device buffers; torch
tensors stand in for them here.  The entry point keeps its per-cell counters in
a static device array (at most MZ_NOALLOC_MAX_CELLS cells) shared by every call,
so consecutive calls must not see each other's counts."""
import ctypes as C

import numpy as np
import pytest

import merzgpu as mz

pytestmark = pytest.mark.gpu


def _keys_and_reference(ctx, n_cells, n, seed):
    rng = np.random.default_rng(seed)
    grid = mz.Grid1DUniform(5e-4, n_cells)
    sp = [mz.Species("Ar", mz.AR_MASS)]
    x = np.column_stack([rng.uniform(grid.min_x, grid.max_x, n), np.arange(n, dtype=float), np.zeros(n)])
    v = rng.normal(0.0, 300.0, (n, 3))
    w = np.full(n, 1e12)
    dom = mz.Domain(ctx, n_cells, sp, n)
    dom.upload(0, w, v, x, np.zeros(n, np.int32))   # logical order = upload order
    perm = dom.sort(0, grid, return_index=True)      # the regular entry point
    ind, nt = dom.indexer(0)
    dom.close()
    keys = np.floor(x[:, 0] * grid.inv_dx).astype(np.int32)  # get_cell, the same FP64 product and floor
    return keys, perm, ind


def test_noalloc_sort_matches_regular_sort_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    import merzgpu.build as b

    b.build()
    lib = mz.lib()
    ctx = mz.Context(0)
    torch.cuda.set_device(0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    cases = [(2000, 300000, 1), (2000, 300000, 1), (777, 50000, 2), (3, 5000, 3)]
    for n_cells, n, seed in cases:
        keys, perm_ref, ind = _keys_and_reference(ctx, n_cells, n, seed)
        d_keys = torch.from_numpy(keys).cuda()
        d_perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        d_start = torch.full((n_cells + 1,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = lib.mz_sort_keys_noalloc(stream, C.c_void_p(d_keys.data_ptr()), n, n_cells,
                                      C.c_void_p(d_perm.data_ptr()), C.c_void_p(d_start.data_ptr()))
        assert rc == mz._lib.MZ_OK
        perm = d_perm.cpu().numpy()
        start = d_start.cpu().numpy()
        assert np.array_equal(perm, perm_ref.astype(np.int32))        # same stable permutation
        assert np.array_equal(np.diff(start), ind[:, 3])              # same per-cell counts
        nz = ind[:, 3] > 0
        assert np.array_equal(start[:-1][nz], ind[nz, 1])             # same cell starts
        assert start[-1] == n
    # sizes beyond the stated maximum are rejected before touching the GPU
    assert lib.mz_sort_keys_noalloc(stream, None, 0, mz._lib.NOALLOC_MAX_CELLS + 1, None,
                                    C.c_void_p(d_start.data_ptr())) == mz._lib.MZ_E_ARG
    ctx.close()


def test_noalloc_sort_at_its_maximum_and_with_a_bad_key():
    """At MZ_NOALLOC_MAX_CELLS cells (the one-block scan then runs 256 cells
    per thread) the permutation is numpy's stable argsort and the cell starts
    the prefix sums of the counts; a key equal to n_cells is clamped and
    reported as MZ_E_STATE, and the next call is clean again."""
    torch = pytest.importorskip("torch")
    import merzgpu.build as b

    b.build()
    lib = mz.lib()
    torch.cuda.set_device(0)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    n_cells = mz._lib.NOALLOC_MAX_CELLS
    rng = np.random.default_rng(11)
    for n in (3 * n_cells, 1000):
        keys = rng.integers(0, n_cells, n).astype(np.int32)
        d_keys = torch.from_numpy(keys).cuda()
        d_perm = torch.full((n,), -1, dtype=torch.int32, device="cuda")
        d_start = torch.full((n_cells + 1,), -1, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        rc = lib.mz_sort_keys_noalloc(stream, C.c_void_p(d_keys.data_ptr()), n, n_cells,
                                      C.c_void_p(d_perm.data_ptr()), C.c_void_p(d_start.data_ptr()))
        assert rc == mz._lib.MZ_OK
        assert np.array_equal(d_perm.cpu().numpy(), np.argsort(keys, kind="stable").astype(np.int32))
        start = np.concatenate(([0], np.cumsum(np.bincount(keys, minlength=n_cells))))
        assert np.array_equal(d_start.cpu().numpy(), start.astype(np.int32))
    n_cells, n = 50, 400
    keys = rng.integers(0, n_cells, n).astype(np.int32)
    keys[123] = n_cells
    d_keys = torch.from_numpy(keys).cuda()
    d_perm = torch.zeros((n,), dtype=torch.int32, device="cuda")
    d_start = torch.zeros((n_cells + 1,), dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    args = (stream, C.c_void_p(d_keys.data_ptr()), n, n_cells, C.c_void_p(d_perm.data_ptr()),
            C.c_void_p(d_start.data_ptr()))
    assert lib.mz_sort_keys_noalloc(*args) == mz._lib.MZ_E_STATE
    d_keys[123] = n_cells - 1
    torch.cuda.synchronize()
    assert lib.mz_sort_keys_noalloc(*args) == mz._lib.MZ_OK
    keys[123] = n_cells - 1
    assert np.array_equal(d_perm.cpu().numpy(), np.argsort(keys, kind="stable").astype(np.int32))
