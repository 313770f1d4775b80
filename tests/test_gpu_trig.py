"""The device sine/cosine of the scattering angle phi = 2 pi rand()
(table-driven, sincos_2pi_u52) against extended-precision values.

The collision kernels use it in place of a general sincos; the test bounds
its error at a few units in the last place over random draws and the sector
edges of its table."""
import numpy as np
import pytest

import merzgpu as mz
from merzgpu import _lib

pytestmark = pytest.mark.gpu


def _exact(m):
    ld = np.longdouble
    if np.finfo(ld).nmant < 63:
        pytest.skip("no extended precision long double on this host")
    two_pi = 2 * np.arccos(ld(-1))
    a = two_pi * (m.astype(ld) / ld(2.0 ** 52))
    return np.sin(a), np.cos(a)


def test_sincos_2pi_against_extended_precision():
    import ctypes as C

    rng = np.random.default_rng(7)
    m = rng.integers(0, 2 ** 52, 200_000, dtype=np.uint64)
    step = np.uint64(1) << np.uint64(44)
    edges = np.arange(256, dtype=np.uint64) * step
    m = np.concatenate([m, edges, edges + np.uint64(1), edges + step - np.uint64(1),
                        np.array([0, 2 ** 52 - 1, 2 ** 50, 2 ** 51, 3 * 2 ** 50], dtype=np.uint64)])
    ctx = mz.Context(0)
    s = np.empty(m.size)
    c = np.empty(m.size)
    rc = _lib.lib().mz_sincos_2pi(ctx.h, m.size, m.ctypes.data_as(C.POINTER(C.c_uint64)), _lib.ptr(s), _lib.ptr(c))
    assert rc == _lib.MZ_OK
    es, ec = _exact(m)
    # two ulp of the value (of 1/64 near the zeros of sin and cos)
    tol_s = 2 * np.spacing(np.maximum(np.abs(es).astype(np.float64), 1 / 64))
    tol_c = 2 * np.spacing(np.maximum(np.abs(ec).astype(np.float64), 1 / 64))
    err_s = np.abs((s - es).astype(np.float64))
    err_c = np.abs((c - ec).astype(np.float64))
    assert np.all(err_s <= tol_s), f"sin: worst {np.max(err_s / tol_s):.2f} of tolerance"
    assert np.all(err_c <= tol_c), f"cos: worst {np.max(err_c / tol_c):.2f} of tolerance"
    # mean error well below one ulp (of 1/64 near the zeros)
    assert np.mean(err_s / (tol_s / 2)) < 0.5
    assert np.mean(err_c / (tol_c / 2)) < 0.5
    ctx.close()
