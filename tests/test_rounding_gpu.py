"""The step kernels turn binary64 cell-relative positions into binary32
with integer operations (d2f_rn in fmdg_df.cuh; the conversion instruction
issues at the binary64 rate on GB300).  Its results must be the conversion
instruction's, bit for bit, on every kind of input: random positions,
exact ties and their neighbours, powers of two, the edges of the normal
range, subnormals, zeros, infinities and values beyond the binary32 range.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs():
    rng = np.random.default_rng(11)
    x = [rng.uniform(-40.0, 40.0, 200000), rng.standard_normal(20000) * 1e-3,
         np.exp(rng.uniform(-80.0, 80.0, 20000)) * rng.choice([-1.0, 1.0], 20000)]
    # halfway between neighbouring binary32 numbers, and one binary64 ulp either side
    f = rng.uniform(-40.0, 40.0, 20000).astype(np.float32)
    mid = (f.astype(np.float64) + np.nextafter(f, np.float32(np.inf)).astype(np.float64)) / 2.0
    x += [mid, np.nextafter(mid, -np.inf), np.nextafter(mid, np.inf)]
    special = [0.0, -0.0, 1.0, -1.0, 2.0 ** -126, -(2.0 ** -126), 2.0 ** -127, 2.0 ** -149, 2.0 ** -150,
               1e-300, float(np.finfo(np.float32).max), 2.0 ** 128, -(2.0 ** 128), 3.5e38, np.inf, -np.inf]
    x.append(np.array(special))
    return np.ascontiguousarray(np.concatenate(x), dtype=np.float64)


def test_d2f_matches_conversion(gpu_lib):
    L = gpu_lib.L
    L.fmdg_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    L.fmdg_check_d2f.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.fmdg_destroy.argtypes = [C.c_void_p]
    h = C.c_void_p()
    assert L.fmdg_create(C.byref(h), 0) == 0
    x = _inputs()
    ours = np.zeros(len(x), np.float32)
    ref = np.zeros(len(x), np.float32)
    assert L.fmdg_check_d2f(h, x.ctypes.data, len(x), ours.ctypes.data, ref.ctypes.data) == 0
    L.fmdg_destroy(h)
    np.testing.assert_array_equal(ours.view(np.uint32), ref.view(np.uint32))
    # and both are IEEE round-to-nearest-even (results in the binary32
    # subnormal range left out: they depend on the flush-to-zero mode)
    keep = (np.abs(x) >= 2.0 ** -126) | (x == 0.0)
    with np.errstate(over="ignore"):
        np.testing.assert_array_equal(ref[keep].view(np.uint32), x[keep].astype(np.float32).view(np.uint32))


def test_ttm_reciprocal_error_bound(gpu_lib):
    """The TTM solver's reciprocal (binary32 seed, two Newton-Raphson steps)
    stays within 2 ulps of 1.0 / x over the electron temperatures and heat
    capacities it meets (1e-3 to 1e9) and across binary32 seed ties."""
    L = gpu_lib.L
    L.fmdg_create.argtypes = [C.POINTER(C.c_void_p), C.c_int]
    L.fmdg_check_recip.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.fmdg_destroy.argtypes = [C.c_void_p]
    h = C.c_void_p()
    assert L.fmdg_create(C.byref(h), 0) == 0
    rng = np.random.default_rng(12)
    f = rng.uniform(1.0, 2.0, 20000).astype(np.float32)
    mid = (f.astype(np.float64) + np.nextafter(f, np.float32(np.inf)).astype(np.float64)) / 2.0
    x = np.concatenate([np.exp(rng.uniform(np.log(1e-3), np.log(1e9), 200000)), rng.uniform(290.0, 3e4, 100000),
                        mid, np.nextafter(mid, 0.0), [1.0, 2.0, 3.0, 300.0, 1e9]])
    x = np.ascontiguousarray(x, dtype=np.float64)
    ours = np.zeros_like(x)
    ref = np.zeros_like(x)
    assert L.fmdg_check_recip(h, x.ctypes.data, len(x), ours.ctypes.data, ref.ctypes.data) == 0
    L.fmdg_destroy(h)
    np.testing.assert_array_equal(ref, 1.0 / x)
    ulps = np.abs(ours - ref) / np.spacing(ref)
    assert ulps.max() <= 2.0, ulps.max()
