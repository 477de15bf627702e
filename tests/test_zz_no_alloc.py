"""mw_dot_noalloc: the inner product for callers that cannot allocate GPU memory when they need it.

Such callers include a process whose device memory is held by another runtime's caching
allocator, and code that must not let cudaMalloc / cudaFree synchronise the device.  The entry
point computes the same sum as mw_dot with the same kernel.  Its node-pair lists and partial
sums sit in a fixed device array instead of freshly allocated memory.

This file is collected last so that a run stopping at its first failure has run every other
test before it.  It passes on its own in a fresh process and after the other tests.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_dot_noalloc_matches_dot_twice(engine):
    lib = engine.load_library()
    mra = engine.MultiResolutionAnalysis(7)
    a = engine.project(1e-6, engine.FunctionTree(mra), [(1.0, 1.5, (0.2, 0.0, -0.1), (1, 0, 0)),
                                                        (0.4, 6.0, (-0.5, 0.3, 0.0), (0, 0, 0))])
    b = engine.project(1e-6, engine.FunctionTree(mra), [(0.8, 2.5, (0.1, 0.1, 0.0), (0, 0, 1)),
                                                        (0.3, 0.9, (0.0, -0.4, 0.2), (0, 0, 0))])
    ref_ab = engine.dot(a, b)
    ref_aa = engine.dot(a, a)
    assert ref_ab != 0.0 and ref_aa > 0.0
    for _ in range(2):  # the array keeps the previous call's contents: a second call must not see them
        for (x, y, ref) in ((a, b, ref_ab), (a, a, ref_aa)):
            v = ctypes.c_double(float("nan"))
            rc = lib.mw_dot_noalloc(x.ptr, y.ptr, ctypes.byref(v))
            assert rc == 0, lib.mw_last_error(mra.ptr)
            assert abs(v.value - ref) <= 1e-14 * abs(ref), (v.value, ref)
