"""mw_dot_noalloc: the inner product for callers that cannot allocate GPU memory when they need it.

Such callers include a process whose device memory is held by another runtime's caching
allocator, and code that must not let cudaMalloc / cudaFree synchronise the device.  The entry
point computes the same sum as mw_dot with the same kernel.  Its node-pair lists and partial
sums sit in a fixed device array, reserved when the context is created, instead of freshly
allocated memory.

This file is collected last so that a run stopping at its first failure has run every other
test before it.  It passes on its own in a fresh process and after the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PAIRS = 32768  # the entry point's documented limit on nodes common to both trees


def _free_device_bytes():
    import torch
    free, _ = torch.cuda.mem_get_info(0)
    return free


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
    mra.synchronize()
    free0 = _free_device_bytes()
    for _ in range(2):  # the array keeps the previous call's contents: a second call must not see them
        for (x, y, ref) in ((a, b, ref_ab), (a, a, ref_aa)):
            v = ctypes.c_double(float("nan"))
            rc = lib.mw_dot_noalloc(x.ptr, y.ptr, ctypes.byref(v))
            assert rc == 0, lib.mw_last_error(mra.ptr)
            assert abs(v.value - ref) <= 1e-14 * abs(ref), (v.value, ref)
    # no device memory was taken by the calls (the array was reserved when the context was made)
    assert _free_device_bytes() == free0


def _uniform_keys(root_scale, depth):
    """Keys (scale, lx, ly, lz) of every node of a uniform tree `depth` scales below the 2x2x2 roots."""
    lv = np.array([(root_scale, x, y, z) for x in (-1, 0) for y in (-1, 0) for z in (-1, 0)], dtype=np.int32)
    out = [lv]
    for _ in range(depth):
        kids = np.repeat(lv, 8, axis=0)
        kids[:, 0] += 1
        off = np.array([(cx, cy, cz) for cz in (0, 1) for cy in (0, 1) for cx in (0, 1)], dtype=np.int32)
        kids[:, 1:] = 2 * kids[:, 1:] + np.tile(off, (len(lv), 1))
        lv = kids
        out.append(lv)
    return np.concatenate(out)


def test_dot_noalloc_rejects_more_pairs_than_its_array_holds(engine):
    lib = engine.load_library()
    mra = engine.MultiResolutionAnalysis(3)  # K = 4: 4 KiB blocks
    keys = _uniform_keys(-5, 4)               # 8 * (1 + 8 + 64 + 512 + 4096) = 37448 nodes
    assert len(keys) > MAX_PAIRS
    coefs = np.random.default_rng(5).standard_normal((len(keys), 8 * 4 ** 3))
    t = engine.FunctionTree(mra).upload(keys, coefs)
    v = ctypes.c_double(0.0)
    rc = lib.mw_dot_noalloc(t.ptr, t.ptr, ctypes.byref(v))
    assert rc == engine.MW_ERR_ARG
    msg = lib.mw_last_error(mra.ptr)
    msg = msg.decode() if isinstance(msg, bytes) else str(msg)
    assert str(MAX_PAIRS) in msg and "mw_dot" in msg, msg
    # the context stays usable, and the allocating entry point handles the same trees
    # mw_dot sums the root nodes' full blocks and every other node's wavelet part
    ref = float(np.sum(coefs[:8] ** 2) + np.sum(coefs[8:, 4 ** 3:] ** 2))
    assert abs(engine.dot(t, t) - ref) <= 1e-12 * ref
