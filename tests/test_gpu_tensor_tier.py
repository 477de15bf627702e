"""The TF32 tensor-core tier of the norm-tiered apply (precision "mixed").

Items whose screening bound b is at most 2e3 x the screening threshold run on the tensor cores
(operands rounded to TF32, FP32 accumulation), so each is off by at most about 3e-3 b.  Checked:
- every basis order (k = 3..9, both tile tails of the kernel) with absolute and relative
  precision: the tier is used, and the result is within prec of the FP64 apply (relative L2 of
  the difference tree, computed on the union grid);
- the error stays within a small multiple of the FP32-only tiering ("mixed-fp32");
- a function with only wavelet content below the root scale still excludes the scaling-scaling
  path exactly (a wrong exclusion gives an O(1) error);
- reruns are bit-identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAUSS = [(1.0, 3.0, (0.15, -0.1, 0.05), (0, 0, 0)), (0.6, 12.0, (-0.4, 0.3, 0.2), (1, 0, 0)),
         (0.3, 40.0, (0.5, 0.25, -0.35), (0, 1, 1))]


def diff_norm(engine, mra, a, b):
    d = engine.FunctionTree(mra)
    engine.add(-1.0, d, [(1.0, a), (-1.0, b)])
    return d.norm()


def run(engine, mra, op, inp, prec, precision, abs_prec):
    out = engine.FunctionTree(mra)
    st = engine.apply(prec, out, op, inp, abs_prec=abs_prec, precision=precision)
    return out, st


@pytest.mark.parametrize("order", [3, 4, 5, 6, 7, 8, 9])
@pytest.mark.parametrize("abs_prec", [True, False])
def test_tensor_tier_every_order(engine, order, abs_prec):
    prec = 1e-5
    mra = engine.MultiResolutionAnalysis(order)
    f = engine.project(prec, engine.FunctionTree(mra), GAUSS, abs_prec=True)
    f.rescale(1.0 / f.norm())
    H = engine.HelmholtzOperator(mra, 1.3, prec)
    v64, s64 = run(engine, mra, H, f, prec, "fp64", abs_prec)
    vtc, stc = run(engine, mra, H, f, prec, "mixed", abs_prec)
    v32, s32 = run(engine, mra, H, f, prec, "mixed-fp32", abs_prec)
    assert s64["items_tf32"] == 0 and s32["items_tf32"] == 0
    assert stc["items_tf32"] > 0
    n64 = v64.norm()
    e_tc = diff_norm(engine, mra, vtc, v64) / n64
    e_32 = diff_norm(engine, mra, v32, v64) / n64
    assert e_tc <= prec, (e_tc, stc)
    assert e_32 <= prec
    assert e_tc <= max(300.0 * e_32, 0.05 * prec), (e_tc, e_32)


def test_tensor_tier_poisson_wavelet_input(engine):
    # input: the difference of two nearby Gaussians (little scaling content at coarse scales)
    prec = 1e-6
    mra = engine.MultiResolutionAnalysis(7)
    terms = [(1.0, 20.0, (0.0, 0.0, 0.0), (0, 0, 0)), (-1.0, 20.0, (0.02, -0.01, 0.015), (0, 0, 0))]
    f = engine.project(prec, engine.FunctionTree(mra), terms, abs_prec=True)
    P = engine.PoissonOperator(mra, prec)
    v64, _ = run(engine, mra, P, f, prec, "fp64", True)
    vtc, stc = run(engine, mra, P, f, prec, "mixed", True)
    assert stc["items_tf32"] > 0
    assert diff_norm(engine, mra, vtc, v64) <= prec * max(v64.norm(), 1.0)


def test_tensor_tier_rerun_bit_identical(engine):
    prec = 1e-5
    mra = engine.MultiResolutionAnalysis(9)
    f = engine.project(prec, engine.FunctionTree(mra), GAUSS, abs_prec=True)
    H = engine.HelmholtzOperator(mra, 0.7, prec)
    a, _ = run(engine, mra, H, f, prec, "mixed", True)
    b, _ = run(engine, mra, H, f, prec, "mixed", True)
    ka, ca, _ = a.download()
    kb, cb, _ = b.download()
    assert np.array_equal(ka, kb) and np.array_equal(ca, cb)


def test_overlapped_groups_bit_identical_to_serial(engine):
    # the batched apply pipelines two job groups on two streams; results must not depend on it
    prec = 1e-5
    mra = engine.MultiResolutionAnalysis(7)
    rng = np.random.default_rng(11)
    phis, ops = [], []
    for i in range(5):
        c = tuple(rng.uniform(-1.0, 1.0, 3))
        f = engine.project(prec, engine.FunctionTree(mra), [(1.0, float(rng.uniform(1.0, 20.0)), c, (i % 2, 0, 0))],
                           abs_prec=True)
        phis.append(f)
        ops.append(engine.HelmholtzOperator(mra, float(rng.uniform(0.5, 2.0)), prec))
    res = {}
    for on in (True, False):
        mra.set_overlap(on)
        outs = [engine.FunctionTree(mra) for _ in phis]
        engine.apply_batch([prec] * 5, outs, ops, phis, abs_prec=True, precision="mixed")
        res[on] = [o.download() for o in outs]
    mra.set_overlap(True)
    for (k1, c1, l1), (k2, c2, l2) in zip(res[True], res[False]):
        assert np.array_equal(k1, k2) and np.array_equal(c1, c2) and np.array_equal(l1, l2)


@pytest.mark.gpu
def test_job_group_count_bit_identical(engine):
    # the number of pipelined job groups (1..8) changes only the schedule, never a result
    prec = 1e-5
    mra = engine.MultiResolutionAnalysis(9)
    rng = np.random.default_rng(12)
    phis, ops = [], []
    for i in range(6):
        c = tuple(rng.uniform(-1.0, 1.0, 3))
        f = engine.project(prec, engine.FunctionTree(mra), [(1.0, float(rng.uniform(1.0, 20.0)), c, (i % 3, 0, 1))],
                           abs_prec=True)
        phis.append(f)
        ops.append(engine.HelmholtzOperator(mra, float(rng.uniform(0.5, 2.0)), prec))
    res = {}
    for g in (1, 2, 3, 4, 6, 8):
        mra.set_groups(g)
        outs = [engine.FunctionTree(mra) for _ in phis]
        st = engine.apply_batch([prec] * 6, outs, ops, phis, abs_prec=True, precision="mixed")
        assert st["items_tf32"] > 0
        res[g] = [o.download() for o in outs]
    mra.set_overlap(True)
    for g in res:
        for (k1, c1, l1), (k2, c2, l2) in zip(res[1], res[g]):
            assert np.array_equal(k1, k2) and np.array_equal(c1, c2) and np.array_equal(l1, l2)
    with pytest.raises(engine.MWError):
        mra.set_groups(9)


def test_autotune_batch(engine):
    # the autotuner keeps one of its candidates, and the tuned apply agrees with the default one far
    # below the requested (absolute) precision: chunk sizes change only the order of the sums.  The
    # FP32-accuracy tier accumulates in FP32 on the tensor cores, items up to 2e6 x the screening
    # threshold: regrouping them moves the sum by a few 1e-3 of prec (5.4e-3 measured)
    prec = 1e-5
    mra = engine.MultiResolutionAnalysis(9)
    rng = np.random.default_rng(13)
    phis, ops = [], []
    for i in range(5):
        c = tuple(rng.uniform(-1.0, 1.0, 3))
        f = engine.project(prec, engine.FunctionTree(mra), [(1.0, float(rng.uniform(1.0, 20.0)), c, (i % 2, 1, 0))],
                           abs_prec=True)
        phis.append(f)
        ops.append(engine.HelmholtzOperator(mra, float(rng.uniform(0.5, 2.0)), prec))
    ref = [engine.FunctionTree(mra) for _ in phis]
    engine.apply_batch([prec] * 5, ref, ops, phis, abs_prec=True, precision="mixed")
    outs = [engine.FunctionTree(mra) for _ in phis]
    t = engine.autotune_batch([prec] * 5, outs, ops, phis, abs_prec=True, precision="mixed", repeats=1)
    assert 2 <= t["groups"] <= 6 and t["ms"] > 0.0
    assert t["chunk"]["tf32"] in (48, 96, 192) and t["chunk"]["fp32"] in (16, 32, 64) and t["chunk"]["df32"] in (4, 8, 16)
    tuned = [engine.FunctionTree(mra) for _ in phis]
    engine.apply_batch([prec] * 5, tuned, ops, phis, abs_prec=True, precision="mixed")
    for a, b, r in zip(outs, tuned, ref):
        for x in (a, b):
            d = engine.FunctionTree(mra)
            engine.add(-1.0, d, [(1.0, x), (-1.0, r)])
            assert d.norm() <= 2e-2 * prec
    mra.set_overlap(False)
    with pytest.raises(engine.MWError):
        engine.autotune_batch([prec] * 5, outs, ops, phis, abs_prec=True, precision="mixed", repeats=1)
    mra.set_overlap(True)


def test_row_counts(engine):
    # every tier kernel sums the x passes of a row (consecutive items of a node with the same term,
    # ly and lz) before one y and one z pass, and counts its rows: at most one per item, and fewer
    # rows than items where neighbouring translations survive together
    prec = 1e-5
    mra = engine.MultiResolutionAnalysis(9)
    f = engine.project(prec, engine.FunctionTree(mra), GAUSS, abs_prec=True)
    H = engine.HelmholtzOperator(mra, 1.1, prec)
    for precision, main in (("mixed", "tf32"), ("fp64", "fp64"), ("mixed-fp32", "fp32"), ("df", "df")):
        _, st = run(engine, mra, H, f, prec, precision, True)
        assert st["items_" + main] > 0, (precision, st)
        for t in ("fp64", "fp32", "tf32", "df"):
            items, rows = st["items_" + t], st["rows_" + t]
            assert (0 < rows <= items) if items else rows == 0, (precision, t, rows, items)
        assert sum(st["rows_" + t] for t in ("fp64", "fp32", "tf32", "df")) < st["items"], (precision, st)
