"""Oracle parity on the benchmark's own workload: the 16-orbital Helmholtz batch at k=9.

The batch is bench.py's (same seed, same orbitals, same mu_i = sqrt(-2 eps_i)), applied as
HelmholtzVector::apply does (src/scf_solver/HelmholtzVector.cpp:141-159): one Helmholtz operator
per orbital, absolute precision, adaptive output grid.  The oracle (CPU, FP64) runs the complete
apply of a few orbitals on the same input trees; the GPU runs the whole batch in one batched
call, as the benchmark step does.

Bars:
  - plain FP64 GPU apply: node set (keys and leaf flags) bit-exact, coefficients within 1e-10
    relative L2 (summation order only);
  - norm-tiered mixed GPU apply: relative L2 <= prec against the oracle, and the same node set
    as the FP64 apply.  Node sets of the two modes could differ only where an output node's
    wavelet norm lies within the mixed error (< 1e-7 relative here) of its refinement threshold;
    on these seeded batches they are identical.
Also the same at prec 1e-5 and 1e-7 (the precision sweep of the benchmark's batch).
"""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402  (the benchmark's workload definition)

ORDER = 9


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def batch():
    rng = np.random.default_rng(bench.SEED)
    terms, mus = bench.orbital_terms(rng)
    return terms, mus


def _run(engine, oracle, terms, mus, prec, which):
    """Oracle applies of orbitals `which`; GPU FP64 and mixed batched applies of all orbitals
    on the oracle's input trees.  Returns, per checked orbital, (GPU fp64 tree, GPU mixed
    tree, oracle tree) and the GPU's engine objects."""
    mra, omra = engine.MultiResolutionAnalysis(ORDER), oracle.MRA(ORDER)
    ophis = []
    for t in terms:
        f = oracle.project_gauss(prec, oracle.Tree(omra), t, abs_prec=True)
        f.rescale(1.0 / f.norm())
        ophis.append(f)
    phis = []
    for f in ophis:
        k, c, _ = f.export()
        phis.append(engine.FunctionTree(mra).upload(k, c))
    ops = engine.HelmholtzOperator.batch(mra, [float(m) for m in mus], prec)
    n = len(phis)
    o64 = [engine.FunctionTree(mra) for _ in range(n)]
    omx = [engine.FunctionTree(mra) for _ in range(n)]
    engine.apply_batch([prec] * n, o64, ops, phis, abs_prec=True, precision="fp64")
    st = engine.apply_batch([prec] * n, omx, ops, phis, abs_prec=True, precision="mixed")
    assert st["items_tf32"] > 0 and st["items_fp32"] > 0  # the tiers the benchmark exercises ran
    outs = []
    for i in which:
        oout = oracle.Tree(omra)
        oracle.apply(prec, oout, oracle.helmholtz(omra, float(mus[i]), prec), ophis[i], abs_prec=True)
        outs.append((o64[i], omx[i], oout))
    return mra, outs


def _check(engine, mra, outs, prec):
    errs = []
    for g64, gmx, oout in outs:
        k2, c2, l2 = oout.export()
        k1, c1, l1 = g64.download()
        assert k1.shape == k2.shape and np.array_equal(k1, k2), "FP64 node set differs from the oracle"
        assert np.array_equal(l1, l2)
        e64 = rel_l2(c1, c2)
        assert e64 <= 1e-10, e64
        km, cm, lm = gmx.download()
        assert km.shape == k2.shape and np.array_equal(km, k2), "mixed node set differs from FP64 / oracle"
        assert np.array_equal(lm, l2)
        emx = rel_l2(cm, c2)
        assert emx <= prec, emx
        errs.append((e64, emx))
    return errs


def test_headline_batch_k9_prec1e6_matches_oracle(engine, oracle, batch):
    terms, mus = batch
    mra, outs = _run(engine, oracle, terms, mus, 1e-6, which=(0, 1, 2))
    errs = _check(engine, mra, outs, 1e-6)
    print("k=9 prec 1e-6 rel L2 vs oracle (fp64, mixed):", errs)


@pytest.mark.parametrize("prec", [1e-5, 1e-7])
def test_precision_sweep_matches_oracle(engine, oracle, batch, prec):
    terms, mus = batch
    mra, outs = _run(engine, oracle, terms, mus, prec, which=(0, 1))
    errs = _check(engine, mra, outs, prec)
    print("k=9 prec %g rel L2 vs oracle (fp64, mixed):" % prec, errs)


def test_rotation_matches_oracle_add(engine, oracle):
    """mw_rotate (orbital::rotate, src/qmfunctions/orbital_utils.cpp:242-248) against the oracle's
    linear combination on the inputs' union grid, row by row of U."""
    prec = 1e-6
    mra, omra = engine.MultiResolutionAnalysis(7), oracle.MRA(7)
    oins = [oracle.project_gauss(prec, oracle.Tree(omra), [(1.0, a, (0.2 * i, -0.1 * i, 0.05), (i % 2, 0, 0))])
            for i, a in enumerate((0.5, 2.0, 8.0, 30.0))]
    ins = []
    for f in oins:
        k, c, _ = f.export()
        ins.append(engine.FunctionTree(mra).upload(k, c))
    U = np.linalg.qr(np.random.default_rng(11).standard_normal((4, 4)))[0]
    outs = [engine.FunctionTree(mra) for _ in range(4)]
    engine.rotate(outs, ins, U)
    for i in range(4):
        oout = oracle.Tree(omra)
        oracle.add(-1.0, oout, U[i], oins)
        k1, c1, l1 = outs[i].download()
        k2, c2, l2 = oout.export()
        assert np.array_equal(k1, k2) and np.array_equal(l1, l2)
        assert rel_l2(c1, c2) <= 1e-13
