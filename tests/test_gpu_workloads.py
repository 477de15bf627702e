"""The benchmark workloads at their full sizes, on the GPU, with size-independent checks.

1. Poisson FP64 apply of 4 normalized Gaussians (k=7, prec 1e-5): analytic erf potential and
   oracle parity on the same input tree.
3. The 16-orbital Helmholtz batch (k=9) at prec 1e-5 and 1e-7, norm-tiered precision: relative
   L2 error of every orbital against the plain FP64 apply.
4. Exchange-like batch: 32 Gaussian-polynomial orbitals, all 528 pair products (tree multiply)
   and their Poisson applies with precision-steering trees (k=7, prec 1e-5), mixed precision:
   error per pair against FP64, and one pair against the oracle.
Also: linearity (apply(2f) = 2 apply(f)) and bit-identical reruns.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SEED = 20261203


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def gaussian_density(rng, n, lo, hi):
    alphas = np.exp(rng.uniform(np.log(lo), np.log(hi), n))
    centres = rng.uniform(-2, 2, (n, 3))
    return alphas, centres, [((a / math.pi) ** 1.5, a, tuple(c), (0, 0, 0)) for a, c in zip(alphas, centres)]


def poly_orbitals(rng, n, lo, hi):
    mons = [(a, b, c) for a in range(4) for b in range(4) for c in range(4) if a + b + c <= 3]
    out = []
    for _ in range(n):
        alpha = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        R = rng.uniform(-2.0, 2.0, 3)
        out.append([(float(c), alpha, tuple(R), m) for c, m in zip(rng.standard_normal(len(mons)), mons)])
    return out


def test_config1_poisson_fp64(engine, oracle):
    prec = 1e-5
    rng = np.random.default_rng(SEED)
    alphas, centres, terms = gaussian_density(rng, 4, 0.5, 50.0)
    mra, omra = engine.MultiResolutionAnalysis(7), oracle.MRA(7)
    orho = oracle.project_gauss(prec, oracle.Tree(omra), terms)
    k, c, _ = orho.export()
    rho = engine.FunctionTree(mra).upload(k, c)
    V = engine.FunctionTree(mra)
    engine.apply(prec, V, engine.PoissonOperator(mra, prec), rho, precision="fp64")
    oV = oracle.Tree(omra)
    oracle.apply(prec, oV, oracle.poisson(omra, prec), orho)
    k1, c1, _ = V.download()
    k2, c2, _ = oV.export()
    assert np.array_equal(k1, k2)
    assert rel_l2(c1, c2) <= 1e-10
    pts = rng.uniform(-4, 4, (300, 3))
    exact = np.array([sum(math.erf(math.sqrt(a) * np.linalg.norm(p - r)) / np.linalg.norm(p - r)
                          for a, r in zip(alphas, centres)) for p in pts])
    assert np.abs(V.evalf(pts) - exact).max() <= 10 * prec * np.abs(exact).max()


@pytest.mark.parametrize("prec", [1e-5, 1e-7])
def test_config3_mixed_error_per_orbital(engine, prec):
    rng = np.random.default_rng(SEED)
    terms = poly_orbitals(rng, 16, 0.3, 20.0)
    mus = np.sqrt(-2.0 * rng.uniform(-2.0, -0.1, 16))
    mra = engine.MultiResolutionAnalysis(9)
    phis = []
    for t in terms:
        f = engine.project(prec, engine.FunctionTree(mra), t, abs_prec=True)
        f.rescale(1.0 / f.norm())
        phis.append(f)
    ops = [engine.HelmholtzOperator(mra, float(m), prec) for m in mus]
    o64 = [engine.FunctionTree(mra) for _ in phis]
    omx = [engine.FunctionTree(mra) for _ in phis]
    engine.apply_batch([prec] * 16, o64, ops, phis, abs_prec=True, precision="fp64")
    st = engine.apply_batch([prec] * 16, omx, ops, phis, abs_prec=True, precision="mixed")
    assert st["items_fp32"] + st["items_tf32"] > st["items_fp64"]
    for a, b in zip(omx, o64):
        ka, ca, _ = a.download()
        kb, cb, _ = b.download()
        assert np.array_equal(ka, kb)
        assert rel_l2(ca, cb) <= prec


def test_config4_exchange_pairs(engine, oracle):
    prec, order = 1e-5, 7
    rng = np.random.default_rng(SEED)
    terms = poly_orbitals(rng, 32, 0.5, 10.0)
    mra = engine.MultiResolutionAnalysis(order)
    phis = []
    for t in terms:
        f = engine.project(prec, engine.FunctionTree(mra), t, abs_prec=True)
        f.rescale(1.0 / f.norm())
        phis.append(f)
    pairs = [(i, j) for i in range(32) for j in range(i, 32)]
    assert len(pairs) == 528
    # exchange precision split, src/qmoperators/two_electron/ExchangePotential.cpp:166-168
    prec_m1, prec_p = prec / 10, prec * 10
    rhos = [engine.FunctionTree(mra) for _ in pairs]
    engine.multiply_batch(prec_m1, rhos, 1.0, [phis[i] for i, _ in pairs], [phis[j] for _, j in pairs],
                          abs_prec=True, use_max_norms=True)
    P = engine.PoissonOperator(mra, prec)
    pt = [[phis[i], phis[j]] if i != j else [phis[i]] for i, j in pairs]
    v64 = [engine.FunctionTree(mra) for _ in pairs]
    vmx = [engine.FunctionTree(mra) for _ in pairs]
    engine.apply_batch(prec_p, v64, [P] * 528, rhos, prec_trees=pt, abs_prec=True, precision="fp64")
    st = engine.apply_batch(prec_p, vmx, [P] * 528, rhos, prec_trees=pt, abs_prec=True, precision="mixed")
    assert st["out_nodes"] > 528 * 8
    # The applies run at absolute precision: the tiering bounds each item's error against the
    # absolute screening threshold, so the difference to FP64 is bounded by prec_p in absolute
    # terms, and relative to the output where the output's norm exceeds 1.  Pairs of distant
    # orbitals have outputs of norm << 1, where a relative bound would be stricter than the call's.
    worst = 0.0
    for a, b in zip(vmx, v64):
        ka, ca, _ = a.download()
        kb, cb, _ = b.download()
        assert np.array_equal(ka, kb)
        err = float(np.linalg.norm(ca - cb))
        worst = max(worst, err / max(float(np.linalg.norm(cb)), 1.0))
    assert worst <= prec_p, worst
    # one pair against the oracle, from the same input trees
    omra = oracle.MRA(order)
    i, j = pairs[37]
    oa = oracle.Tree.from_arrays(omra, *phis[i].download()[:2])
    ob = oracle.Tree.from_arrays(omra, *phis[j].download()[:2])
    orho = oracle.Tree(omra)
    oracle.multiply(prec_m1, orho, 1.0, oa, ob, -1, True, True)
    k1, c1, _ = rhos[37].download()
    k2, c2, _ = orho.export()
    assert np.array_equal(k1, k2) and rel_l2(c1, c2) <= 1e-10
    oV = oracle.Tree(omra)
    oracle.apply(prec_p, oV, oracle.poisson(omra, prec), orho, abs_prec=True, prec_trees=[oa, ob])
    k1, c1, _ = v64[37].download()
    k2, c2, _ = oV.export()
    assert np.array_equal(k1, k2) and rel_l2(c1, c2) <= 1e-10


def test_linearity_and_rerun(engine):
    prec = 1e-6
    mra = engine.MultiResolutionAnalysis(7)
    f = engine.project(prec, engine.FunctionTree(mra), [(1.0, 2.0, (0.2, 0.0, -0.3), (1, 1, 0))], abs_prec=True)
    g = engine.FunctionTree(mra)
    engine.add(prec, g, [(2.0, f)])
    H = engine.HelmholtzOperator(mra, 1.1, prec)
    a, b, c = (engine.FunctionTree(mra) for _ in range(3))
    # relative precision: thresholds scale with the output norm, so 2f takes the same decisions as f
    engine.apply(prec, a, H, f)
    engine.apply(prec, b, H, g)
    engine.apply(prec, c, H, f)
    ka, ca, _ = a.download()
    kb, cb, _ = b.download()
    kc, cc, _ = c.download()
    assert np.array_equal(ka, kc) and np.array_equal(ca, cc)  # bit-identical rerun
    assert np.array_equal(ka, kb)
    assert rel_l2(cb, 2 * ca) <= 1e-13
