"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle on the same inputs.

Bars: integer structure (node keys, leaf flags) bit-exact; FP64 coefficients to
relative L2 <= 1e-10 (different summation orders only); mixed precision to
relative L2 <= prec against the FP64 path.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAUSS4 = [(1.0, 1.5, (0.3, -0.2, 0.1), (0, 0, 0)),
          (0.7, 4.0, (-0.5, 0.4, 0.2), (1, 0, 0)),
          (0.3, 0.8, (0.1, 0.2, -0.6), (0, 1, 1)),
          (0.5, 9.0, (0.0, 0.0, 0.0), (0, 0, 0))]


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def to_oracle(po, omra, tree):
    keys, coefs, _ = tree.download()
    return po.Tree.from_arrays(omra, keys, coefs)


def to_engine(mw, mra, otree):
    keys, coefs, _ = otree.export()
    return mw.FunctionTree(mra).upload(keys, coefs)


def same_tree(tree, otree, tol):
    k1, c1, l1 = tree.download()
    k2, c2, l2 = otree.export()
    assert k1.shape == k2.shape, (k1.shape, k2.shape)
    assert np.array_equal(k1, k2)
    assert np.array_equal(l1, l2)
    err = rel_l2(c1, c2)
    assert err <= tol, err
    return err


@pytest.fixture(scope="module")
def k5(engine, oracle):
    return engine.MultiResolutionAnalysis(5), oracle.MRA(5)


@pytest.fixture(scope="module")
def k7(engine, oracle):
    return engine.MultiResolutionAnalysis(7), oracle.MRA(7)


@pytest.mark.parametrize("order,basis", [(5, "interpolating"), (7, "legendre"), (9, "interpolating")])
def test_basis_matches_oracle(engine, oracle, order, basis):
    a = engine.MultiResolutionAnalysis(order, basis=basis).basis_data()
    b = oracle.MRA(order, basis=basis).basis_data()
    for key in ("qx", "qw", "W", "c2v", "v2c"):
        assert np.abs(a[key] - b[key]).max() < 1e-13, key
    W = a["W"]
    assert np.abs(W @ W.T - np.eye(W.shape[0])).max() < 1e-13


def test_poisson_operator_matches_oracle(engine, oracle, k7):
    mra, omra = k7
    P = engine.PoissonOperator(mra, 1e-5)
    Q = oracle.poisson(omra, 1e-5)
    c1, a1 = P.terms()
    c2, a2 = Q.terms()
    assert c1.shape == c2.shape
    assert np.allclose(c1, c2, rtol=1e-13, atol=0) and np.allclose(a1, a2, rtol=1e-13, atol=0)
    for t in range(0, P.nterms, 7):
        for n in (-5, -2, 0, 3, 6):
            L = P.band(t, n)
            assert L == Q.band(t, n)
            if L < 0:
                continue
            # tolerance relative to the (term, scale)'s largest block, NS(0): the blocks at the band
            # edge are many orders smaller and come out of cancellation in the Gaussian moments,
            # so their last digits depend on the order of the quadrature sums
            scale = max(np.abs(Q.block(t, n, 0)[0]).max(), 1e-300)
            for l in {-L, 0, L}:
                b1, n1 = P.block(t, n, l)
                b2, n2 = Q.block(t, n, l)
                assert np.abs(b1 - b2).max() <= 1e-12 * scale
                assert np.allclose(n1, n2, rtol=1e-12, atol=1e-12 * scale)


def test_helmholtz_batch_operators_identical(engine, k7):
    # operators built together are the operators built one by one, bit for bit
    mra, _ = k7
    mus = [0.5, 1.1, 1.9]
    one = [engine.HelmholtzOperator(mra, m, 1e-5) for m in mus]
    many = engine.HelmholtzOperator.batch(mra, mus, 1e-5)
    for p, q in zip(one, many):
        c1, a1 = p.terms()
        c2, a2 = q.terms()
        assert np.array_equal(c1, c2) and np.array_equal(a1, a2)
        for t in range(0, p.nterms, 5):
            for n in (-5, -1, 2, 6):
                L = p.band(t, n)
                assert L == q.band(t, n)
                for l in {-L, 0, L} if L >= 0 else ():
                    b1, n1 = p.block(t, n, l)
                    b2, n2 = q.block(t, n, l)
                    assert np.array_equal(b1, b2) and np.array_equal(n1, n2)


def test_projection_matches_oracle(engine, oracle, k7):
    mra, omra = k7
    t = engine.project(1e-6, engine.FunctionTree(mra), GAUSS4)
    o = oracle.project_gauss(1e-6, oracle.Tree(omra), GAUSS4)
    same_tree(t, o, 1e-12)
    assert abs(t.integrate() - o.integrate()) < 1e-12 * abs(o.integrate())


def test_hydrogen_projection_matches_oracle(engine, oracle, k5):
    mra, omra = k5
    t = engine.project_hydrogen(1e-4, engine.FunctionTree(mra), 2, 1, 2)
    o = oracle.project_hydrogen(1e-4, oracle.Tree(omra), 2, 1, 2)
    same_tree(t, o, 1e-11)


@pytest.mark.parametrize("prec,order", [(1e-4, 5), (1e-5, 7)])
def test_poisson_apply_matches_oracle(engine, oracle, prec, order):
    mra, omra = engine.MultiResolutionAnalysis(order), oracle.MRA(order)
    orho = oracle.project_gauss(prec, oracle.Tree(omra), GAUSS4)
    rho = to_engine(engine, mra, orho)
    P, Q = engine.PoissonOperator(mra, prec), oracle.poisson(omra, prec)
    V = engine.FunctionTree(mra)
    st = engine.apply(prec, V, P, rho)
    oV = oracle.Tree(omra)
    ost = oracle.apply(prec, oV, Q, orho)
    same_tree(V, oV, 1e-10)
    assert st["out_nodes"] == ost["out_nodes"]
    assert st["items"] == ost["items"]


def test_helmholtz_apply_abs_matches_oracle(engine, oracle, k7):
    mra, omra = k7
    prec, mu = 1e-5, 1.2
    ophi = oracle.project_gauss(prec, oracle.Tree(omra), GAUSS4, abs_prec=True)
    phi = to_engine(engine, mra, ophi)
    H, Q = engine.HelmholtzOperator(mra, mu, prec), oracle.helmholtz(omra, mu, prec)
    out, oout = engine.FunctionTree(mra), oracle.Tree(omra)
    engine.apply(prec, out, H, phi, abs_prec=True)
    oracle.apply(prec, oout, Q, ophi, abs_prec=True)
    same_tree(out, oout, 1e-10)


def test_apply_with_precision_trees_matches_oracle(engine, oracle, k5):
    mra, omra = k5
    prec = 1e-4
    oa = oracle.project_hydrogen(prec, oracle.Tree(omra), 1, 0, 0)
    ob = oracle.project_hydrogen(prec, oracle.Tree(omra), 2, 0, 0)
    orho = oracle.Tree(omra)
    oracle.multiply(prec / 10, orho, 1.0, oa, ob, -1, True, True)
    a, b, rho = (to_engine(engine, mra, x) for x in (oa, ob, orho))
    P, Q = engine.PoissonOperator(mra, prec), oracle.poisson(omra, prec)
    V, oV = engine.FunctionTree(mra), oracle.Tree(omra)
    engine.apply(prec * 10, V, P, rho, prec_trees=[a, b], abs_prec=True)
    oracle.apply(prec * 10, oV, Q, orho, abs_prec=True, prec_trees=[oa, ob])
    same_tree(V, oV, 1e-10)


def test_erf_potential(engine, k7):
    """Poisson apply of normalized Gaussians against the analytic erf potential."""
    mra, _ = k7
    prec = 1e-6
    rng = np.random.default_rng(20261203)
    alphas = np.exp(rng.uniform(np.log(0.5), np.log(50.0), 4))
    centres = rng.uniform(-2, 2, (4, 3))
    terms = [((a / math.pi) ** 1.5, a, tuple(c), (0, 0, 0)) for a, c in zip(alphas, centres)]
    rho = engine.project(prec, engine.FunctionTree(mra), terms)
    assert abs(rho.integrate() - 4.0) < 1e-8
    V = engine.FunctionTree(mra)
    engine.apply(prec, V, engine.PoissonOperator(mra, prec), rho)
    pts = rng.uniform(-3, 3, (200, 3))
    from math import erf
    exact = np.array([sum(erf(math.sqrt(a) * np.linalg.norm(p - c)) / np.linalg.norm(p - c)
                          for a, c in zip(alphas, centres)) for p in pts])
    got = V.evalf(pts)
    assert np.abs(got - exact).max() <= 10 * prec * np.abs(exact).max()


def test_mixed_precision_close_to_fp64(engine, k7):
    mra, _ = k7
    prec = 1e-6
    rho = engine.project(prec, engine.FunctionTree(mra), GAUSS4)
    P = engine.PoissonOperator(mra, prec)
    v64, vmx = engine.FunctionTree(mra), engine.FunctionTree(mra)
    engine.apply(prec, v64, P, rho, precision="fp64")
    st = engine.apply(prec, vmx, P, rho, precision="mixed")
    assert st["items_fp32"] + st["items_tf32"] > 0
    k1, c1, _ = v64.download()
    k2, c2, _ = vmx.download()
    assert np.array_equal(k1, k2)
    assert rel_l2(c2, c1) <= prec


def test_apply_deterministic_and_batch_equal(engine, k5):
    mra, _ = k5
    prec = 1e-4
    phis = [engine.project(prec, engine.FunctionTree(mra), [(1.0, a, (0.1 * i, 0, 0), (i % 2, 0, 0))], abs_prec=True)
            for i, a in enumerate((0.7, 2.0, 5.0))]
    ops = [engine.HelmholtzOperator(mra, mu, prec) for mu in (0.5, 1.0, 1.7)]
    single = []
    for phi, op in zip(phis, ops):
        out = engine.FunctionTree(mra)
        engine.apply(prec, out, op, phi, abs_prec=True)
        single.append(out.download())
    outs = [engine.FunctionTree(mra) for _ in phis]
    engine.apply_batch([prec] * 3, outs, ops, phis, abs_prec=True)
    for (k1, c1, l1), out in zip(single, outs):
        k2, c2, l2 = out.download()
        assert np.array_equal(k1, k2) and np.array_equal(c1, c2)


def test_multiply_matches_oracle(engine, oracle, k7):
    mra, omra = k7
    prec = 1e-6
    oa = oracle.project_gauss(prec, oracle.Tree(omra), GAUSS4[:2])
    ob = oracle.project_gauss(prec, oracle.Tree(omra), GAUSS4[2:])
    a, b = to_engine(engine, mra, oa), to_engine(engine, mra, ob)
    for use_max in (False, True):
        out, oout = engine.FunctionTree(mra), oracle.Tree(omra)
        engine.multiply(prec, out, 0.5, a, b, use_max_norms=use_max)
        oracle.multiply(prec, oout, 0.5, oa, ob, -1, False, use_max)
        same_tree(out, oout, 1e-11)


def test_batched_multiply_equals_single_products(engine, k7):
    # a batch whose trees feed several products maps their nodes to values once and shares the
    # generation of missing nodes; every product must come out bit-identical to a single multiply
    mra, _ = k7
    prec = 1e-6
    fs = [engine.project(prec, engine.FunctionTree(mra), [g], abs_prec=True) for g in GAUSS4[:3]]
    pairs = [(0, 0), (0, 1), (1, 2), (2, 0), (2, 2)]
    for use_max in (False, True):
        outs = [engine.FunctionTree(mra) for _ in pairs]
        engine.multiply_batch(prec, outs, 1.3, [fs[i] for i, _ in pairs], [fs[j] for _, j in pairs], abs_prec=True,
                              use_max_norms=use_max)
        for (i, j), o in zip(pairs, outs):
            ref = engine.FunctionTree(mra)
            engine.multiply(prec, ref, 1.3, fs[i], fs[j], abs_prec=True, use_max_norms=use_max)
            k1, c1, l1 = o.download()
            k2, c2, l2 = ref.download()
            assert np.array_equal(k1, k2) and np.array_equal(l1, l2) and np.array_equal(c1, c2), (i, j, use_max)


def test_square_fixed_grid_and_integral_identity(engine, k7):
    """int f*f = |f|^2 (tests/qmfunctions/qmfunction.cpp:258-259), on the copied grid."""
    mra, _ = k7
    f = engine.project(1e-6, engine.FunctionTree(mra), GAUSS4)
    g = engine.FunctionTree(mra)
    engine.copy_grid(g, f)
    engine.square(1e-6, g, f)
    assert abs(g.integrate() - f.squared_norm()) < 1e-9 * f.squared_norm()


def test_add_matches_oracle(engine, oracle, k7):
    mra, omra = k7
    prec = 1e-6
    oa = oracle.project_gauss(prec, oracle.Tree(omra), GAUSS4[:2])
    ob = oracle.project_gauss(prec, oracle.Tree(omra), GAUSS4[2:])
    a, b = to_engine(engine, mra, oa), to_engine(engine, mra, ob)
    out, oout = engine.FunctionTree(mra), oracle.Tree(omra)
    engine.add(prec, out, [(2.0, a), (-0.5, b)])
    oracle.add(prec, oout, [2.0, -0.5], [oa, ob])
    same_tree(out, oout, 1e-13)


def test_dot_and_crop(engine, oracle, k7):
    mra, omra = k7
    oa = oracle.project_gauss(1e-7, oracle.Tree(omra), GAUSS4)
    a = to_engine(engine, mra, oa)
    assert abs(engine.dot(a, a) - oracle.dot(oa, oa)) < 1e-12 * oracle.dot(oa, oa)
    a.crop(1e-4)
    oa.crop(1e-4)
    same_tree(a, oa, 1e-14)
