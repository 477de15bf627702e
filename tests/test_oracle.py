"""CPU oracle pinned against the reference's own test values and analytic results (no GPU)."""
import json
import math
import os

import numpy as np
import pytest

GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_values.json")))


def test_filters_orthogonal(oracle):
    for order in (5, 7, 9):
        for basis in ("interpolating", "legendre"):
            W = oracle.MRA(order, basis=basis).basis_data()["W"]
            assert np.abs(W @ W.T - np.eye(W.shape[0])).max() < 1e-13


def test_projection_integral_and_pointwise(oracle):
    mra = oracle.MRA(7)
    a = 3.0
    t = oracle.project_gauss(1e-6, oracle.Tree(mra), [((a / math.pi) ** 1.5, a, (0.1, -0.2, 0.3), (0, 0, 0))])
    assert abs(t.integrate() - 1.0) < 1e-10
    assert abs(t.sqnorm() - (a / (2 * math.pi)) ** 1.5) < 1e-9
    r = np.array([0.15, -0.1, 0.25])
    d = r - np.array([0.1, -0.2, 0.3])
    assert abs(t.eval(r) - (a / math.pi) ** 1.5 * math.exp(-a * d @ d)) < 1e-5


def test_export_import_roundtrip(oracle):
    mra = oracle.MRA(5)
    t = oracle.project_gauss(1e-4, oracle.Tree(mra), [(1.0, 2.0, (0.0, 0.0, 0.0), (1, 0, 0))])
    k, c, l = t.export()
    perm = np.random.default_rng(0).permutation(len(k))
    t2 = oracle.Tree.from_arrays(mra, k[perm], c[perm])
    k2, c2, l2 = t2.export()
    assert np.array_equal(k, k2) and np.array_equal(c, c2) and np.array_equal(l, l2)


@pytest.mark.parametrize("kind", ["poisson", "helmholtz"])
def test_kernel_expansion_accuracy(oracle, kind):
    mra = oracle.MRA(5)
    prec, mu = 1e-6, 1.3
    op = oracle.poisson(mra, prec) if kind == "poisson" else oracle.helmholtz(mra, mu, prec)
    for r in np.logspace(-5, 2, 60):
        exact = 1.0 / r if kind == "poisson" else math.exp(-mu * r) / r
        assert abs(op.kernel(r) - exact) * r <= 0.1 * prec


def test_operator_blocks_symmetry(oracle):
    mra = oracle.MRA(5)
    P = oracle.poisson(mra, 1e-4)
    for t in range(0, P.nterms, 11):
        for n in (-5, -3, 0, 2):
            L = P.band(t, n)
            for l in range(0, L + 1):
                b1, _ = P.block(t, n, l)
                b2, _ = P.block(t, n, -l)
                assert np.abs(b1 - b2.T).max() <= 1e-15 * max(np.abs(b1).max(), 1e-300)


def test_poisson_erf_potential(oracle):
    mra = oracle.MRA(5)
    prec, a = 1e-4, 2.0
    rho = oracle.project_gauss(prec, oracle.Tree(mra), [((a / math.pi) ** 1.5, a, (0.0, 0.0, 0.0), (0, 0, 0))])
    V = oracle.Tree(mra)
    oracle.apply(prec, V, oracle.poisson(mra, prec), rho)
    rng = np.random.default_rng(1)
    err = max(abs(V.eval(r) - math.erf(math.sqrt(a) * np.linalg.norm(r)) / np.linalg.norm(r))
              for r in rng.uniform(-3, 3, (100, 3)))
    assert err < 10 * prec
    assert abs(oracle.dot(rho, V) - math.sqrt(2 * a / math.pi)) < 5 * prec


def test_helmholtz_gaussian_closed_form(oracle):
    from scipy.special import erfc
    mra = oracle.MRA(5)
    prec, mu, a = 1e-4, 1.3, 2.0
    g = oracle.project_gauss(prec, oracle.Tree(mra), [((a / math.pi) ** 1.5, a, (0.0, 0.0, 0.0), (0, 0, 0))],
                             abs_prec=True)
    V = oracle.Tree(mra)
    oracle.apply(prec, V, oracle.helmholtz(mra, mu, prec), g, abs_prec=True)
    sa = math.sqrt(a)
    for r in np.random.default_rng(2).uniform(-2, 2, (50, 3)):
        d = np.linalg.norm(r)
        ex = math.exp(mu ** 2 / (4 * a)) / (2 * d) * (math.exp(-mu * d) * erfc(mu / (2 * sa) - sa * d)
                                                       - math.exp(mu * d) * erfc(mu / (2 * sa) + sa * d))
        assert abs(V.eval(r) - ex) < 10 * prec


def test_multiply_identity_and_add(oracle):
    """int f*f = |f|^2 (tests/qmfunctions/qmfunction.cpp:258-259) and linearity of add."""
    mra = oracle.MRA(7)
    f = oracle.project_gauss(1e-6, oracle.Tree(mra), [(1.0, 1.0, (0.3, 0, 0), (1, 0, 0)),
                                                        (0.5, 3.0, (-0.5, 0.2, 0), (0, 0, 0))])
    g = oracle.Tree(mra)
    oracle.multiply(1e-6, g, 1.0, f, f, -1, False, True)
    assert abs(g.integrate() - f.sqnorm()) < 1e-10
    h = oracle.Tree(mra)
    oracle.add(1e-6, h, [2.0, -1.0], [f, g])
    assert abs(h.integrate() - (2 * f.integrate() - g.integrate())) < 1e-12


def _hydrogen_coulomb(oracle, prec, order):
    mra = oracle.MRA(order)
    ref = GOLDEN["coulomb"]
    phis = [oracle.project_hydrogen(prec, oracle.Tree(mra), *o) for o in ref["orbitals"]]
    rhos = []
    for p in phis:
        r = oracle.Tree(mra)
        oracle.copy_grid(r, p)
        oracle.multiply(prec, r, 1.0, p, p)
        rhos.append(r)
    rho = oracle.Tree(mra)
    oracle.add(prec, rho, [ref["occupation"]] * len(phis), rhos)
    J = oracle.Tree(mra)
    oracle.apply(prec / rho.norm(), J, oracle.poisson(mra, prec), rho)
    out, jphis = [], []
    for p in phis:
        jp = oracle.Tree(mra)
        oracle.copy_grid(jp, p)
        oracle.multiply(prec, jp, 1.0, J, p)
        out.append(oracle.dot(p, jp))
        jphis.append(jp)
    # off-diagonal element <phi_0|J|phi_1>
    out01 = oracle.dot(phis[0], jphis[1])
    return rho, out, out01


def test_reference_coulomb_values(oracle):
    """<phi_i|J|phi_i> of tests/qmoperators/coulomb_operator.cpp:78-84 (k=5, prec 1e-3).

    The reference pins MRCPP's own discretisation to 1e-8; this restatement
    reproduces the values to a few 1e-6 relative.
    """
    rho, vals, v01 = _hydrogen_coulomb(oracle, GOLDEN["coulomb"]["prec"], GOLDEN["mra"]["order"])
    assert abs(rho.integrate() - 10.0) < 1e-4
    E = GOLDEN["coulomb"]["E_P"]
    for i, v in enumerate(vals):
        assert abs(v - E["%d,%d" % (i, i)]) < 1e-5 * E["%d,%d" % (i, i)], (i, v)
    # the off-diagonal pin E_P(0,1) (1s / 2s): measured 5e-6 relative
    assert abs(v01 - E["0,1"]) < 2e-5 * E["0,1"], v01


def _exchange_kij(oracle, mra, P, phis, precf, k, i, j):
    """calcExchange_kij (src/qmoperators/two_electron/ExchangePotential.cpp:161-234) for real orbitals:
    rho_ij = phi_i phi_j at precf/10, V_ij = P[rho_ij] at precf*10 steered by phi_k, phi_j, phi_i,
    then phi_k V_ij and phi_j V_ij at precf/100; absolute precision, max-norm estimates."""
    rho = oracle.Tree(mra)
    oracle.multiply(precf / 10, rho, 1.0, phis[i], phis[j], -1, True, True)
    if rho.norm() < precf:
        return None, None
    steer = [phis[k]] + ([phis[j]] if j != k else []) + ([phis[i]] if i not in (k, j) else [])
    V = oracle.Tree(mra)
    oracle.apply(precf * 10, V, P, rho, -1, True, steer)
    out_kij, out_jji = oracle.Tree(mra), oracle.Tree(mra)
    oracle.multiply(precf / 100, out_kij, 1.0, phis[k], V, -1, True, True)
    oracle.multiply(precf / 100, out_jji, 1.0, phis[j], V, -1, True, True)
    return out_kij, out_jji


def test_reference_exchange_values(oracle):
    """<phi_i|K|phi_j> of tests/qmoperators/exchange_operator.cpp:75-78 (H 1s, 2s; k=5, prec 1e-3).

    K is built as ExchangePotentialD1::setupInternal does (ExchangePotentialD1.cpp:142-300, no
    bank): precf = prec / sqrt(N); K phi_i = phi_i P[phi_i phi_i] + sum_{j != i} (pair terms of
    calcExchange_kij).  The reference's own value is 3.4% away from the continuum (0.6469 for
    (0,0)), a discretisation effect at this precision that the restatement reproduces: (0,0) to
    1.4e-4 relative, the other elements within 1.2 prec absolute.
    """
    ref = GOLDEN["exchange"]
    prec = ref["prec"]
    mra = oracle.MRA(GOLDEN["mra"]["order"])
    phis = [oracle.project_hydrogen(prec, oracle.Tree(mra), *o) for o in ref["orbitals"]]
    P = oracle.poisson(mra, prec)
    precf = prec / math.sqrt(len(phis))
    ex00, _ = _exchange_kij(oracle, mra, P, phis, precf, 0, 0, 0)
    ex11, _ = _exchange_kij(oracle, mra, P, phis, precf, 1, 1, 1)
    ex_110, ex_001 = _exchange_kij(oracle, mra, P, phis, precf, 1, 1, 0)  # pair (i=1, j=0)
    K0 = [ex00, ex_110]  # contributions to K phi_0
    K1 = [ex11, ex_001]  # contributions to K phi_1
    E = {"0,0": sum(oracle.dot(phis[0], t) for t in K0), "1,1": sum(oracle.dot(phis[1], t) for t in K1),
         "0,1": sum(oracle.dot(phis[0], t) for t in K1), "1,0": sum(oracle.dot(phis[1], t) for t in K0)}
    assert abs(E["0,0"] - ref["E_P"]["0,0"]) < 3e-4 * ref["E_P"]["0,0"], E
    for key in ("0,1", "1,0", "1,1"):
        assert abs(E[key] - ref["E_P"][key]) < 2 * prec, (key, E[key])
    assert abs(E["0,1"] - E["1,0"]) < 1e-10  # K is symmetric


def test_density_integrals(oracle):
    """int rho = 7 / 3 / 5 / 2 (tests/qmfunctions/density.cpp:68-69,79-80): 5 alpha + 2 beta orbitals."""
    prec = GOLDEN["density"]["prec"]
    mra = oracle.MRA(5)
    alpha = [(1, 0, 0), (2, 0, 0), (2, 1, 0), (2, 1, 1), (2, 1, 2)]
    beta = [(1, 0, 0), (1, 0, 0)]

    def dens(orbs):
        sq = []
        for o in orbs:
            p = oracle.project_hydrogen(prec, oracle.Tree(mra), *o)
            r = oracle.Tree(mra)
            oracle.copy_grid(r, p)
            oracle.multiply(prec, r, 1.0, p, p)
            sq.append(r)
        rho = oracle.Tree(mra)
        oracle.add(prec, rho, [1.0] * len(sq), sq)
        return rho.integrate()

    na, nb = dens(alpha), dens(beta)
    d = GOLDEN["density"]
    assert abs(na - d["alpha"]) < 1e-3 and abs(nb - d["beta"]) < 1e-3
    assert abs(na + nb - d["total"]) < 2e-3 and abs(na - nb - d["spin"]) < 2e-3
