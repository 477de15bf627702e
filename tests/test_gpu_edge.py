"""Edge cases of the GPU path against the oracle: zero input, functions at the world boundary,
non-cubic worlds and other root scales, the Legendre basis, maxIter = 0, relative precision in
mixed mode, and the error returns of the C ABI (no abort, no host fallback)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def parity(engine, oracle, mra, omra, terms, prec, kind="poisson", abs_prec=False, max_iter=-1, mu=1.0):
    orho = oracle.project_gauss(prec, oracle.Tree(omra), terms, abs_prec=abs_prec)
    k, c, _ = orho.export()
    rho = engine.FunctionTree(mra).upload(k, c)
    if kind == "poisson":
        op, oop = engine.PoissonOperator(mra, prec), oracle.poisson(omra, prec)
    else:
        op, oop = engine.HelmholtzOperator(mra, mu, prec), oracle.helmholtz(omra, mu, prec)
    out, oout = engine.FunctionTree(mra), oracle.Tree(omra)
    engine.apply(prec, out, op, rho, max_iter=max_iter, abs_prec=abs_prec)
    oracle.apply(prec, oout, oop, orho, max_iter=max_iter, abs_prec=abs_prec)
    k1, c1, l1 = out.download()
    k2, c2, l2 = oout.export()
    assert np.array_equal(k1, k2) and np.array_equal(l1, l2)
    if np.linalg.norm(c2) > 0:
        assert rel_l2(c1, c2) <= 1e-10
    else:
        assert np.abs(c1).max() == 0.0
    return out


def test_zero_function(engine, oracle):
    mra, omra = engine.MultiResolutionAnalysis(5), oracle.MRA(5)
    out = parity(engine, oracle, mra, omra, [(0.0, 1.0, (0.0, 0.0, 0.0), (0, 0, 0))], 1e-4, abs_prec=True)
    assert out.nnodes == 8 and out.squared_norm() == 0.0


def test_function_at_world_corner(engine, oracle):
    mra, omra = engine.MultiResolutionAnalysis(5), oracle.MRA(5)
    parity(engine, oracle, mra, omra, [(1.0, 2.0, (31.5, -31.2, 31.0), (0, 0, 0))], 1e-4)


@pytest.mark.parametrize("root,corner,boxes", [(-4, (0, -1, -2), (1, 2, 3)), (-3, (-1, -1, -1), (2, 2, 2))])
def test_other_worlds(engine, oracle, root, corner, boxes):
    mra = engine.MultiResolutionAnalysis(5, root_scale=root, corner=corner, boxes=boxes, max_depth=12)
    omra = oracle.MRA(5, root_scale=root, corner=corner, boxes=boxes, max_depth=12)
    parity(engine, oracle, mra, omra, [(1.0, 3.0, (0.5, 0.3, -0.2), (0, 1, 0))], 1e-4, kind="helmholtz",
           abs_prec=True, mu=0.8)


def test_legendre_basis(engine, oracle):
    mra, omra = engine.MultiResolutionAnalysis(6, basis="legendre"), oracle.MRA(6, basis="legendre")
    parity(engine, oracle, mra, omra, [(1.0, 1.5, (0.1, 0.2, 0.3), (0, 0, 0))], 1e-5)


def test_max_iter_zero(engine, oracle):
    mra, omra = engine.MultiResolutionAnalysis(5), oracle.MRA(5)
    out = parity(engine, oracle, mra, omra, [(1.0, 2.0, (0.0, 0.0, 0.0), (0, 0, 0))], 1e-4, max_iter=0)
    assert out.nnodes == 8


def test_mixed_relative_precision(engine):
    mra = engine.MultiResolutionAnalysis(7)
    prec = 1e-6
    rho = engine.project(prec, engine.FunctionTree(mra), [(1.0, 4.0, (0.3, 0.0, 0.0), (0, 0, 0)),
                                                           (0.5, 0.5, (-0.7, 0.2, 0.0), (1, 0, 0))])
    P = engine.PoissonOperator(mra, prec)
    a, b = engine.FunctionTree(mra), engine.FunctionTree(mra)
    engine.apply(prec, a, P, rho, precision="fp64")
    st = engine.apply(prec, b, P, rho, precision="mixed")
    assert st["items_fp32"] + st["items_tf32"] > 0
    k1, c1, _ = a.download()
    k2, c2, _ = b.download()
    assert np.array_equal(k1, k2) and rel_l2(c2, c1) <= prec


def test_error_returns(engine):
    mra = engine.MultiResolutionAnalysis(5)
    f = engine.project(1e-3, engine.FunctionTree(mra), [(1.0, 1.0, (0.0, 0.0, 0.0), (0, 0, 0))])
    P = engine.PoissonOperator(mra, 1e-3)
    with pytest.raises(engine.MWError) as e:  # output not empty (CoulombPotential.cpp:122-123)
        engine.apply(1e-3, f, P, f)
    assert e.value.code == 1  # aliasing is rejected before anything runs
    g = engine.FunctionTree(mra)
    engine.apply(1e-3, g, P, f)
    with pytest.raises(engine.MWError) as e:
        engine.apply(1e-3, g, P, f)
    assert e.value.code == 5 and "empty" in str(e.value)
    with pytest.raises(engine.MWError):
        engine.MultiResolutionAnalysis(10)  # K = 11 has no GPU kernel
    with pytest.raises(engine.MWError):
        engine.HelmholtzOperator(mra, -1.0, 1e-3)
    adj = engine.FunctionTree(mra)  # kept alive across the call: handles are owned by the caller
    with pytest.raises(engine.MWError):  # the adjoint needs absolute precision
        engine._check(engine._lib.mw_apply_adjoint(1e-3, adj.ptr, P.ptr, f.ptr, f.ptr, 0), mra.ptr)
    # the context stays usable after errors
    h = engine.FunctionTree(mra)
    engine.apply(1e-3, h, P, f)
    assert h.nnodes >= 8
