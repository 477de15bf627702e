"""Adjoint apply and the Coulomb-energy gradient (6-Gaussian density, k=9, prec 1e-6, FP64).

- dot-product test: <y, A x> = <A^T y, x> for the fixed-grid apply A (same item set);
- dJ/drho for J = 1/2 <rho, P rho> equals the forward potential V (symmetric kernel);
- dJ/dR (Gaussian centre, through torch.autograd and the adjoint) against central finite
  differences with h = 1e-4 on the same fixed grid;
- adjoint multiply: <s, a b> = <M_b^T s, a> for the fixed-grid product on a grid finer than a's
  in some boxes and coarser in others; the gradient of J(phi) = 1/2 <rho, P rho> with
  rho = 2 phi^2 (torch.autograd through the adjoint multiply and the adjoint apply) against
  central finite differences along a direction on phi's grid.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
SEED, PREC, ORDER = 20261203, 1e-6, 9


def six_gaussians():
    rng = np.random.default_rng(SEED + 5)
    alphas = np.exp(rng.uniform(np.log(1.0), np.log(30.0), 6))
    centres = rng.uniform(-2, 2, (6, 3))
    return alphas, centres


def density_terms(alphas, centres):
    return [((a / math.pi) ** 1.5, a, tuple(c), (0, 0, 0)) for a, c in zip(alphas, centres)]


@pytest.fixture(scope="module")
def setup(engine):
    mra = engine.MultiResolutionAnalysis(ORDER)
    alphas, centres = six_gaussians()
    rho = engine.project(PREC, engine.FunctionTree(mra), density_terms(alphas, centres), abs_prec=True)
    P = engine.PoissonOperator(mra, PREC)
    return mra, alphas, centres, rho, P


def on_grid(engine, mra, grid_tree, terms, prec=1e-10):
    """Projection of an analytic function onto a fixed grid."""
    f = engine.project(prec, engine.FunctionTree(mra), terms, abs_prec=True)
    out = engine.FunctionTree(mra)
    engine.copy_grid(out, grid_tree)
    engine.copy_func(out, f)
    return out


def fixed_apply(engine, mra, P, x):
    V = engine.FunctionTree(mra)
    engine.copy_grid(V, x)
    engine.apply_fixed(PREC, V, P, x, abs_prec=True)
    return V


def test_adjoint_dot_product(engine, setup):
    mra, alphas, centres, rho, P = setup
    y = on_grid(engine, mra, rho, [(1.0, 0.7, (0.5, -0.3, 0.2), (1, 0, 0)), (0.4, 3.0, (-1.0, 0.5, 0.0), (0, 0, 0))])
    Ax = fixed_apply(engine, mra, P, rho)
    lhs = engine.dot(y, Ax)
    ATy = engine.FunctionTree(mra)
    st = engine.apply_adjoint(PREC, ATy, P, rho, y)
    assert st["items"] > 0
    rhs = engine.dot(ATy, rho)
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1e-300), (lhs, rhs)


def test_gradient_equals_potential(engine, setup):
    torch = pytest.importorskip("torch")
    from mrchem_gb300.autograd import FixedGrid, coulomb_energy
    mra, alphas, centres, rho, P = setup
    grid = FixedGrid(mra, rho.download()[0])
    x = torch.from_numpy(grid.to_vec(rho)).requires_grad_(True)
    J = coulomb_energy(x, grid, P, PREC)
    J.backward()
    V = fixed_apply(engine, mra, P, rho)
    v = grid.to_vec(V)
    # the adaptive NS-form apply is symmetric only up to its truncation (scale corrections are
    # kept on the output grid by A and on the input grid by A^T), so dJ/drho = (A + A^T) rho / 2
    # and V = A rho agree to the discretisation's accuracy, not to rounding
    err = np.linalg.norm(x.grad.numpy() - v) / np.linalg.norm(v)
    assert err <= 1e-4, err
    # as functions, both are the Coulomb potential of rho to the apply's precision
    pts = np.random.default_rng(3).uniform(-3, 3, (200, 3))
    exact = np.array([sum(math.erf(math.sqrt(a) * np.linalg.norm(p - c)) / np.linalg.norm(p - c)
                          for a, c in zip(alphas, centres)) for p in pts])
    gtree = grid.to_tree(x.grad.numpy())
    vmax = np.abs(exact).max()
    assert np.abs(V.evalf(pts) - exact).max() <= 10 * PREC * vmax
    assert np.abs(gtree.evalf(pts) - exact).max() <= 10 * PREC * vmax
    # J itself against the analytic Coulomb energy of the Gaussians (pairs: erf(sqrt(ab/(a+b)) d)/d)
    ex = 0.0
    for a, ca in zip(alphas, centres):
        for b, cb in zip(alphas, centres):
            d = np.linalg.norm(ca - cb)
            g = math.sqrt(a * b / (a + b))
            ex += 2 * g / math.sqrt(math.pi) if d < 1e-12 else math.erf(g * d) / d
    assert abs(float(J.detach()) - 0.5 * ex) <= 20 * PREC * abs(0.5 * ex)


def test_centre_gradient_vs_finite_differences(engine, setup):
    torch = pytest.importorskip("torch")
    from mrchem_gb300.autograd import FixedGrid, coulomb_energy
    mra, alphas, centres, rho, P = setup
    grid = FixedGrid(mra, rho.download()[0])
    a0, R0 = alphas[0], centres[0]
    N = (a0 / math.pi) ** 1.5
    # drho/dR0_d projected on the grid: N 2 a (r_d - R_d) exp(-a |r - R|^2)
    cols = []
    for d in range(3):
        pw = [0, 0, 0]
        pw[d] = 1
        cols.append(grid.to_vec(on_grid(engine, mra, rho, [(N * 2 * a0, a0, tuple(R0), tuple(pw))])))
    dxdR = torch.from_numpy(np.stack(cols, axis=1))
    x0 = torch.from_numpy(grid.to_vec(rho))
    R = torch.zeros(3, dtype=torch.float64, requires_grad=True)
    J = coulomb_energy(x0 + dxdR @ R, grid, P, PREC)
    J.backward()
    h = 1e-4
    fd = []
    for d in range(3):
        vals = []
        for sgn in (1, -1):
            c = centres.copy()
            c[0, d] += sgn * h
            r = on_grid(engine, mra, rho, density_terms(alphas, c))
            vals.append(0.5 * engine.dot(r, fixed_apply(engine, mra, P, r)))
        fd.append((vals[0] - vals[1]) / (2 * h))
    fd = np.array(fd)
    g = R.grad.numpy()
    assert np.abs(g - fd).max() <= 1e-3 * max(np.abs(fd).max(), 1e-3), (g, fd)


def test_multiply_adjoint_dot_product(engine, setup):
    mra, alphas, centres, rho, P = setup
    prec = 1e-7
    a = engine.project(prec, engine.FunctionTree(mra), [(1.0, 2.0, (0.3, -0.2, 0.1), (1, 0, 0))], abs_prec=True)
    b = engine.project(prec, engine.FunctionTree(mra), [(0.8, 5.0, (-0.4, 0.2, 0.3), (0, 0, 0))], abs_prec=True)
    # the product's grid: rho's (finer than a's in some boxes, coarser in others)
    h = engine.FunctionTree(mra)
    engine.copy_grid(h, rho)
    engine.multiply(prec, h, 1.7, a, b, max_iter=0, abs_prec=True)
    s = on_grid(engine, mra, rho, [(1.0, 0.9, (0.2, 0.1, -0.5), (0, 1, 0)), (0.5, 6.0, (-0.3, 0.4, 0.2), (0, 0, 0))])
    out = engine.FunctionTree(mra)
    engine.multiply_adjoint(prec, out, 1.7, a, b, s)
    ka, _, _ = a.download()
    ko, _, _ = out.download()
    assert np.array_equal(ka, ko)  # on a's grid
    lhs, rhs = engine.dot(s, h), engine.dot(out, a)
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), 1e-300), (lhs, rhs)


def test_density_gradient_vs_finite_differences(engine, setup):
    torch = pytest.importorskip("torch")
    from mrchem_gb300.autograd import FixedGrid, coulomb_energy, orbital_density
    mra, alphas, centres, rho, P = setup
    prec = 1e-7
    phi = engine.project(prec, engine.FunctionTree(mra),
                         [(1.0, 1.5, (0.2, -0.1, 0.3), (0, 0, 0)), (0.6, 4.0, (-0.5, 0.4, -0.2), (0, 0, 1))],
                         abs_prec=True)
    grid = FixedGrid(mra, phi.download()[0])
    x = torch.from_numpy(grid.to_vec(phi)).requires_grad_(True)
    J = coulomb_energy(orbital_density(x, grid, 2.0, prec), grid, P, PREC)
    J.backward()
    # direction: a Gaussian-polynomial projected on phi's grid
    d = torch.from_numpy(grid.to_vec(on_grid(engine, mra, phi, [(1.0, 2.5, (0.1, 0.2, -0.2), (1, 1, 0))])))
    h = 1e-3
    vals = []
    for sgn in (1, -1):
        xs = (x.detach() + sgn * h * d).clone()
        vals.append(float(coulomb_energy(orbital_density(xs, grid, 2.0, prec), grid, P, PREC)))
    fd = (vals[0] - vals[1]) / (2 * h)
    an = float(x.grad @ d)
    # J is quartic in phi, so the central difference carries an h^2 term (about 1e-6 relative
    # here), and the screened apply's item set follows rho's norms (items near the threshold,
    # about prec relative, over 2h); an error in either adjoint would be of order one
    assert abs(an - fd) <= 1e-4 * abs(fd), (an, fd)
