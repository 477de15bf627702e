"""The C++ boundary: tests/cpp/shim_check.cpp spells MRChem's call sites against
include/mrcpp_gb300.hpp, is compiled with g++ and linked against libmwgb300.so, and its results
are compared with the CPU oracle on the same Gaussians.

Covered: CoulombPotential::setupGlobalPotential (project, PoissonOperator, relative-precision
apply, dot), the per-operator precision mode, HelmholtzVector::apply(i, phi) on complex orbitals
and their conjugates (CoulombPotential.cpp:115-160, HelmholtzVector.cpp:141-159) and its batched
replacement, cplxfunc::multiply with conjugation (ExchangePotential.cpp:175),
cplxfunc::linear_combination with complex coefficients (KAIN.cpp:170,182), ComplexFunction
add / rescale / dagger and cplxfunc::dot.
"""
import json
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "shim_check.cpp")
PREC = 1e-5
PI = math.pi

RHO = [(((a / PI) ** 1.5), a, r, (0, 0, 0)) for a, r in
       zip((0.7, 2.0, 6.5, 21.0), ((0.3, -0.2, 0.1), (-0.6, 0.5, 0.0), (0.1, 0.9, -0.4), (-0.2, -0.7, 0.6)))]
PHI_RE = [(1.0, 1.2, (0.2, 0.0, -0.1), (0, 0, 0)), (0.3, 4.0, (-0.3, 0.2, 0.1), (1, 0, 0))]
PHI_IM = [(0.6, 2.5, (0.0, 0.3, 0.2), (0, 1, 0))]
CHI_RE = [(0.9, 0.8, (-0.1, -0.2, 0.3), (0, 0, 0))]
CHI_IM = [(0.5, 3.0, (0.4, 0.1, -0.2), (0, 0, 1))]


def compile_check(lib_path, out_dir):
    gxx = shutil.which("g++") or shutil.which("c++")
    if not gxx:
        pytest.skip("no C++ compiler")
    exe = os.path.join(out_dir, "shim_check")
    lib_dir = os.path.dirname(lib_path)
    cmd = [gxx, "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-L", lib_dir, "-lmwgb300", "-Wl,-rpath," + lib_dir, "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_and_links(engine, tmp_path):
    """No GPU needed: the header compiles warning-free and every shim call resolves in the library."""
    exe = compile_check(engine.LIB_PATH, str(tmp_path))
    assert os.path.exists(exe)


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.gpu
def test_shim_call_sites_match_oracle(engine, oracle, tmp_path):
    exe = compile_check(engine.LIB_PATH, str(tmp_path))
    r = subprocess.run([exe, str(tmp_path)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    res = json.loads(r.stdout.strip().splitlines()[-1])

    mra, omra = engine.MultiResolutionAnalysis(7), oracle.MRA(7)

    def load(name):
        t = engine.load_tree(engine.FunctionTree(mra), str(tmp_path / (name + ".mwt")))
        return t.download()

    def proj(terms):
        return oracle.project_gauss(PREC, oracle.Tree(omra), terms)

    def same(name, otree, tol):
        k1, c1, l1 = load(name)
        k2, c2, l2 = otree.export()
        assert k1.shape == k2.shape and np.array_equal(k1, k2), name
        assert np.array_equal(l1, l2), name
        e = rel_l2(c1, c2)
        assert e <= tol, (name, e)
        return e

    # CoulombPotential::setupGlobalPotential
    orho = proj(RHO)
    same("rho", orho, 1e-12)
    oV = oracle.Tree(omra)
    oracle.apply(PREC / 4.0, oV, oracle.poisson(omra, PREC), orho)
    same("V", oV, 1e-10)
    k1, c1, _ = load("Vm")
    k2, c2, _ = oV.export()
    assert np.array_equal(k1, k2) and rel_l2(c1, c2) <= PREC  # mixed-precision operator, same node set
    assert abs(res["E_coulomb"] - oracle.dot(orho, oV)) <= 1e-10 * abs(res["E_coulomb"])
    assert res["rejected_nonempty_output"]

    A, B, C, D = proj(PHI_RE), proj(PHI_IM), proj(CHI_RE), proj(CHI_IM)
    same("phi_re", A, 1e-12)
    same("phi_im", B, 1e-12)
    same("chi_re", C, 1e-12)
    same("chi_im", D, 1e-12)

    # HelmholtzVector::apply(i, phi): out = -H[re]/(2 pi) + i (-+) H[im]/(2 pi), mu = sqrt(-2 lambda)
    def helm(f, lam, scale):
        out = oracle.Tree(omra)
        oracle.apply(PREC, out, oracle.helmholtz(omra, math.sqrt(-2.0 * lam), PREC), f, abs_prec=True)
        out.rescale(scale)
        return out

    hA, hB = helm(A, -0.5, -1 / (2 * PI)), helm(B, -0.5, -1 / (2 * PI))
    hBc = helm(B, -0.5, 1 / (2 * PI))
    same("h0_re", hA, 1e-10)
    same("h0_im", hB, 1e-10)
    same("h1_re", hA, 1e-10)
    same("h1_im", hBc, 1e-10)  # phi^dagger: the imaginary part's sign flips
    same("hv0_re", hA, 1e-10)
    same("hv0_im", hB, 1e-10)
    same("hv1_im", hBc, 1e-10)
    same("hv2_re", helm(C, -1.2, -1 / (2 * PI)), 1e-10)
    same("hv2_im", helm(D, -1.2, -1 / (2 * PI)), 1e-10)

    # rho_ij = phi^dagger chi: real = A C + B D, imag = A D - B C, each product adaptive, then summed
    def prod(x, y, coef):
        out = oracle.Tree(omra)
        oracle.multiply(PREC / 10, out, coef, x, y, -1, True, True)
        return out

    def comb(coefs, trees):
        out = oracle.Tree(omra)
        oracle.add(-1.0, out, coefs, trees)
        return out

    same("rhoij_re", comb([1.0, 1.0], [prod(A, C, 1.0), prod(B, D, 1.0)]), 1e-11)
    same("rhoij_im", comb([1.0, 1.0], [prod(A, D, 1.0), prod(B, C, -1.0)]), 1e-11)

    # linear combination c0 phi^dagger + c1 chi, c0 = 0.5 - i, c1 = 2 + 0.25 i
    c0, c1 = complex(0.5, -1.0), complex(2.0, 0.25)
    same("lc_re", comb([c0.real, c0.imag, c1.real, -c1.imag], [A, B, C, D]), 1e-13)
    same("lc_im", comb([c0.imag, -c0.real, c1.imag, c1.real], [A, B, C, D]), 1e-13)

    # <phi|chi> = AC + BD + i (AD - BC); <phi| i phi> = i |phi|^2; phi^dagger dagger dagger = phi^dagger
    dre = oracle.dot(A, C) + oracle.dot(B, D)
    dim = oracle.dot(A, D) - oracle.dot(B, C)
    assert abs(res["dot_phi_chi"][0] - dre) <= 1e-12 * abs(dre)
    assert abs(res["dot_phi_chi"][1] - dim) <= 1e-12 * max(abs(dim), 1e-300)
    n2 = res["phi_sqnorm"]
    assert abs(n2 - (oracle.dot(A, A) + oracle.dot(B, B))) <= 1e-12 * n2
    assert abs(res["dot_phi_iphi"][0]) <= 1e-12 * n2 and abs(res["dot_phi_iphi"][1] - n2) <= 1e-12 * n2
    # acc = phi^dagger-flagged accumulator + phi holds phi; read through dagger().dagger() it is phi again
    assert abs(res["dot_phi_acc"][0] - n2) <= 1e-12 * n2 and abs(res["dot_phi_acc"][1]) <= 1e-12 * n2
