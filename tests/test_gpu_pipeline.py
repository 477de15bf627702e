"""The steps either side of the apply, on the device: density build (density::compute), the
Coulomb potential from it (CoulombPotential::setupGlobalPotential), V*phi followed by the
Helmholtz update (QMPotential::apply + HelmholtzVector::apply), orbital rotation, and the tree
file round trip (checkpoint)."""
import json
import math
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_values.json")))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def test_density_and_coulomb_reference_values(engine):
    """tests/qmoperators/coulomb_operator.cpp:78-84 through the device-resident pipeline."""
    ref = GOLDEN["coulomb"]
    prec = ref["prec"]
    mra = engine.MultiResolutionAnalysis(GOLDEN["mra"]["order"])
    phis = [engine.project_hydrogen(prec, engine.FunctionTree(mra), *o) for o in ref["orbitals"]]
    rho = engine.FunctionTree(mra)
    engine.density(prec, rho, phis, [ref["occupation"]] * len(phis), crop=False)
    assert abs(rho.integrate() - 10.0) < 1e-4
    J = engine.FunctionTree(mra)
    engine.apply(prec / rho.norm(), J, engine.PoissonOperator(mra, prec), rho)
    E = ref["E_P"]
    for i, p in enumerate(phis):
        jp = engine.FunctionTree(mra)
        engine.copy_grid(jp, p)
        engine.multiply(prec, jp, 1.0, J, p)
        v = engine.dot(p, jp)
        assert abs(v - E["%d,%d" % (i, i)]) < 1e-5 * E["%d,%d" % (i, i)], (i, v)


def test_density_matches_oracle(engine, oracle):
    prec = 1e-5
    mra, omra = engine.MultiResolutionAnalysis(7), oracle.MRA(7)
    terms = [[(1.0, 1.2, (0.3, 0.0, 0.0), (0, 0, 0))], [(1.0, 0.8, (-0.4, 0.2, 0.0), (1, 0, 0))]]
    ophis = [oracle.project_gauss(prec, oracle.Tree(omra), t) for t in terms]
    phis = [engine.FunctionTree(mra).upload(*o.export()[:2]) for o in ophis]
    rho = engine.FunctionTree(mra)
    engine.density(prec, rho, phis, [2.0, 1.0], crop=False)
    sq = []
    for p in ophis:
        r = oracle.Tree(omra)
        oracle.copy_grid(r, p)
        oracle.multiply(prec, r, 1.0, p, p)
        sq.append(r)
    orho = oracle.Tree(omra)
    oracle.add(prec, orho, [2.0, 1.0], sq)
    k1, c1, _ = rho.download()
    k2, c2, _ = orho.export()
    assert np.array_equal(k1, k2) and rel_l2(c1, c2) <= 1e-12


def test_potential_times_orbital_then_helmholtz(engine, oracle):
    """psi = -1/(2 pi) H_mu[V phi] on the device against the same steps in the oracle."""
    prec, mu = 1e-5, 1.1
    mra, omra = engine.MultiResolutionAnalysis(7), oracle.MRA(7)
    oV = oracle.project_gauss(prec, oracle.Tree(omra), [(-2.0, 0.7, (0.0, 0.0, 0.0), (0, 0, 0))])
    ophi = oracle.project_gauss(prec, oracle.Tree(omra), [(1.0, 1.5, (0.2, 0.1, 0.0), (0, 0, 0))])
    V = engine.FunctionTree(mra).upload(*oV.export()[:2])
    phi = engine.FunctionTree(mra).upload(*ophi.export()[:2])
    vphi = engine.FunctionTree(mra)
    engine.copy_grid(vphi, phi)
    engine.multiply_batch(prec, [vphi], 1.0, [V], [phi])
    out = engine.FunctionTree(mra)
    engine.apply_batch(prec, [out], [engine.HelmholtzOperator(mra, mu, prec)], [vphi], abs_prec=True)
    out.rescale(-1.0 / (2.0 * math.pi))
    ovphi = oracle.Tree(omra)
    oracle.copy_grid(ovphi, ophi)
    oracle.multiply(prec, ovphi, 1.0, oV, ophi)
    oout = oracle.Tree(omra)
    oracle.apply(prec, oout, oracle.helmholtz(omra, mu, prec), ovphi, abs_prec=True)
    oout.rescale(-1.0 / (2.0 * math.pi))
    k1, c1, _ = out.download()
    k2, c2, _ = oout.export()
    assert np.array_equal(k1, k2) and rel_l2(c1, c2) <= 1e-10


def test_rotation(engine):
    prec = 1e-6
    mra = engine.MultiResolutionAnalysis(7)
    ins = [engine.project(prec, engine.FunctionTree(mra), [(1.0, a, (0.2 * i, 0.0, 0.0), (0, 0, 0))])
           for i, a in enumerate((0.5, 2.0, 8.0))]
    th = 0.3
    U = np.array([[math.cos(th), math.sin(th), 0.0], [-math.sin(th), math.cos(th), 0.0], [0.0, 0.0, 1.0]])
    outs = [engine.FunctionTree(mra) for _ in range(3)]
    engine.rotate(outs, ins, U)
    # orthogonal U preserves the Gram matrix
    G_in = np.array([[engine.dot(a, b) for b in ins] for a in ins])
    G_out = np.array([[engine.dot(a, b) for b in outs] for a in outs])
    assert np.abs(G_out - U @ G_in @ U.T).max() < 1e-12
    pts = np.random.default_rng(4).uniform(-1, 1, (20, 3))
    vin = np.stack([t.evalf(pts) for t in ins])
    vout = np.stack([t.evalf(pts) for t in outs])
    assert np.abs(vout - U @ vin).max() < 1e-12


def test_tree_file_roundtrip(engine, tmp_path):
    mra = engine.MultiResolutionAnalysis(7)
    f = engine.project(1e-6, engine.FunctionTree(mra), [(1.0, 2.0, (0.1, 0.2, 0.3), (1, 0, 0))])
    path = str(tmp_path / "f.mwt")
    engine.save_tree(f, path)
    g = engine.load_tree(engine.FunctionTree(mra), path)
    k1, c1, l1 = f.download()
    k2, c2, l2 = g.download()
    assert np.array_equal(k1, k2) and np.array_equal(c1, c2) and np.array_equal(l1, l2)
    other = engine.MultiResolutionAnalysis(5)
    with pytest.raises(engine.MWError):
        engine.load_tree(engine.FunctionTree(other), path)
    with open(path, "r+b") as fh:
        fh.truncate(100)
    with pytest.raises(engine.MWError):
        engine.load_tree(engine.FunctionTree(mra), path)


def test_batched_upload_download_match_single(engine):
    # mw_tree_upload_batch / mw_tree_download_batch: the same trees, blocks and norms as one call
    # per tree, with keys given in a shuffled order
    mra = engine.MultiResolutionAnalysis(7)
    srcs = [engine.project(1e-5, engine.FunctionTree(mra), [(1.0, a, (0.1 * i, -0.2, 0.3), (i % 2, 0, 0))],
                           abs_prec=True) for i, a in enumerate((1.5, 6.0, 20.0))]
    data = [s.download() for s in srcs]
    rng = np.random.default_rng(3)
    shuffled = []
    for k, c, _ in data:
        p = rng.permutation(k.shape[0])
        shuffled.append((k[p], c[p]))
    single = [engine.FunctionTree(mra).upload(k, c) for k, c in shuffled]
    batch = engine.upload_batch([engine.FunctionTree(mra) for _ in shuffled], shuffled)
    got = engine.download_batch(batch)
    again = engine.download_batch(batch, outs=got)  # into the same buffers
    for s, b, (k0, c0, l0), (k1, c1, l1), (k2, c2, l2) in zip(single, batch, data, got, again):
        ks, cs, ls = s.download()
        assert np.array_equal(ks, k0) and np.array_equal(k1, k0) and np.array_equal(k2, k0)
        assert np.array_equal(cs, c0) and np.array_equal(c1, c0) and np.array_equal(c2, c0)
        assert np.array_equal(l1, l0) and s.norm() == b.norm()
    # pinned buffers: direct copies, with the reordering done on the device
    pinned_in = [(k.copy(), c.copy()) for k, c in shuffled]
    for _, c in pinned_in:
        engine.pin_host(mra, c)
    outs = [(np.empty_like(k), np.empty_like(c), np.empty_like(l)) for k, c, l in data]
    for o in outs:
        engine.pin_host(mra, o[1])
    pb = engine.upload_batch([engine.FunctionTree(mra) for _ in pinned_in], pinned_in)
    res = engine.download_batch(pb, outs=outs)
    for (k0, c0, l0), (k1, c1, l1), o, s, t in zip(data, res, outs, single, pb):
        assert c1 is o[1] and np.array_equal(k1, k0) and np.array_equal(c1, c0) and np.array_equal(l1, l0)
        assert s.norm() == t.norm()
    for _, c in pinned_in:
        engine.unpin_host(mra, c)
    for o in outs:
        engine.unpin_host(mra, o[1])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_apply_batch_host_matches_upload_then_apply(engine, precision):
    # mw_apply_batch_host (inputs uploaded per job group, overlapped with the first groups'
    # levels) against mw_tree_upload_batch + mw_apply_batch: the same input trees, bit-identical
    # outputs, with pinned and with pageable input buffers
    prec = 1e-6
    rng = np.random.default_rng(20261203)
    mra = engine.MultiResolutionAnalysis(9)
    mons = [(a, b, c) for a in range(4) for b in range(4) for c in range(4) if a + b + c <= 3]
    srcs, mus = [], []
    for _ in range(6):
        alpha = float(np.exp(rng.uniform(np.log(0.3), np.log(20.0))))
        R = tuple(rng.uniform(-2.0, 2.0, 3))
        terms = [(float(c), alpha, R, m) for c, m in zip(rng.standard_normal(len(mons)), mons)]
        f = engine.project(prec, engine.FunctionTree(mra), terms, abs_prec=True)
        f.rescale(1.0 / f.norm())
        srcs.append(f)
        mus.append(math.sqrt(-2.0 * rng.uniform(-2.0, -0.1)))
    ops = [engine.HelmholtzOperator(mra, mu, prec) for mu in mus]
    host = [s.download() for s in srcs]

    inps_a = engine.upload_batch([engine.FunctionTree(mra) for _ in srcs], host)
    outs_a = [engine.FunctionTree(mra) for _ in srcs]
    engine.apply_batch([prec] * len(srcs), outs_a, ops, inps_a, abs_prec=True, precision=precision)
    ref = engine.download_batch(outs_a)
    ref_in = engine.download_batch(inps_a)
    for pinned in (True, False):
        buffers = [(k, c.copy(), l) for k, c, l in host]
        if pinned:
            for _, c, _ in buffers:
                engine.pin_host(mra, c)
        inps_b = [engine.FunctionTree(mra) for _ in srcs]
        outs_b = [engine.FunctionTree(mra) for _ in srcs]
        st = engine.apply_batch_host([prec] * len(srcs), outs_b, ops, inps_b, buffers, abs_prec=True,
                                     precision=precision)
        assert st["items"] > 0
        for (k1, c1, l1), (k2, c2, l2) in zip(engine.download_batch(outs_b), ref):
            assert np.array_equal(k1, k2) and np.array_equal(c1, c2) and np.array_equal(l1, l2)
        for (k1, c1, _), (k2, c2, _) in zip(engine.download_batch(inps_b), ref_in):
            assert np.array_equal(k1, k2) and np.array_equal(c1, c2)
        # the input trees' host norms are those of an upload
        assert [t.norm() for t in inps_b] == [t.norm() for t in inps_a]
        if pinned:
            for _, c, _ in buffers:
                engine.unpin_host(mra, c)


def test_apply_batch_host_groups_and_node_order(engine):
    # the host-buffer apply with one to three job groups (each group's blocks on the copy stream,
    # its preparation on its own stream) and with the caller's nodes in a shuffled order (the
    # blocks permuted into tree order on the device): outputs bit-identical to upload + apply
    prec = 1e-6
    rng = np.random.default_rng(20261205)
    mra = engine.MultiResolutionAnalysis(9)
    srcs, ops = [], []
    for _ in range(5):
        R = tuple(rng.uniform(-2.0, 2.0, 3))
        alpha = float(np.exp(rng.uniform(np.log(0.5), np.log(10.0))))
        f = engine.project(prec, engine.FunctionTree(mra), [(1.0, alpha, R, (0, 1, 0)), (0.7, 1.5 * alpha, R, (0, 0, 1))],
                           abs_prec=True)
        f.rescale(1.0 / f.norm())
        srcs.append(f)
        ops.append(engine.HelmholtzOperator(mra, float(rng.uniform(0.5, 2.0)), prec))
    host = [s.download() for s in srcs]
    inps_a = engine.upload_batch([engine.FunctionTree(mra) for _ in srcs], host)
    outs_a = [engine.FunctionTree(mra) for _ in srcs]
    engine.apply_batch([prec] * 5, outs_a, ops, inps_a, abs_prec=True, precision="mixed")
    ref = engine.download_batch(outs_a)
    shuffled = []
    for k, c, l in host:
        p = rng.permutation(k.shape[0])
        b = (np.ascontiguousarray(k[p]), np.ascontiguousarray(c[p]), np.ascontiguousarray(l[p]))
        engine.pin_host(mra, b[1])
        shuffled.append(b)
    try:
        for groups in (1, 2, 3):
            mra.set_groups(groups)
            outs = [engine.FunctionTree(mra) for _ in srcs]
            st = engine.apply_batch_host([prec] * 5, outs, ops, [engine.FunctionTree(mra) for _ in srcs], shuffled,
                                         abs_prec=True, precision="mixed")
            assert st["items"] > 0
            for (k1, c1, l1), (k2, c2, l2) in zip(engine.download_batch(outs), ref):
                assert np.array_equal(k1, k2) and np.array_equal(c1, c2) and np.array_equal(l1, l2)
    finally:
        mra.set_groups(4)
        for b in shuffled:
            engine.unpin_host(mra, b[1])


def test_apply_batch_host_outputs(engine):
    # the outputs of mw_apply_batch_host go down per job group into the caller's pinned buffers:
    # equal to a download_batch afterwards; an output whose buffer is too small is left for
    # download_batch (its count comes back negative)
    prec = 1e-6
    rng = np.random.default_rng(20261204)
    mra = engine.MultiResolutionAnalysis(9)
    srcs, ops = [], []
    for _ in range(5):
        R = tuple(rng.uniform(-2.0, 2.0, 3))
        alpha = float(np.exp(rng.uniform(np.log(0.5), np.log(10.0))))
        f = engine.project(prec, engine.FunctionTree(mra), [(1.0, alpha, R, (1, 0, 0)), (0.5, 2 * alpha, R, (0, 0, 0))],
                           abs_prec=True)
        f.rescale(1.0 / f.norm())
        srcs.append(f)
        ops.append(engine.HelmholtzOperator(mra, float(rng.uniform(0.5, 2.0)), prec))
    host = [s.download() for s in srcs]
    for _, c, _ in host:
        engine.pin_host(mra, c)
    inps = [engine.FunctionTree(mra) for _ in srcs]
    outs = [engine.FunctionTree(mra) for _ in srcs]
    engine.apply_batch_host([prec] * 5, outs, ops, inps, host, abs_prec=True, precision="mixed")
    ref = engine.download_batch(outs)
    bufs = []
    for i, (k, c, l) in enumerate(ref):
        m = k.shape[0] - (1 if i == 2 else 0)  # job 2's buffer is one node short
        b = (np.zeros((m, 4), np.int32), np.zeros((m, c.shape[1])), np.zeros(m, np.uint8))
        engine.pin_host(mra, b[1])
        bufs.append(b)
    outs2 = [engine.FunctionTree(mra) for _ in srcs]
    st = engine.apply_batch_host([prec] * 5, outs2, ops, [engine.FunctionTree(mra) for _ in srcs], host,
                                 abs_prec=True, precision="mixed", outputs=bufs)
    assert st["outputs_filled"] == [True, True, False, True, True]
    for i, ((k1, c1, l1), (k2, c2, l2)) in enumerate(zip(bufs, ref)):
        if i == 2:
            continue
        assert np.array_equal(k1, k2) and np.array_equal(c1, c2) and np.array_equal(l1, l2)
    k3, c3, l3 = engine.download_batch([outs2[2]])[0]
    assert np.array_equal(k3, ref[2][0]) and np.array_equal(c3, ref[2][1])
    for b in bufs:
        engine.unpin_host(mra, b[1])
    for _, c, _ in host:
        engine.unpin_host(mra, c)
