"""The double-FP32 tier of the apply (values as unevaluated pairs of FP32 numbers).

Precision "df" runs every item whose bound b is at most 1e11 x the screening threshold in
double-FP32 (about 3e-13 b per item), so the result must agree with the FP64 apply to about
1e-12. That is a tolerance no FP32 or TF32 path could meet (1e-7 and 1e-4 per item), so a slip
in the error-free transformations or the exclusion of the scaling-scaling path shows at once.
In "mixed" the tier takes the items between 2e6 and 1e11 x the threshold.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GAUSS = [(1.0, 3.0, (0.15, -0.1, 0.05), (0, 0, 0)), (0.6, 12.0, (-0.4, 0.3, 0.2), (1, 0, 0)),
         (0.3, 40.0, (0.5, 0.25, -0.35), (0, 1, 1))]
TOL = 1e-10


def diff_rel(engine, mra, a, b):
    d = engine.FunctionTree(mra)
    engine.add(-1.0, d, [(1.0, a), (-1.0, b)])
    return d.norm() / b.norm()


@pytest.mark.parametrize("order,prec", [(3, 1e-4), (5, 1e-5), (7, 1e-6), (9, 1e-6)])
@pytest.mark.parametrize("abs_prec", [True, False])
def test_df_matches_fp64(engine, order, prec, abs_prec):
    mra = engine.MultiResolutionAnalysis(order)
    f = engine.project(prec, engine.FunctionTree(mra), GAUSS, abs_prec=True)
    f.rescale(1.0 / f.norm())
    H = engine.HelmholtzOperator(mra, 0.9, prec)
    v64, vdf = engine.FunctionTree(mra), engine.FunctionTree(mra)
    engine.apply(prec, v64, H, f, abs_prec=abs_prec, precision="fp64")
    st = engine.apply(prec, vdf, H, f, abs_prec=abs_prec, precision="df")
    assert st["items_df"] > 0 and st["items_df"] == st["items"] - st["items_fp64"]
    assert st["items_fp32"] == 0 and st["items_tf32"] == 0
    assert vdf.nnodes == v64.nnodes
    assert diff_rel(engine, mra, vdf, v64) <= TOL


def test_df_poisson_batch_matches_fp64(engine):
    prec = 1e-7
    mra = engine.MultiResolutionAnalysis(7)
    rng = np.random.default_rng(5)
    rhos = []
    for _ in range(3):
        c = tuple(rng.uniform(-1.0, 1.0, 3))
        rhos.append(engine.project(prec, engine.FunctionTree(mra), [(1.0, float(rng.uniform(2.0, 30.0)), c, (0, 0, 0))],
                                   abs_prec=True))
    P = engine.PoissonOperator(mra, prec)
    o64 = [engine.FunctionTree(mra) for _ in rhos]
    odf = [engine.FunctionTree(mra) for _ in rhos]
    engine.apply_batch([prec] * 3, o64, [P] * 3, rhos, abs_prec=True, precision="fp64")
    st = engine.apply_batch([prec] * 3, odf, [P] * 3, rhos, abs_prec=True, precision="df")
    assert st["items_df"] > 0
    for a, b in zip(odf, o64):
        assert diff_rel(engine, mra, a, b) <= TOL


def test_mixed_uses_df_for_large_bounds(engine):
    # at prec 1e-7 many near-diagonal items have bounds far above the FP32 limit
    prec = 1e-7
    mra = engine.MultiResolutionAnalysis(9)
    f = engine.project(prec, engine.FunctionTree(mra), GAUSS, abs_prec=True)
    f.rescale(1.0 / f.norm())
    H = engine.HelmholtzOperator(mra, 1.1, prec)
    v64, vmx, v32 = engine.FunctionTree(mra), engine.FunctionTree(mra), engine.FunctionTree(mra)
    engine.apply(prec, v64, H, f, abs_prec=True, precision="fp64")
    st = engine.apply(prec, vmx, H, f, abs_prec=True, precision="mixed")
    s32 = engine.apply(prec, v32, H, f, abs_prec=True, precision="mixed-fp32")
    assert st["items_df"] > 0 and s32["items_df"] == 0
    assert st["items_fp64"] < s32["items_fp64"]
    assert diff_rel(engine, mra, vmx, v64) <= prec
