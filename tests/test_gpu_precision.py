"""Precision mode (eik_options.precision = 1): tets flagged by the condition
number of their metric edge Gram matrix run their local updates in FP64; the
rest of the solve is the reference's FP32 arithmetic.  Held against an FP64 run
of the same scheme (the oracle at precision 64, same partition)."""
import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def prec_case(mg):
    xyz, tets, sl = mg.sliver_cube(13, 0.10, seed=5)
    M6 = mg.anisotropic_metrics(tets.shape[0], seed=6)
    rng = np.random.Generator(np.random.PCG64(8))
    seeds = rng.choice(xyz.shape[0], 4, replace=False).astype(np.int32)
    return xyz, tets, sl, M6, seeds


def _solve(eik, case, precision, kappa=1e4):
    xyz, tets, _, M6, seeds = case
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.initSpeedMtxMultipliers(M6.ravel())
    e.setSeeds(seeds)
    e.maxIterations_ = 1000
    e.precisionMode_ = precision
    e.precisionKappa_ = kappa
    e.solveEikonal()
    return e


def test_precision_mode_moves_toward_fp64(need_gpu, eik, O, prec_case):
    xyz, tets, sl, M6, seeds = prec_case
    assert sl.mean() > 0.03  # the mesh does carry slivers
    e32 = _solve(eik, prec_case, 0)
    emx = _solve(eik, prec_case, 1)
    lab, nb = e32.getPartition()
    M = O.metrics_from_speeds(tets.shape[0], M6.ravel())
    r64 = O.solve3d(xyz, tets, M, lab, nb, seeds, max_iters=1000, precision=64)["result"].astype(np.float64)
    st = emx.stats()
    assert st["flagged_tets"] > 0.5 * sl.sum()
    assert e32.stats()["flagged_tets"] == 0
    err32 = np.abs(e32.getFinalResult() - r64) / np.maximum(np.abs(r64), 1e-6)
    errmx = np.abs(emx.getFinalResult() - r64) / np.maximum(np.abs(r64), 1e-6)
    # FP64 on the flagged tets and the FP64 polish remove the FP32 error: the
    # largest relative error against the FP64 run is at least 10x below FP32's
    assert errmx.max() <= 0.1 * err32.max(), (errmx.max(), err32.max())
    assert errmx.mean() < 0.2 * err32.mean(), (errmx.mean(), err32.mean())
    # the polish leaves no vertex that an FP64 update of its tets would lower by
    # 1e-4 relative or more (device check), and the CPU restatement agrees
    assert st["polish_rounds"] >= 1
    assert st["residual_max_rel"] < 1e-4, st["residual_max_rel"]
    assert st["residual_max_abs"] < 1e-4 * float(np.max(emx.getFinalResult()))
    res = O.fp64_residual(xyz, tets, M, emx.getFinalResult())
    assert res["lowerable"] < 1e-4, res
    # times below every FP64 update of their tets (the update is not monotone in
    # its inputs) are reported; the CPU restatement (FP64 products for every tet,
    # where the device keeps FP32 products for unflagged ones) finds a gap of the
    # same size
    b = st["residual_below_rel"]
    assert b <= 2 * res["below"] + 1e-5 and res["below"] <= 2 * b + 1e-5, (b, res)


def test_precision_kernel_without_flags_is_the_fp32_kernel(need_gpu, eik, prec_case):
    """With nothing flagged the precision kernel takes the FP32 path for every
    slot and must give the FP32 bits."""
    e32 = _solve(eik, prec_case, 0)
    enf = _solve(eik, prec_case, 1, kappa=1e30)
    assert enf.stats()["flagged_tets"] == 0
    assert bits_equal(e32.getFinalResult(), enf.getFinalResult())
    assert e32.numIterations() == enf.numIterations()


def test_fp64_update_matches_the_fp64_oracle(need_gpu, eik, O):
    """The precision mode's FP64 tet update (FP32 roots of the candidate distances)
    against the CPU restatement in FP64, on random tets over eight decades of size
    with random arrival times."""
    rng = np.random.default_rng(17)
    n = 20000
    P = rng.normal(size=(n, 4, 3)) * np.exp(rng.uniform(-4, 4, (n, 1, 1)))
    T = rng.uniform(0, 2, (n, 3)) * np.abs(P[:, :1, 0])
    AC, BC, CD = P[:, 2] - P[:, 0], P[:, 2] - P[:, 1], P[:, 3] - P[:, 2]
    g = np.stack([(AC * AC).sum(1), (AC * BC).sum(1), (AC * CD).sum(1), (BC * BC).sum(1), (BC * CD).sum(1),
                  (CD * CD).sum(1)], 1)
    inp = np.concatenate([T, g], 1).astype(np.float32)
    got = eik.selftest_local_update(5, inp).astype(np.float64)
    f = O.lib().oracle_tet_update_f64
    want = np.array([f(*map(float, row)) for row in inp])
    rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-30)
    # FP32 roots of the candidate distances: ~1e-7; a candidate whose barycentric
    # test sits on its boundary may switch in rare cases
    assert np.median(rel) < 1e-7
    assert np.mean(rel < 1e-6) > 0.999
