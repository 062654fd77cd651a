"""The 3D sweep kernel runs a visit's sweeps from lists of the apex updates that can
change something (exact skips: inputs at LARGENUM, unchanged inputs, upwind apexes,
non-owned apexes in the last sweep); the precision kernel keeps the loop over every
slot.  With nothing flagged the precision kernel computes the FP32 updates, so the
two must agree bit for bit for any number of sweeps per visit."""
import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sweeps", [1, 2, 3])
def test_packed_last_sweep_equals_plain_loop(need_gpu, eik, mg, O, sweeps):
    xyz, tets = mg.kuhn_cube(21, 0.2, seed=21)
    sp = mg.log_uniform_speeds(tets.shape[0], 0.5, 2.0, seed=22)
    metric = (1.0 / sp.astype(np.float64) ** 2).astype(np.float32)
    out = []
    for prec in (0, 1):
        e = eik.Eikonal(False)
        e.set_mesh(xyz, tets)
        e.initSpeedMtxMultipliers(metric)
        e.setSeeds([0, xyz.shape[0] - 1])
        e.maxVertsPerBlock_ = 64
        e.keepHistory_ = 0
        e.fimSweeps_ = sweeps
        e.precisionMode_ = prec
        e.precisionKappa_ = 1e30  # nothing flagged: the FP32 path everywhere
        e.solveEikonal()
        assert e.stats()["flagged_tets"] == 0
        out.append(e)
    assert bits_equal(out[0].getFinalResult(), out[1].getFinalResult())
    assert out[0].numIterations() == out[1].numIterations()
    assert out[0].stats()["vertex_updates"] == out[1].stats()["vertex_updates"]
    # and the scheme itself: the CPU restatement with the same sweep count
    lab, nb = out[0].getPartition()
    want = O.solve3d(xyz, tets, O.metrics_from_speeds(tets.shape[0], metric), lab, nb,
                     [0, xyz.shape[0] - 1], nsweeps=sweeps)["result"]
    rel = np.abs(out[0].getFinalResult() - want) / np.maximum(np.abs(want), 1e-6)
    assert np.median(rel) < 1e-6 and rel.max() < 1e-2


def test_cta_size_does_not_change_results(need_gpu, eik, mg):
    """Blocks larger than the CTA run several slots or apex items per thread in
    every loop (the item lists, the check memo, the copies); the results must not
    depend on the CTA size."""
    xyz, tets = mg.kuhn_cube(25, 0.2, seed=31)
    sp = mg.log_uniform_speeds(tets.shape[0], 0.5, 2.0, seed=32)
    metric = (1.0 / sp.astype(np.float64) ** 2).astype(np.float32)
    out = []
    for threads in (0, 256, 128, 384, 512, 768, 1024):
        e = eik.Eikonal(False)
        e.set_mesh(xyz, tets)
        e.initSpeedMtxMultipliers(metric)
        e.setSeeds([7])
        e.maxVertsPerBlock_ = 64
        e.keepHistory_ = 0
        e.threadsPerBlock_ = threads
        e.solveEikonal()
        out.append(e)
    for e in out[1:]:
        assert bits_equal(out[0].getFinalResult(), e.getFinalResult())
        assert out[0].numIterations() == e.numIterations()
        assert out[0].stats()["check_visits"] == e.stats()["check_visits"]


def test_cta_size_choice_over_the_first_solves_keeps_the_bits(need_gpu, eik, mg):
    """With no CTA size given a handle runs the item kernels' size (or, in precision
    mode, tries two sizes over its first solves); every solve gives the same bits."""
    xyz, tets = mg.kuhn_cube(25, 0.2, seed=41)
    sp = mg.log_uniform_speeds(tets.shape[0], 0.5, 2.0, seed=42)
    metric = (1.0 / sp.astype(np.float64) ** 2).astype(np.float32)
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.initSpeedMtxMultipliers(metric)
    e.setSeeds([3])
    e.maxVertsPerBlock_ = 64
    e.keepHistory_ = 0
    res = []
    for _ in range(5):
        e.solveEikonal()
        res.append((e.getFinalResult().copy(), e.numIterations(), e.stats()["vertex_updates"]))
    for r, it, upd in res[1:]:
        assert bits_equal(res[0][0], r) and it == res[0][1] and upd == res[0][2]
