"""The 3D check kernel skips slots whose input times an earlier check of the same
solve found settled.  The memo must not outlive its solve: re-solving a handle
with other seeds, speeds or precision mode gives the bits of a fresh handle."""
import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _cube(mg, n=25):
    xyz, tets = mg.kuhn_cube(n, 0.2, seed=11)
    sp1 = mg.log_uniform_speeds(tets.shape[0], 0.5, 2.0, seed=12)
    sp2 = mg.log_uniform_speeds(tets.shape[0], 0.5, 2.0, seed=13)
    m1 = (1.0 / sp1.astype(np.float64) ** 2).astype(np.float32)
    m2 = (1.0 / sp2.astype(np.float64) ** 2).astype(np.float32)
    return xyz, tets, m1, m2


def _handle(eik, xyz, tets, metric, seeds):
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.initSpeedMtxMultipliers(metric)
    e.setSeeds(list(seeds))
    e.maxVertsPerBlock_ = 64
    e.keepHistory_ = 0
    return e


def _same(a, b):
    assert bits_equal(a.getFinalResult(), b.getFinalResult())
    assert a.numIterations() == b.numIterations()
    assert a.stats()["vertex_updates"] == b.stats()["vertex_updates"]
    assert a.stats()["check_visits"] == b.stats()["check_visits"]


def test_resolve_with_new_seeds_matches_fresh_handle(need_gpu, eik, mg):
    xyz, tets, m1, _ = _cube(mg)
    e = _handle(eik, xyz, tets, m1, [0])
    e.solveEikonal()
    e.solveEikonal()  # the same solve twice: memos from the first must not leak
    f = _handle(eik, xyz, tets, m1, [0])
    f.solveEikonal()
    _same(e, f)
    e.setSeeds([xyz.shape[0] // 2, 7])
    e.solveEikonal()
    g = _handle(eik, xyz, tets, m1, [xyz.shape[0] // 2, 7])
    g.solveEikonal()
    _same(e, g)


def test_resolve_with_new_speeds_matches_fresh_handle(need_gpu, eik, mg):
    xyz, tets, m1, m2 = _cube(mg)
    e = _handle(eik, xyz, tets, m1, [3])
    e.solveEikonal()
    e.initSpeedMtxMultipliers(m2)
    e.solveEikonal()
    f = _handle(eik, xyz, tets, m2, [3])
    f.solveEikonal()
    _same(e, f)


def test_precision_toggle_matches_fresh_handle(need_gpu, eik, mg):
    xyz, tets, m1, _ = _cube(mg, 17)
    e = _handle(eik, xyz, tets, m1, [5])
    e.solveEikonal()
    e.precisionMode_ = 1
    e.precisionKappa_ = 30.0  # flags some of the jittered tets
    e.solveEikonal()
    f = _handle(eik, xyz, tets, m1, [5])
    f.precisionMode_ = 1
    f.precisionKappa_ = 30.0
    f.solveEikonal()
    assert f.stats()["flagged_tets"] > 0
    _same(e, f)


def test_checks_inside_the_sweep_launch_are_counted(need_gpu, eik, mg):
    """On the item path the neighbour checks of iteration k run in the sweep launch
    of iteration k + 1: no check launch, the per-iteration counts add up to the
    solve's totals, and the vertex-update count is the reference's (owned vertices x
    2 per sweep visit + owned vertices per check visit)."""
    xyz, tets, m1, _ = _cube(mg, 21)
    e = _handle(eik, xyz, tets, m1, [0])
    e.solveEikonal()
    st = e.stats()
    its = e.iterationStats()
    assert its.shape == (e.numIterations(), len(e.ITERATION_STAT_COLUMNS)) == (e.numIterations(), 16)
    assert st["check_launches"] == 0 and st["check_kernel_ms"] == 0.0
    assert st["check_visits"] > 0
    assert its[:, 2].sum() == st["fim_visits"] and its[:, 6].sum() == st["check_visits"]
    assert its[:, 5].sum() * 2 + its[:, 9].sum() == st["vertex_updates"]
    # sweeps of blocks staged by their own check: a subset of each iteration's visits
    assert (its[:, 12] <= its[:, 2]).all() and its[:, 12].sum() > 0
    assert (its[:, 13] <= its[:, 3]).all()
    # launch start offsets on the device timer, in iteration order
    starts = its[:, 10]
    assert starts[0] == 0 and (np.diff(starts) > 0).all()


def test_telemetry_off_keeps_results(need_gpu, eik, mg):
    """Without telemetry the solve records no launch spans or per-iteration rows and
    gives the same bits, iterations and vertex updates."""
    xyz, tets, m1, _ = _cube(mg, 17)
    out = []
    for tele in (1, 0):
        e = _handle(eik, xyz, tets, m1, [0])
        e.telemetry_ = tele
        e.solveEikonal()
        out.append(e)
    on, off = out
    assert bits_equal(on.getFinalResult(), off.getFinalResult())
    assert on.numIterations() == off.numIterations()
    assert on.stats()["vertex_updates"] == off.stats()["vertex_updates"]
    assert on.stats()["fim_kernel_ms"] > 0 and on.iterationStats().shape[0] == on.numIterations()
    assert off.stats()["fim_kernel_ms"] == 0 and off.stats()["fim_launches"] == 0
    assert off.iterationStats().shape[0] == 0
    # switching back on rebuilds the loop with telemetry
    off.telemetry_ = 1
    off.solveEikonal()
    assert off.iterationStats().shape[0] == off.numIterations()
    assert bits_equal(on.getFinalResult(), off.getFinalResult())
