"""Batched solves (eik_batch_*): every instance of a batch must equal, bit for bit,
the solve of its handle alone, with the same iteration count.  The batch has no
counterpart in the reference (src/Eikonal.cu solves one mesh per object); the
standalone solve it is held to is the one the other GPU tests pin against the
reference's own kernels."""
import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _cube_solver(eik, mg, n, seed, seeds, vpb=64, max_iters=100):
    xyz, tets = mg.kuhn_cube(n, 0.2, seed=seed)
    speed = mg.log_uniform_speeds(tets.shape[0], seed=seed + 100)
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.initSpeedMtxMultipliers((1.0 / speed.astype(np.float64) ** 2).astype(np.float32))
    e.setSeeds(list(seeds))
    e.maxVertsPerBlock_ = vpb
    e.maxIterations_ = max_iters
    return e


def _sphere_solver(eik, mg, level, seeds, vpb=32, max_iters=100):
    xyz, faces = mg.icosphere(level)
    e = eik.Eikonal(True)
    e.set_mesh(xyz, faces)
    e.initSpeedMtxMultipliers(mg.batch_speed(xyz, faces))
    e.setSeeds(list(seeds))
    e.maxVertsPerBlock_ = vpb
    e.maxIterations_ = max_iters
    return e


def _alone(e):
    e.solveEikonal()
    return e.getFinalResult(), e.numIterations()


def test_batch3d_equals_standalone(need_gpu, eik, mg):
    rng = np.random.default_rng(11)
    specs = [(9, 1), (13, 2), (7, 3), (17, 4), (11, 5)]
    solvers = []
    for n, sd in specs:
        seeds = rng.choice(n ** 3, size=int(rng.integers(1, 4)), replace=False)
        solvers.append(_cube_solver(eik, mg, n, sd, seeds))
    want = [_alone(e) for e in solvers]
    b = eik.EikonalBatch(solvers)
    b.solveEikonal()
    for i, (res, it) in enumerate(want):
        assert b.numIterations(i) == it, (i, b.numIterations(i), it)
        assert bits_equal(b.getFinalResult(i), res), i
    got = b.getFinalResults()
    for i, (res, _) in enumerate(want):
        assert bits_equal(got[i], res), i
    st = b.stats()
    assert st["iterations"] == max(it for _, it in want)


def test_batch2d_equals_standalone(need_gpu, eik, mg):
    rng = np.random.default_rng(12)
    levels = [1, 3, 2, 4, 2, 1]
    solvers = []
    for lv in levels:
        nv = 10 * 4 ** lv + 2
        seeds = rng.choice(nv, size=int(rng.integers(1, 9)), replace=False)
        solvers.append(_sphere_solver(eik, mg, lv, seeds))
    want = [_alone(e) for e in solvers]
    b = eik.EikonalBatch(solvers)
    b.solveEikonal()
    for i, (res, it) in enumerate(want):
        assert b.numIterations(i) == it, (i, b.numIterations(i), it)
        assert bits_equal(b.getFinalResult(i), res), i


def test_batch_per_instance_iteration_caps(need_gpu, eik, mg):
    caps = [3, 100, 1, 7]
    solvers = [_cube_solver(eik, mg, 13, 20 + i, [mg.center_vertex(13)], max_iters=c) for i, c in enumerate(caps)]
    want = [_alone(e) for e in solvers]
    assert [it for _, it in want][0] == 3
    b = eik.EikonalBatch(solvers)
    b.solveEikonal()
    for i, (res, it) in enumerate(want):
        assert b.numIterations(i) == it
        assert bits_equal(b.getFinalResult(i), res), i


def test_batch_resolve_with_new_seeds_and_repeated_handle(need_gpu, eik, mg):
    a = _sphere_solver(eik, mg, 3, [0])
    c = _sphere_solver(eik, mg, 2, [5, 17])
    b = eik.EikonalBatch([a, c, a])  # the same handle twice: two identical instances
    b.solveEikonal()
    r0 = b.getFinalResults()
    assert bits_equal(r0[0], r0[2])
    # new seeds are picked up without a repack; a speed change forces one
    a.setSeeds([100, 200])
    c.initSpeedMtxMultipliers(mg.batch_speed(*mg.icosphere(2)) * np.float32(1.5))
    b.solveEikonal()
    got = b.getFinalResults()
    wa, _ = _alone(a)
    wc, _ = _alone(c)
    assert bits_equal(got[0], wa) and bits_equal(got[2], wa)
    assert bits_equal(got[1], wc)
    assert not bits_equal(got[0], r0[0])


def test_autotuner_picks_a_measured_shape_and_keeps_results(need_gpu, eik, mg):
    tune = __import__("importlib").import_module("sci-solver_eikonal_gb300.autotune")
    rng = np.random.default_rng(21)
    solvers = [_sphere_solver(eik, mg, lv, rng.choice(10 * 4 ** lv + 2, size=3, replace=False))
               for lv in (2, 3, 3, 4)]
    res, batch = tune.tune_batch(solvers, vpb_candidates=(16, 64), reps=1, workers=2)
    assert res.verts_per_block in (16, 64)
    assert len(res.table) == 2 and all("solve_ms" in r for r in res.table)
    best = min(res.table, key=lambda r: r["solve_ms"])
    assert best["verts_per_block"] == res.verts_per_block
    batch.solveEikonal()
    for i, e in enumerate(solvers):  # handles keep the chosen block size
        assert e.maxVertsPerBlock_ == res.verts_per_block
        want, it = _alone(e)
        assert bits_equal(batch.getFinalResult(i), want)


@pytest.mark.parametrize("dim", [2, 3])
def test_batch_device_build_equals_host_build(need_gpu, eik, mg, dim):
    """A batch whose handles build on the device builds one layout for all
    instances there (the meshes as one disconnected mesh); it equals the
    concatenated host layouts, and every instance its standalone solve."""
    rng = np.random.default_rng(30 + dim)
    if dim == 2:
        solvers = [_sphere_solver(eik, mg, lv, rng.choice(10 * 4 ** lv + 2, size=3, replace=False))
                   for lv in (3, 1, 4, 2, 3)]
        solvers[2].initSpeedMtxMultipliers(np.ones(0, np.float32))  # default speeds on one instance
    else:
        solvers = [_cube_solver(eik, mg, n, 40 + n, rng.choice(n ** 3, size=2, replace=False)) for n in (9, 13, 11)]
        # one instance with 6-entry metrics: the device pass expands the others' scalars
        xyz, tets = mg.kuhn_cube(10, 0.2, seed=7)
        e = eik.Eikonal(False)
        e.set_mesh(xyz, tets)
        e.initSpeedMtxMultipliers(mg.anisotropic_metrics(tets.shape[0], seed=8).ravel())
        e.setSeeds([3])
        solvers.insert(1, e)
    runs = {}
    for dev in (1, 0):
        for e in solvers:
            e.deviceSetup_ = dev
        b = eik.EikonalBatch(solvers)
        b.solveEikonal()
        runs[dev] = (b.getFinalResults(), [b.numIterations(i) for i in range(len(solvers))], b.stats())
    for i in range(len(solvers)):
        assert bits_equal(runs[1][0][i], runs[0][0][i]), i
    assert runs[1][1] == runs[0][1]
    for k in ("num_blocks", "total_slots", "vertex_updates", "fim_visits", "check_visits", "max_slots_per_block"):
        assert runs[1][2][k] == runs[0][2][k], (k, runs[1][2][k], runs[0][2][k])
    for i, e in enumerate(solvers):
        e.deviceSetup_ = 1
        res, it = _alone(e)
        assert it == runs[1][1][i] and bits_equal(res, runs[1][0][i]), i
