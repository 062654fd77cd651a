"""3D block layout built on the GPU (eik_options.device_setup = 1) against the
host build (device_setup = 0): same block statistics, same iteration and
vertex-update counts, same result bits."""
import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _solve(eik, xyz, tets, metric, seeds, device, vpb=64, structured=None, labels=None):
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    if metric is not None:
        e.initSpeedMtxMultipliers(metric)
    e.setSeeds(list(seeds))
    e.maxVertsPerBlock_ = vpb
    e.deviceSetup_ = 1 if device else 0
    if structured:
        e.isStructured_ = True
        e.squareLength_, e.squareWidth_, e.squareDepth_ = structured[0]
        e.squareBlockLength_, e.squareBlockWidth_, e.squareBlockDepth_ = structured[1]
    if labels is not None:
        e.setPartition(labels[0], labels[1])
    e.solveEikonal()
    return e


def _same(a, b):
    sa, sb = a.stats(), b.stats()
    for k in ("iterations", "num_blocks", "vertex_updates", "fim_visits", "check_visits", "total_slots",
              "max_slots_per_block", "max_local_vertices", "slot_visits", "halo_visits"):
        assert sa[k] == sb[k], (k, sa[k], sb[k])
    assert bits_equal(a.getFinalResult(), b.getFinalResult())


@pytest.mark.parametrize("n,vpb", [(9, 64), (17, 32), (33, 64), (25, 128)])
def test_device_layout_equals_host_layout_cubes(need_gpu, eik, mg, n, vpb):
    xyz, tets = mg.kuhn_cube(n, 0.2, seed=n)
    v = mg.log_uniform_speeds(tets.shape[0], seed=n + 1)
    metric = (1.0 / v.astype(np.float64) ** 2).astype(np.float32)
    seeds = np.random.default_rng(n).choice(xyz.shape[0], 3, replace=False)
    _same(_solve(eik, xyz, tets, metric, seeds, True, vpb), _solve(eik, xyz, tets, metric, seeds, False, vpb))


def test_device_layout_reference_fixtures(need_gpu, eik, golden):
    # sphere334, the anisotropic torus with its 6-entry metrics, the structured 16^3 cube
    _same(_solve(eik, golden["sphere334_xyz"], golden["sphere334_tets"], None, [0], True),
          _solve(eik, golden["sphere334_xyz"], golden["sphere334_tets"], None, [0], False))
    tm = golden["torus_metric"]
    _same(_solve(eik, golden["torus_xyz"], golden["torus_tets"], tm, [0], True),
          _solve(eik, golden["torus_xyz"], golden["torus_tets"], tm, [0], False))
    st = ((16, 16, 16), (4, 4, 4))
    _same(_solve(eik, golden["CubeMesh_size16_xyz"], golden["CubeMesh_size16_tets"], None, [0], True, structured=st),
          _solve(eik, golden["CubeMesh_size16_xyz"], golden["CubeMesh_size16_tets"], None, [0], False, structured=st))


def test_device_layout_user_partition_and_speed_change(need_gpu, eik, mg):
    xyz, tets = mg.kuhn_cube(17, 0.2, seed=3)
    p = eik.Eikonal(False)
    p.set_mesh(xyz, tets)
    p.maxVertsPerBlock_ = 48
    p.prepare()  # host partition only
    lab, nb = p.getPartition()
    # the same blocks under shuffled block ids (block order is not vertex order)
    labels = np.random.default_rng(4).permutation(nb).astype(np.int32)[lab]
    m1 = mg.log_uniform_speeds(tets.shape[0], seed=5)
    a = _solve(eik, xyz, tets, m1, [7, 900], True, labels=(labels, nb))
    b = _solve(eik, xyz, tets, m1, [7, 900], False, labels=(labels, nb))
    _same(a, b)
    # new speeds on the same handles: the device path recomputes the metric terms on the GPU
    m2 = mg.log_uniform_speeds(tets.shape[0], seed=6)
    for e in (a, b):
        e.initSpeedMtxMultipliers(m2)
        e.solveEikonal()
    _same(a, b)
    c = _solve(eik, xyz, tets, m2, [7, 900], True, labels=(labels, nb))
    _same(a, c)
    # the same handle switched between the two builds
    a.deviceSetup_ = 0
    a.solveEikonal()
    _same(a, c)
    a.deviceSetup_ = 1
    a.solveEikonal()
    _same(a, c)


def _solve2d(eik, xyz, faces, speeds, seeds, device, opts):
    e = eik.Eikonal(True)
    e.set_mesh(xyz, faces)
    if speeds is not None:
        e.initSpeedMtxMultipliers(speeds)
    e.setSeeds(list(seeds))
    for k, v in opts.items():
        setattr(e, k, v)
    e.deviceSetup_ = 1 if device else 0
    e.solveEikonal()
    return e


@pytest.mark.parametrize("case", ["grid", "ico", "sphere_speed", "square_structured"])
def test_device_layout_2d_equals_host_layout(need_gpu, eik, mg, golden, case):
    # triangle meshes: slots (inside, shared, virtual faces of obtuse corners),
    # halo lists, inverse face speeds and the copies the reference never refreshes
    if case == "grid":
        xyz, f = mg.grid2d(41)
        args = (None, [0, 700], {"maxVertsPerBlock_": 16})
    elif case == "ico":
        xyz, f = mg.icosphere(5)
        args = (mg.batch_speed(xyz, f), [0, 7], {"maxVertsPerBlock_": 32})
    elif case == "sphere_speed":
        xyz, f = golden["sphere_1154verts_xyz"], golden["sphere_1154verts_faces"]
        args = (mg.batch_speed(xyz, f), [0, 500], {"maxVertsPerBlock_": 32})
    else:
        xyz, f = golden["SquareMesh_size16_xyz"], golden["SquareMesh_size16_faces"]
        args = (None, [0], {"isStructured_": 1, "squareBlockLength_": 4, "squareBlockWidth_": 4})
    sp, seeds, opts = args
    a = _solve2d(eik, xyz, f, sp, seeds, True, opts)
    b = _solve2d(eik, xyz, f, sp, seeds, False, opts)
    _same(a, b)
    # new face speeds on the same handles: the device path recomputes them on the GPU
    sp2 = np.random.default_rng(len(f)).uniform(0.5, 2.0, len(f)).astype(np.float32)
    for e in (a, b):
        e.initSpeedMtxMultipliers(sp2)
        e.solveEikonal()
    _same(a, b)
    _same(a, _solve2d(eik, xyz, f, sp2, seeds, True, opts))
