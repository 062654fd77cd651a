"""The oracle (CPU restatement of the reference scheme) pinned against the
reference: its tet update against the reference's own localSolverTet1 compiled
for the host, and whole solves against the reference tests' known answers
(src/test/3d/3D-small.cc, 3D-converge.cc, 2D-improve.cc)."""
import numpy as np
import pytest

from conftest import relerr


def random_tet_cases(rng, n):
    P = rng.normal(size=(n, 4, 3)).astype(np.float32) * np.exp(rng.uniform(-3, 3, size=(n, 1, 1))).astype(np.float32)
    T = rng.uniform(0, 2, size=(n, 3)).astype(np.float32) * np.abs(P[:, :1, 0]).astype(np.float32)
    T[rng.random((n, 3)) < 0.15] = 1e9
    AC, BC, CD = P[:, 2] - P[:, 0], P[:, 2] - P[:, 1], P[:, 3] - P[:, 2]
    g = np.stack([(AC * AC).sum(1), (AC * BC).sum(1), (AC * CD).sum(1), (BC * BC).sum(1), (BC * CD).sum(1),
                  (CD * CD).sum(1)], 1).astype(np.float32)
    return np.concatenate([T, g], 1).astype(np.float32)


def test_tet_update_matches_reference_host_build(O):
    ref = O.ref_lib()
    if ref is None:
        pytest.skip("reference host build not present (built from the reference tree)")
    rng = np.random.default_rng(7)
    cases = random_tet_cases(rng, 20000)
    L = O.lib()
    for row in cases:
        a = [float(x) for x in row]
        r = np.float32(ref.ref_tet_local_solver(*a))
        o = np.float32(L.oracle_tet_update_f32(*a))
        assert r.tobytes() == o.tobytes(), (a, r, o)


def test_tet_update_fp64_close_on_mesh_tets(O, mg):
    """On well-shaped tets with causal arrival times the FP32 update agrees with the
    FP64 one to single-precision accuracy in almost every case; the reference's
    quadratic loses accuracy when the wavefront is nearly planar across a small tet
    (the FP64 path of the precision mode exists for this), so the worst case is
    bounded separately."""
    rng = np.random.default_rng(3)
    xyz, tets = mg.kuhn_cube(7, 0.2, seed=1)
    L = O.lib()
    errs = []
    for t in rng.choice(tets.shape[0], 400, replace=False):
        P = xyz[tets[t]].astype(np.float64)
        src = rng.normal(size=3) * 3
        for apex in range(4):
            idx = [(apex + k) % 4 for k in (1, 2, 3)] + [apex]
            A, B, C, D = P[idx]
            T = [np.linalg.norm(A - src), np.linalg.norm(B - src), np.linalg.norm(C - src)]
            AC, BC, CD = C - A, C - B, D - C
            g = [AC @ AC, AC @ BC, AC @ CD, BC @ BC, BC @ CD, CD @ CD]
            a32 = L.oracle_tet_update_f32(*[float(np.float32(x)) for x in T + g])
            a64 = L.oracle_tet_update_f64(*(T + g))
            errs.append(abs(a32 - a64) / max(1.0, abs(a64)))
    errs = np.array(errs)
    assert np.percentile(errs, 99) <= 1e-5, np.percentile(errs, 99)
    assert errs.max() <= 1e-3, errs.max()


@pytest.mark.parametrize("name,tol", [("sphere8", None), ("sphere13", 1e-4)])
def test_known_answer_small_balls(O, golden, name, tol):
    """3D-small.cc: seed vertex 0 at 0, every other vertex at 19.58."""
    xyz, tets = golden[name + "_xyz"], golden[name + "_tets"]
    M = O.metrics_from_speeds(tets.shape[0], None)
    for lab in (np.r_[0, np.ones(xyz.shape[0] - 1)], np.arange(xyz.shape[0]) % 2):
        r = O.solve3d(xyz, tets, M, lab.astype(np.int32), 2, [0])["result"]
        assert r[0] == 0.0
        if tol is None:  # EXPECT_FLOAT_EQ: within 4 ulps
            assert np.all(np.abs(r[1:] - np.float32(19.58)) <= 4 * np.spacing(np.float32(19.58)))
        else:
            assert np.all(np.abs(r[1:] - 19.58) <= tol)


def test_history_monotone_sphere334(O, golden):
    """3D-converge.cc: travel times never increase from one iteration to the next."""
    xyz, tets = golden["sphere334_xyz"], golden["sphere334_tets"]
    lab = (np.arange(xyz.shape[0]) * 6 // xyz.shape[0]).astype(np.int32)
    r = O.solve3d(xyz, tets, O.metrics_from_speeds(tets.shape[0], None), lab, 6, [0], history=True)
    h = r["history"]
    assert h.shape[0] == r["iterations"] >= 2
    for i in range(2, h.shape[0]):
        prev, cur = h[i - 1], h[i]
        m = prev != 0
        assert np.all(cur[m] <= prev[m])


def test_uniform_cube_fp32_vs_fp64_and_distance(O, mg):
    xyz, tets = mg.kuhn_cube(13, 0.2, seed=1)
    seed = mg.center_vertex(13)
    lab = (np.arange(xyz.shape[0]) // 64).astype(np.int32)
    nb = int(lab.max()) + 1
    M = O.metrics_from_speeds(tets.shape[0], None)
    r32 = O.solve3d(xyz, tets, M, lab, nb, [seed], max_iters=500)
    r64 = O.solve3d(xyz, tets, M, lab, nb, [seed], max_iters=500, precision=64)
    d = np.linalg.norm(xyz.astype(np.float64) - xyz[seed], axis=1)
    h = 1.0 / 12
    # first-order scheme around a point source on a jittered mesh: error within
    # about one edge length
    assert np.abs(r64["result"] - d).max() < 1.5 * h
    # FP32 against the FP64 run of the same scheme (rounding plus convergence
    # decisions taken at the 1e-5 threshold)
    assert np.abs(r32["result"] - r64["result"]).max() < 5e-3


def test_grid2d_oracle_against_distance(O, eik, mg):
    xyz, faces = mg.grid2d(17)
    e = eik.Eikonal(True)
    e.set_mesh(xyz, faces)
    f, obt, off, vfv = e.triPrep()
    lab = ((np.arange(xyz.shape[0]) % 17) // 4 + 5 * ((np.arange(xyz.shape[0]) // 17) // 4)).astype(np.int32)
    init = np.full(xyz.shape[0], 1e7, np.float32)
    init[0] = 0
    r = O.solve2d(xyz, f, np.ones(f.shape[0], np.float32), obt, off, vfv, lab, int(lab.max()) + 1, [0], init)
    d = np.linalg.norm(xyz.astype(np.float64), axis=1)
    assert r["result"][0] == 0
    # a first-order scheme from a corner: a few percent at the coarsest vertices
    assert relerr(r["result"], d, 1e-3).max() < 0.05


def test_improve2d_rms_decreases(O, eik, golden):
    """2D-improve.cc: the RMS error against the geodesic distance on the radius-100
    sphere decreases as the mesh is refined (64 vertices per block, 150 for the
    finest mesh, as in the reference test; the product's partitioner)."""
    rms = []
    for name, mvb in [("sphere_12verts", 64), ("sphere_74verts", 64), ("sphere_1154verts", 64),
                      ("sphere_4610verts", 150)]:
        xyz, faces = golden[name + "_xyz"], golden[name + "_faces"]
        e = eik.Eikonal(True)
        e.set_mesh(xyz, faces)
        e.maxVertsPerBlock_ = mvb
        e.prepare()
        lab, nb = e.getPartition()
        f, obt, off, vfv = e.triPrep()
        init = np.full(xyz.shape[0], 1e7, np.float32)
        init[0] = 0
        r = O.solve2d(xyz, f, np.ones(f.shape[0], np.float32), obt, off, vfv, lab, nb, [0], init)["result"]
        p0 = xyz[0].astype(np.float64)
        c = (xyz.astype(np.float64) @ p0) / np.linalg.norm(xyz, axis=1) / np.linalg.norm(p0)
        sol = 100.0 * np.arccos(np.clip(c, -1, 1))
        rms.append(np.sqrt(np.mean((sol - r) ** 2)))
    assert rms[0] > rms[1] > rms[2] > rms[3], rms


@pytest.mark.parametrize("case", ["cube9_64", "cube33_64", "cube65_64", "icosphere4_16", "grid33_16"])
def test_oracle_bisection_equals_the_products_partition(O, eik, mg, case):
    """The benchmark's reference arm and CPU baseline take their partition from the
    oracle's restatement of the default bisection, so that leg loads no product
    code; it must give the product's labels exactly."""
    if case.startswith("cube"):
        n, k = (int(x) for x in case[4:].split("_"))
        xyz, elems = mg.kuhn_cube(n, 0.2, seed=1)
        dim = 3
    elif case.startswith("icosphere"):
        xyz, elems = mg.icosphere(4)
        k, dim = 16, 2
    else:
        xyz, elems = mg.grid2d(33)
        k, dim = 16, 2
    e = eik.Eikonal(dim == 2)
    e.set_mesh(xyz, elems)
    e.maxVertsPerBlock_ = k
    e.prepare()
    lab, nb = e.getPartition()
    olab, onb = O.partition_rcb(xyz, k, dim)
    assert onb == nb
    assert np.array_equal(olab, lab)
