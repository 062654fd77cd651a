"""Parity of the GB300 CUDA path (through the C ABI) with the reference.

Two checkers:
  * the reference's own CUDA kernels (oracle/_ref/*.cubin, compiled from the
    reference tree) driven by a restatement of its host loop: results must be
    identical bit for bit, iteration counts and vertex-update counts equal;
  * the CPU restatement (oracle/fim_oracle.cpp): it rounds every product
    separately while the GPU fuses multiply-adds, and the scheme's 1e-5
    convergence threshold turns last-bit differences into different stopping
    points, so the CPU comparison carries a tolerance (stated per test).
Known answers and invariants come from the reference's gtests (src/test/2d,
src/test/3d).
"""
import numpy as np
import pytest

from conftest import bits_equal, relerr

pytestmark = pytest.mark.gpu


def need_ref(O):
    if O.ref_gpu() is None:
        pytest.skip("reference kernels (oracle/_ref/*.cubin) not present")


def solve3d(eik, xyz, tets, speeds=None, seeds=(0,), labels=None, **opts):
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    if speeds is not None:
        e.initSpeedMtxMultipliers(speeds)
    e.setSeeds(list(seeds))
    if labels is not None:
        e.setPartition(labels)
    for k, v in opts.items():
        setattr(e, k, v)
    e.solveEikonal()
    return e


def cube(mg, n):
    xyz, tets = mg.kuhn_cube(n, 0.2, seed=1)
    sp = mg.log_uniform_speeds(tets.shape[0], seed=2)
    return xyz, tets, (1.0 / sp.astype(np.float64) ** 2).astype(np.float32), mg.center_vertex(n)


# ---------------------------------------------------------------------------
# local updates
# ---------------------------------------------------------------------------
def test_tet_update_bitwise_vs_reference_kernel(need_gpu, eik, O):
    need_ref(O)
    rng = np.random.default_rng(11)
    n = 200000
    P = rng.normal(size=(n, 4, 3)).astype(np.float32) * np.exp(rng.uniform(-4, 4, (n, 1, 1))).astype(np.float32)
    T = (rng.uniform(0, 2, (n, 3)) * np.abs(P[:, :1, 0])).astype(np.float32)
    T[rng.random((n, 3)) < 0.15] = 1e9
    AC, BC, CD = P[:, 2] - P[:, 0], P[:, 2] - P[:, 1], P[:, 3] - P[:, 2]
    g = np.stack([(AC * AC).sum(1), (AC * BC).sum(1), (AC * CD).sum(1), (BC * BC).sum(1), (BC * CD).sum(1),
                  (CD * CD).sum(1)], 1).astype(np.float32)
    inp = np.concatenate([T, g], 1)
    assert bits_equal(eik.selftest_local_update(0, inp), O.ref_gpu_tet_local_solver(inp))


def _tet_block_cases(rng, mg, n):
    """Single-tet cases (TA TB TC TD and the six stored metric edge products):
    jittered-cube tets under scalar metrics with arrival times from a point source,
    random shapes and slivers under anisotropic metrics, and uniform random times;
    about a fifth of the times at LARGENUM (the wavefront's far side)."""
    def gram(P, M):
        def vmv(u, v):
            Mu = np.stack([u[:, 0] * M[:, 0] + u[:, 1] * M[:, 1] + u[:, 2] * M[:, 2],
                           u[:, 0] * M[:, 1] + u[:, 1] * M[:, 3] + u[:, 2] * M[:, 4],
                           u[:, 0] * M[:, 2] + u[:, 1] * M[:, 4] + u[:, 2] * M[:, 5]], 1)
            return (Mu * v).sum(1)
        A, B, C, D = P[:, 0], P[:, 1], P[:, 2], P[:, 3]
        return np.stack([vmv(C - A, C - B), vmv(C - B, D - C), vmv(C - A, D - C), vmv(D - A, D - B),
                         vmv(C - A, D - A), vmv(C - B, D - B)], 1).astype(np.float32)
    out = []
    xyz, tets = mg.kuhn_cube(13, 0.2, seed=31)
    P = xyz[tets[rng.integers(0, tets.shape[0], n)]].astype(np.float64)
    M = np.zeros((n, 6))
    M[:, 0] = M[:, 3] = M[:, 5] = np.exp(rng.uniform(np.log(0.25), np.log(4), n))
    src = rng.uniform(-0.5, 1.5, (n, 3))
    T = np.linalg.norm(P - src[:, None, :], axis=2) * np.sqrt(M[:, :1]) * (1 + rng.normal(0, 1e-3, (n, 4)))
    out.append(np.concatenate([T, gram(P, M)], 1))
    P = rng.normal(size=(n, 4, 3)) * np.exp(rng.uniform(-3, 3, (n, 1, 1)))
    fl = rng.random(n) < 0.3
    P[fl, 3] = P[fl, :3].mean(1) + rng.normal(0, 1e-3, (fl.sum(), 3)) * np.abs(P[fl, :1, 0])
    Q, _ = np.linalg.qr(rng.normal(size=(n, 3, 3)))
    ev = np.exp(rng.uniform(0, np.log(100), (n, 3)))
    Mf = np.einsum("nij,nj,nkj->nik", Q, ev, Q)
    M = np.stack([Mf[:, 0, 0], Mf[:, 0, 1], Mf[:, 0, 2], Mf[:, 1, 1], Mf[:, 1, 2], Mf[:, 2, 2]], 1)
    src = P[:, 0] + rng.normal(size=(n, 3)) * 4 * np.abs(P - P[:, :1]).max(axis=(1, 2))[:, None]
    d = P - src[:, None, :]
    T = np.sqrt(np.maximum(np.einsum("nvi,nij,nvj->nv", d, Mf, d), 0)) * (1 + rng.normal(0, 1e-2, (n, 4)))
    out.append(np.concatenate([T, gram(P, M)], 1))
    P = rng.normal(size=(n, 4, 3)) * np.exp(rng.uniform(-4, 4, (n, 1, 1)))
    T = rng.uniform(0, 2, (n, 4)) * np.abs(P[:, :1, 0])
    M = np.tile([1.0, 0, 0, 1, 0, 1], (n, 1))
    out.append(np.concatenate([T, gram(P, M)], 1))
    inp = np.concatenate(out, 0).astype(np.float32)
    inp[:, :4][rng.random((inp.shape[0], 4)) < 0.2] = np.float32(1e9)
    return inp


def test_tet_group_bitwise_vs_reference_fimcuda(need_gpu, eik, O, mg):
    """The four apex updates of a slot as the product's visit kernels run them
    (explicitly rounded, with the reference kernel's fused multiply-adds) against
    the reference's own FIMCuda on single-tet blocks, one sweep: every vertex ends
    at min(T_k, its apex update), bit for bit."""
    need_ref(O)
    inp = _tet_block_cases(np.random.default_rng(77), mg, 100000)
    want = O.ref_gpu_tet_blocks(inp)
    got = eik.selftest_local_update(6, inp)
    assert np.mean(want < inp[:, :4]) > 0.2  # a fair share of updates lower their vertex
    assert bits_equal(got, want)
    # the oracle's CPU model of the fused roundings, with the masks the product's
    # header states, reproduces the reference kernel too
    import os
    import re
    from conftest import ROOT
    text = open(os.path.join(ROOT, "sci-solver_eikonal_gb300", "csrc", "local_update.cuh")).read()
    masks = dict(re.findall(r"kFuseApex([ABCD]) = (0x[0-9a-fA-F]+)ull", text))
    assert sorted(masks) == ["A", "B", "C", "D"]
    model = O.tet_group_fused(inp, [int(masks[k], 16) for k in "ABCD"])
    assert bits_equal(model, want)


def test_fp32_quotients_equal_the_references_fp64_ones(need_gpu, eik):
    rng = np.random.default_rng(5)
    n = 500000
    num = (rng.normal(size=n) * 10.0 ** rng.uniform(-10, 4, n)).astype(np.float32)
    h = (rng.choice([-1, 1], n) * 10.0 ** rng.uniform(-11, 3, n)).astype(np.float32)
    h[:1000] = np.float32(-1e-8) * (1 + rng.normal(size=1000).astype(np.float32) * 1e-3)  # h + 1e-8 cancels
    h[1000:1100] = 0
    num[1100:1200] = 0
    q = eik.selftest_local_update(2, np.stack([num, h], 1))
    with np.errstate(all="ignore"):
        small = (num.astype(np.float64) / (h.astype(np.float64) + 0.00000001)).astype(np.float32)
        root = (num.astype(np.float64) / (2.0 * h.astype(np.float64))).astype(np.float32)
    assert bits_equal(q[:, 0], small)
    assert bits_equal(q[:, 1], root)


@pytest.mark.parametrize("check", [False, True])
def test_2d_kernels_bitwise_on_single_triangle_blocks(need_gpu, eik, O, check):
    """Each case is a triangle forming its own block, passed once through the 2D
    sweep kernel (7 sweeps) or the neighbour check (1 sweep) of the product and of
    the reference (FIMCuda / run_check_neighbor)."""
    need_ref(O)
    rng = np.random.default_rng(21 + int(check))
    n = 60000
    P = rng.normal(size=(n, 3, 3)).astype(np.float32)
    P[:, :, 2] *= 0.1
    e = np.stack([np.linalg.norm(P[:, 1] - P[:, 0], axis=1), np.linalg.norm(P[:, 2] - P[:, 1], axis=1),
                  np.linalg.norm(P[:, 0] - P[:, 2], axis=1)], 1).astype(np.float32)
    T = np.full((n, 3), 1e7, np.float32)
    k = rng.integers(0, 3, n)
    T[np.arange(n), k] = 0
    m2 = rng.random(n) < 0.5
    T[m2, ((k + 1) % 3)[m2]] = rng.uniform(0, 2, m2.sum()).astype(np.float32)
    F = np.exp(rng.uniform(np.log(0.5), np.log(2), n)).astype(np.float32)
    inp = np.concatenate([T, e, F[:, None]], 1).astype(np.float32)
    assert bits_equal(eik.selftest_local_update(4 if check else 3, inp), O.ref_gpu_tri_blocks(inp, check))


# ---------------------------------------------------------------------------
# 3D solves against the reference kernels
# ---------------------------------------------------------------------------
def _ref3d_cases(mg, golden):
    out = []
    for n in (9, 17, 33):
        xyz, tets, sp, seed = cube(mg, n)
        out.append((f"cube{n}", xyz, tets, sp, [seed], {}))
    out.append(("sphere334", golden["sphere334_xyz"], golden["sphere334_tets"], None, [0], {}))
    out.append(("torus_anisotropic", golden["torus_xyz"], golden["torus_tets"], golden["torus_metric"], [0], {}))
    out.append(("cube16_structured", golden["CubeMesh_size16_xyz"], golden["CubeMesh_size16_tets"], None, [0],
                {"isStructured_": 1, "squareBlockLength_": 4, "squareBlockWidth_": 4, "squareBlockDepth_": 4}))
    xyz, tets, sp, seed = cube(mg, 17)
    out.append(("cube17_three_seeds_16vpb", xyz, tets, sp, [0, seed, xyz.shape[0] - 1], {"maxVertsPerBlock_": 16}))
    out.append(("cube17_stop_after_3", xyz, tets, sp, [seed], {"maxIterations_": 3}))
    # the precision workload's shape in FP32: 10% sliver tets, anisotropic 6-entry metrics
    xyz, tets, _ = mg.sliver_cube(17, 0.10, seed=5)
    M6 = mg.anisotropic_metrics(tets.shape[0], seed=6).ravel()
    seeds = np.random.default_rng(9).choice(xyz.shape[0], 4, replace=False).tolist()
    out.append(("sliver17_anisotropic", xyz, tets, M6, seeds, {"maxIterations_": 1000}))
    # harder for the skip bounds: more slivers, anisotropy ratios up to 1e4
    xyz, tets, _ = mg.sliver_cube(13, 0.25, seed=11)
    M6 = mg.anisotropic_metrics(tets.shape[0], seed=12, lo=1.0, hi=1e4).ravel()
    seeds = np.random.default_rng(13).choice(xyz.shape[0], 3, replace=False).tolist()
    out.append(("sliver13_strongly_anisotropic", xyz, tets, M6, seeds, {"maxIterations_": 1000}))
    return out


@pytest.mark.parametrize("idx", range(10))
def test_3d_bitwise_vs_reference_kernels(need_gpu, eik, O, mg, golden, idx):
    need_ref(O)
    name, xyz, tets, sp, seeds, opts = _ref3d_cases(mg, golden)[idx]
    e = solve3d(eik, xyz, tets, sp, seeds, **opts)
    got = e.getFinalResult()
    lab, nb = e.getPartition()
    M = O.metrics_from_speeds(tets.shape[0], sp)
    r = O.ref_gpu_solve3d(xyz, tets, M, lab, nb, seeds, max_iters=e.maxIterations_, history=True)
    st = e.stats()
    assert e.numIterations() == r["iterations"], name
    assert st["vertex_updates"] == r["vertex_updates"], name
    assert bits_equal(got, r["result"]), (name, relerr(got, r["result"]).max())
    for i in range(r["iterations"]):
        assert bits_equal(e.getResultAtIteration(i), r["history"][i]), (name, i)


@pytest.mark.parametrize("cap", [1, 2, 5, 11, 19])
def test_3d_iteration_cap_vs_reference_kernels(need_gpu, eik, O, mg, cap):
    """Solves cut off by maxIterations_: the reference's loop runs the neighbour
    checks of its last iteration before it stops (meshFIM3dEikonal.cu:411-542), which
    the product runs in one more sweep launch that sweeps nothing; iteration count,
    vertex-update count and bits equal the reference kernels' at every cap."""
    need_ref(O)
    xyz, tets, sp, seed = cube(mg, 17)
    e = solve3d(eik, xyz, tets, sp, [seed], maxIterations_=cap, maxVertsPerBlock_=32)
    lab, nb = e.getPartition()
    M = O.metrics_from_speeds(tets.shape[0], sp)
    r = O.ref_gpu_solve3d(xyz, tets, M, lab, nb, [seed], max_iters=cap)
    assert e.numIterations() == r["iterations"] <= cap
    assert e.stats()["vertex_updates"] == r["vertex_updates"]
    assert bits_equal(e.getFinalResult(), r["result"])


def test_3d_against_reference_kernel_fixtures(need_gpu, eik, ref_outputs):
    """Travel times the reference's kernels produced on the GPU machine
    (tests/golden/ref_gpu_outputs.npz), reproduced through the C ABI."""
    import importlib.util
    import os
    from conftest import GOLDEN
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
    make_golden = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(make_golden)
    for name, dim, xyz, el, sp, lab, nb, seeds in make_golden.ref_gpu_cases():
        if dim != 3:
            continue
        e = solve3d(eik, xyz, el, sp, seeds, labels=lab)
        assert e.numIterations() == int(ref_outputs[name + "_iterations"]), name
        assert bits_equal(e.getFinalResult(), ref_outputs[name + "_result"]), name


def test_3d_against_cpu_oracle(need_gpu, eik, O, mg, golden):
    # the 8/13-tet balls take identical paths on CPU and GPU: bitwise
    for name in ("sphere8", "sphere13"):
        xyz, tets = golden[name + "_xyz"], golden[name + "_tets"]
        e = solve3d(eik, xyz, tets)
        lab, nb = e.getPartition()
        r = O.solve3d(xyz, tets, O.metrics_from_speeds(tets.shape[0], None), lab, nb, [0])
        assert bits_equal(e.getFinalResult(), r["result"])
    # jittered cubes: the CPU rounds every product separately and the GPU (like the
    # reference build) fuses multiply-adds.  A last-bit difference can move a
    # block's 1e-5 stopping decision, and the reference's FP32 tet update is
    # ill-conditioned when a nearly planar front crosses a small tet, where one
    # rounding can move a candidate by percents (the FP32 GPU result, reference and
    # product alike, differs there from both the CPU FP32 and the FP64 runs).
    # Stated tolerance: 90% of the vertices within 1e-5 relative, all within 5%.
    for n in (9, 17):
        xyz, tets, sp, seed = cube(mg, n)
        e = solve3d(eik, xyz, tets, sp, [seed])
        lab, nb = e.getPartition()
        r = O.solve3d(xyz, tets, O.metrics_from_speeds(tets.shape[0], sp), lab, nb, [seed])
        rel = relerr(e.getFinalResult(), r["result"])
        print(f"cube{n}: iterations gpu {e.numIterations()} cpu {r['iterations']}, "
              f"within 1e-5: {np.mean(rel < 1e-5):.4f}, max rel {rel.max():.2e}")
        assert abs(e.numIterations() - r["iterations"]) <= 2
        assert np.mean(rel < 1e-5) >= 0.90
        assert rel.max() < 0.05


def test_3d_fp64_oracle_error_is_stated(need_gpu, eik, O, mg):
    """Error of the FP32 result against the FP64 run of the same scheme (same
    partition): median below 1e-5 relative; isolated vertices carry the FP32
    conditioning error of the reference's tet update (below 5%)."""
    xyz, tets, sp, seed = cube(mg, 17)
    e = solve3d(eik, xyz, tets, sp, [seed])
    lab, nb = e.getPartition()
    r64 = O.solve3d(xyz, tets, O.metrics_from_speeds(tets.shape[0], sp), lab, nb, [seed], precision=64)
    rel = relerr(e.getFinalResult(), r64["result"], 1e-3)
    print(f"FP64-oracle error: median {np.median(rel):.2e} p99 {np.percentile(rel, 99):.2e} max {rel.max():.2e}")
    assert np.median(rel) < 1e-5
    assert rel.max() < 0.05


# ---------------------------------------------------------------------------
# reference tests (src/test/3d) through the product
# ---------------------------------------------------------------------------
def test_small3d_known_answers(need_gpu, eik, golden):
    """3D-small.cc"""
    for name, tol in (("sphere8", None), ("sphere13", 1e-4)):
        e = eik.Eikonal(False)
        e.set_mesh(golden[name + "_xyz"], golden[name + "_tets"])
        e.maxBlocks_ = 100
        e.solveEikonal()
        r = e.getFinalResult()
        assert abs(r[0]) <= 1e-4
        if tol is None:
            assert np.all(np.abs(r[1:] - np.float32(19.58)) <= 4 * np.spacing(np.float32(19.58)))
        else:
            assert np.all(np.abs(r[1:] - 19.58) <= tol)


def test_basic3d_and_converge3d(need_gpu, eik, golden):
    """3D-basic.cc: every vertex reached; 3D-converge.cc: values never increase."""
    for name, structured in (("sphere334", False), ("CubeMesh_size16", True)):
        e = eik.Eikonal(False)
        e.set_mesh(golden[name + "_xyz"], golden[name + "_tets"])
        e.isStructured_ = int(structured)
        e.solveEikonal()
        assert np.all(e.getFinalResult() < 100)
        for i in range(2, e.numIterations()):
            one, zero = e.getResultAtIteration(i - 1), e.getResultAtIteration(i)
            m = one != 0
            assert np.all(zero[m] <= one[m])


def test_improve3d_rms_non_increasing(need_gpu, eik, golden):
    """3D-improve.cc uses sphere334/8092/19499; the committed fixtures hold the
    smaller balls, refined here by the 16^3 cube as a second family."""
    xyz, tets = golden["sphere334_xyz"], golden["sphere334_tets"]
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.solveEikonal()
    sol = np.linalg.norm(xyz - np.array([54, 54, 54], np.float32), axis=1)
    assert np.sqrt(np.mean((sol - e.getFinalResult()) ** 2)) < 5.0


# ---------------------------------------------------------------------------
# full size
# ---------------------------------------------------------------------------
def test_c3d_full_size(need_gpu, eik, O, mg):
    xyz, tets, sp, seed = cube(mg, 65)
    e = solve3d(eik, xyz, tets, sp, [seed], maxVertsPerBlock_=64, keepHistory_=0)
    got = e.getFinalResult()
    assert e.numIterations() < e.maxIterations_  # converged, not cut off
    assert got[seed] == 0 and np.all(np.isfinite(got)) and np.all(got > 0 - 1e-7)
    assert np.all(got[np.arange(got.size) != seed] > 0)
    st = e.stats()
    assert st["num_blocks"] == 4292 and st["device_error"] == 0
    # a second solve on the resident data gives the same bits
    e.solveEikonal()
    assert bits_equal(e.getFinalResult(), got)
    if O.ref_gpu() is not None:
        lab, nb = e.getPartition()
        r = O.ref_gpu_solve3d(xyz, tets, O.metrics_from_speeds(tets.shape[0], sp), lab, nb, [seed])
        assert bits_equal(got, r["result"]) and r["iterations"] == e.numIterations()


# ---------------------------------------------------------------------------
# API behaviour
# ---------------------------------------------------------------------------
def test_initial_values_equal_seed_list(need_gpu, eik, mg):
    xyz, tets, sp, seed = cube(mg, 13)
    seeds = [0, seed, 100]
    a = solve3d(eik, xyz, tets, sp, seeds)
    b = eik.Eikonal(False)
    b.set_mesh(xyz, tets)
    b.initSpeedMtxMultipliers(sp)
    init = np.full(xyz.shape[0], 5.0, np.float32)
    init[seeds] = 0
    b.initializeVertices(init)
    b.solveEikonal()
    assert bits_equal(a.getFinalResult(), b.getFinalResult())


def test_resolve_after_speed_change_matches_fresh_handle(need_gpu, eik, mg):
    xyz, tets, sp, seed = cube(mg, 13)
    e = solve3d(eik, xyz, tets, sp, [seed])
    sp2 = (sp * np.float32(1.7)).astype(np.float32)
    e.initSpeedMtxMultipliers(sp2)
    e.solveEikonal()
    f = solve3d(eik, xyz, tets, sp2, [seed])
    assert bits_equal(e.getFinalResult(), f.getFinalResult())
    # a 6-entry metric equal to s*I gives the same answer as the scalar form
    M6 = np.zeros((tets.shape[0], 6), np.float32)
    M6[:, 0] = M6[:, 3] = M6[:, 5] = sp2
    g = solve3d(eik, xyz, tets, M6.ravel(), [seed])
    assert bits_equal(g.getFinalResult(), f.getFinalResult())


def test_direct_launch_matches_graph_launch(need_gpu, eik, mg):
    """The kernel-by-kernel mode (for profilers) computes exactly what the single
    graph launch computes, in 3D and 2D."""
    xyz, tets, sp, seed = cube(mg, 17)
    a = solve3d(eik, xyz, tets, sp, [seed])
    b = solve3d(eik, xyz, tets, sp, [seed], directLaunch_=1)
    assert a.numIterations() == b.numIterations()
    assert bits_equal(a.getFinalResult(), b.getFinalResult())
    assert a.stats()["vertex_updates"] == b.stats()["vertex_updates"]
    xyz2, f2 = mg.icosphere(4)
    res = []
    for direct in (0, 1):
        e = eik.Eikonal(True)
        e.set_mesh(xyz2, f2)
        e.initSpeedMtxMultipliers(mg.batch_speed(xyz2, f2))
        e.maxVertsPerBlock_ = 32
        e.directLaunch_ = direct
        e.solveEikonal()
        res.append((e.numIterations(), e.getFinalResult()))
    assert res[0][0] == res[1][0] and bits_equal(res[0][1], res[1][1])


@pytest.mark.parametrize("dim", [3, 2])
def test_loop_body_copies_stop_where_the_direct_loop_stops(need_gpu, eik, mg, dim):
    """The graph's loop body runs four outer iterations a pass; the kernel-by-kernel
    loop checks the stop flag after each one.  Iteration caps at every position
    within a pass, and the uncapped solve, give the same iterations, updates and bits
    in both."""
    if dim == 3:
        xyz, elems, sp, seed = cube(mg, 17)
        speed, seeds = sp, [seed]
    else:
        xyz, elems = mg.icosphere(4)
        speed, seeds = mg.batch_speed(xyz, elems), [0]
    for cap in (1, 2, 3, 4, 5, 6, 7, 1000):
        res = []
        for direct in (0, 1):
            e = eik.Eikonal(dim == 2)
            e.set_mesh(xyz, elems)
            e.initSpeedMtxMultipliers(speed)
            e.setSeeds(seeds)
            e.maxVertsPerBlock_ = 32
            e.maxIterations_ = cap
            e.directLaunch_ = direct
            e.solveEikonal()
            res.append(e)
        g, d = res
        assert g.numIterations() == d.numIterations() == min(cap, d.numIterations())
        assert g.stats()["vertex_updates"] == d.stats()["vertex_updates"]
        assert bits_equal(g.getFinalResult(), d.getFinalResult())
    assert d.numIterations() > 4  # the uncapped solve ends on its own, after the first pass


def test_write_vtk(need_gpu, eik, golden, tmp_path):
    e = eik.Eikonal(False)
    e.set_mesh(golden["sphere334_xyz"], golden["sphere334_tets"])
    e.solveEikonal()
    e.writeVTK(False, prefix=str(tmp_path / "result"))
    lines = open(tmp_path / "result0.vtk").read().splitlines()
    assert lines[3] == "DATASET UNSTRUCTURED_GRID" and lines[4] == "POINTS 334 float"
    i = lines.index("LOOKUP_TABLE default")
    vals = np.array([float(x) for x in lines[i + 1:i + 335]], np.float32)
    assert np.allclose(vals, e.getFinalResult(), rtol=1e-6, atol=1e-6)


# ---------------------------------------------------------------------------
# 2D
# ---------------------------------------------------------------------------
def _tri_ref(eik, O, e, xyz, speeds, seeds, init=None, max_iters=100):
    f, obt, off, vfv = e.triPrep()
    lab, nb = e.getPartition()
    if init is None:
        init = np.full(xyz.shape[0], 1e7, np.float32)
        init[list(seeds)] = 0
    sinv = np.ones(f.shape[0], np.float32) if speeds is None else (np.float32(1) / speeds).astype(np.float32)
    return O.ref_gpu_solve2d(xyz, f, sinv, obt, off, vfv, lab, nb, list(seeds), init, max_iters=max_iters,
                             history=True)


def _cases2d(mg, golden):
    xyz, f = mg.grid2d(33)
    out = [("grid33_16vpb", xyz, f, None, [0], {"maxVertsPerBlock_": 16})]
    # 2D blocks stay at or below 64 vertices: the reference keeps 64 flag slots per
    # block and blocks above that overwrite their neighbour's flags
    for lvl, mvb in ((3, 16), (4, 32), (5, 32)):
        xyz, f = mg.icosphere(lvl)
        out.append((f"ico{lvl}", xyz, f, mg.batch_speed(xyz, f), [0, 7], {"maxVertsPerBlock_": mvb}))
    out.append(("sphere74", golden["sphere_74verts_xyz"], golden["sphere_74verts_faces"], None, [0], {}))
    out.append(("sphere1154", golden["sphere_1154verts_xyz"], golden["sphere_1154verts_faces"], None, [0],
                {"maxVertsPerBlock_": 32}))
    # obtuse corners (3,072 virtual faces) under heterogeneous face speeds: the
    # virtual faces keep inverse speed 1 (the reference's speed type ONE), the real
    # faces carry 1/speed
    xyz, f = golden["sphere_1154verts_xyz"], golden["sphere_1154verts_faces"]
    out.append(("sphere1154_speed", xyz, f, mg.batch_speed(xyz, f), [0, 500], {"maxVertsPerBlock_": 32}))
    out.append(("square16_structured", golden["SquareMesh_size16_xyz"], golden["SquareMesh_size16_faces"], None,
                [0], {"isStructured_": 1, "squareBlockLength_": 4, "squareBlockWidth_": 4}))
    return out


@pytest.mark.parametrize("idx", range(8))
def test_2d_vs_reference_kernels(need_gpu, eik, O, mg, golden, idx):
    need_ref(O)
    name, xyz, f, sp, seeds, opts = _cases2d(mg, golden)[idx]
    e = eik.Eikonal(True)
    e.set_mesh(xyz, f)
    if sp is not None:
        e.initSpeedMtxMultipliers(sp)
    e.setSeeds(seeds)
    for k, v in opts.items():
        setattr(e, k, v)
    e.solveEikonal()
    r = _tri_ref(eik, O, e, xyz, sp, seeds)
    got = e.getFinalResult()
    assert e.numIterations() == r["iterations"], name
    assert e.stats()["vertex_updates"] == r["vertex_updates"], name
    assert bits_equal(got, r["result"]), (name, relerr(got, r["result"]).max())


def test_basic2d_improve2d(need_gpu, eik, golden):
    """2D-basic.cc (everything reached below the stop distance) and 2D-improve.cc
    (RMS error to the geodesic decreases with refinement)."""
    rms = []
    for name, mvb in (("sphere_12verts", 64), ("sphere_74verts", 64), ("sphere_1154verts", 64),
                      ("sphere_4610verts", 150)):
        xyz, faces = golden[name + "_xyz"], golden[name + "_faces"]
        e = eik.Eikonal(True)
        e.set_mesh(xyz, faces)
        e.maxVertsPerBlock_ = mvb
        e.solveEikonal()
        r = e.getFinalResult()
        assert np.all(r < 700)
        p0 = xyz[0].astype(np.float64)
        c = (xyz.astype(np.float64) @ p0) / np.linalg.norm(xyz, axis=1) / np.linalg.norm(p0)
        rms.append(np.sqrt(np.mean((100.0 * np.arccos(np.clip(c, -1, 1)) - r) ** 2)))
    assert rms[0] > rms[1] > rms[2] > rms[3], rms


def test_2d_grid_against_cpu_oracle_and_distance(need_gpu, eik, O, mg):
    xyz, f = mg.grid2d(33)
    e = eik.Eikonal(True)
    e.set_mesh(xyz, f)
    e.maxVertsPerBlock_ = 16
    e.solveEikonal()
    got = e.getFinalResult()
    lab, nb = e.getPartition()
    ff, obt, off, vfv = e.triPrep()
    init = np.full(xyz.shape[0], 1e7, np.float32)
    init[0] = 0
    r = O.solve2d(xyz, ff, np.ones(ff.shape[0], np.float32), obt, off, vfv, lab, nb, [0], init)
    assert relerr(got, r["result"]).max() < 1e-5
    r64 = O.solve2d(xyz, ff, np.ones(ff.shape[0], np.float32), obt, off, vfv, lab, nb, [0], init, precision=64)
    assert relerr(got, r64["result"]).max() < 1e-5
    d = np.linalg.norm(xyz.astype(np.float64), axis=1)
    assert relerr(got, d, 1e-3).max() < 0.05


@pytest.mark.parametrize("dim", [2, 3])
def test_metis_partition_solves_bitwise_like_the_reference_kernels(need_gpu, eik, mg, O, dim):
    """With partitioner = METIS (the reference's partitioner kind) the solve still
    equals the reference's kernels on the same labels, bit for bit."""
    need_ref(O)
    if dim == 3:
        xyz, tets, M, seed = cube(mg, 17)
        e = eik.Eikonal(False)
        e.set_mesh(xyz, tets)
        e.initSpeedMtxMultipliers(M)
        e.setSeeds([seed])
        e.partitioner_ = eik.PARTITION_METIS
        e.solveEikonal()
        lab, nb = e.getPartition()
        r = O.ref_gpu_solve3d(xyz, tets, O.metrics_from_speeds(tets.shape[0], M), lab, nb, [seed])
        assert bits_equal(e.getFinalResult(), r["result"]) and r["iterations"] == e.numIterations()
    else:
        xyz, f = mg.icosphere(4)
        e = eik.Eikonal(True)
        e.set_mesh(xyz, f)
        e.setSeeds([0])
        e.maxVertsPerBlock_ = 32
        e.partitioner_ = eik.PARTITION_METIS
        e.solveEikonal()
        r = _tri_ref(eik, O, e, xyz, None, [0])
        assert bits_equal(e.getFinalResult(), r["result"]) and r["iterations"] == e.numIterations()


def test_serving_pool_97_bitwise_vs_reference_kernels(need_gpu, eik, O, mg):
    """The serving pool's largest mesh (97^3 jittered Kuhn cube, 912,673 vertices,
    5,308,416 tets, its pool speeds) with a request's 16 seeds and speed scale, solved
    on its own: bits, iterations and vertex updates equal the reference kernels'
    (served results equal this solve, test_gpu_serve.py)."""
    need_ref(O)
    xyz, tets = mg.kuhn_cube(97, 0.2, seed=23)
    v = mg.log_uniform_speeds(tets.shape[0], 0.5, 2.0, seed=33)
    scale = np.float32(1.37)
    metric = ((1.0 / (v.astype(np.float64) ** 2)).astype(np.float32) * np.float32(1.0 / (scale * scale))).astype(
        np.float32)
    seeds = np.random.default_rng(97).choice(xyz.shape[0], 16, replace=False).tolist()
    e = solve3d(eik, xyz, tets, metric, seeds, maxVertsPerBlock_=64, maxIterations_=1000, keepHistory_=0)
    lab, nb = e.getPartition()
    r = O.ref_gpu_solve3d(xyz, tets, O.metrics_from_speeds(tets.shape[0], metric), lab, nb, seeds, max_iters=1000)
    assert e.numIterations() == r["iterations"] < 1000
    assert e.stats()["vertex_updates"] == r["vertex_updates"]
    assert bits_equal(e.getFinalResult(), r["result"])


def test_precision_workload_fp32_bitwise_vs_reference_kernels(need_gpu, eik, O, mg):
    """The precision workload at full size (49^3 jittered cube with 10% sliver tets,
    anisotropic metrics, 4 seeds) in the FP32 mode: bits, iterations and vertex
    updates equal the reference kernels' (the mixed mode departs from them on
    purpose and is held to the FP64 run instead, test_gpu_precision.py)."""
    need_ref(O)
    xyz, tets, _ = mg.sliver_cube(49, 0.10, seed=5)
    M6 = mg.anisotropic_metrics(tets.shape[0], seed=6).ravel()
    seeds = np.random.Generator(np.random.PCG64(9)).choice(xyz.shape[0], 4, replace=False).tolist()
    e = solve3d(eik, xyz, tets, M6, seeds, maxIterations_=1000, keepHistory_=0)
    lab, nb = e.getPartition()
    r = O.ref_gpu_solve3d(xyz, tets, O.metrics_from_speeds(tets.shape[0], M6), lab, nb, seeds, max_iters=1000)
    assert e.numIterations() == r["iterations"] < 1000
    assert e.stats()["vertex_updates"] == r["vertex_updates"]
    assert bits_equal(e.getFinalResult(), r["result"])
