"""The C ABI without a GPU: the library loads, exports every declared entry point,
validates its inputs, runs the host half of a solve (partition, layout) and fails
loudly, with a status code, when no GPU is available."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT, gpu_available

HEADER = os.path.join(ROOT, "include", "eikonal_gb300.h")


def declared_symbols():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(eik_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(eik):
    lib = ctypes.CDLL(eik.LIB_PATH)
    syms = declared_symbols()
    assert len(syms) >= 25
    for s in syms:
        assert hasattr(lib, s), s
    # the Python binding declares the same set
    assert set(syms) == set(eik.SIGNATURES), set(syms) ^ set(eik.SIGNATURES)


def test_default_options_are_the_references(eik):
    o = eik.EikOptions()
    eik.lib().eik_default_options(ctypes.byref(o))
    # src/Eikonal.cu:4-24
    assert (o.max_blocks, o.max_verts_per_block, o.stop_distance, o.is_structured, o.speed_type) == (16, 64, 50000.0, 0, 1)
    assert (o.square_length, o.square_width, o.square_depth) == (16, 16, 16)
    assert (o.square_block_length, o.square_block_width, o.square_block_depth) == (1, 1, 1)
    assert o.max_iterations == 100
    # options of this build beside the reference's: telemetry on, checked values
    assert o.telemetry == 1
    e = eik.Eikonal(False)
    o2 = eik.EikOptions()
    e._check(e._lib.eik_get_options(e._h, ctypes.byref(o2)))
    o2.telemetry = 0
    e._check(e._lib.eik_set_options(e._h, ctypes.byref(o2)))
    o3 = eik.EikOptions()
    e._check(e._lib.eik_get_options(e._h, ctypes.byref(o3)))
    assert o3.telemetry == 0
    o2.telemetry = 2
    assert e._lib.eik_set_options(e._h, ctypes.byref(o2)) == 1  # EIK_ERR_ARG


def test_error_codes(eik, mg, tmp_path):
    E = eik
    e = E.Eikonal(False)
    with pytest.raises(E.EikonalError) as ex:  # solve before a mesh
        e._check(e._lib.eik_solve(e._h))
    assert ex.value.code == 2
    with pytest.raises(E.EikonalError) as ex:  # initializeVertices before the mesh (reference: exit(0))
        e.initializeVertices(np.zeros(3, np.float32))
    assert ex.value.code == 2
    xyz, tets = mg.kuhn_cube(3, 0.0)
    with pytest.raises(E.EikonalError) as ex:  # indices start at 2
        e.set_mesh(xyz, tets + 2)
    assert ex.value.code == 3
    e.set_mesh(xyz, tets + 1)  # 1-based indices are accepted (tetmesh.cu:42-49)
    with pytest.raises(E.EikonalError) as ex:  # size mismatch
        e.initializeVertices(np.zeros(xyz.shape[0] + 1, np.float32))
    assert ex.value.code == 1
    with pytest.raises(E.EikonalError) as ex:
        e.setSeeds([xyz.shape[0]])
    assert ex.value.code == 1
    e.maxVertsPerBlock_ = 0
    with pytest.raises(E.EikonalError) as ex:
        e.prepare()
    assert ex.value.code == 1
    # unreadable mesh file: the reference exits with status 1 (2D-sanity.cc, 3D-sanity.cc)
    bad = E.Eikonal(True)
    bad.filename_ = str(tmp_path / "nope.ply")
    with pytest.raises(E.EikonalError) as ex:
        bad.initializeMesh()
    assert ex.value.code == 3
    bad3 = E.Eikonal(False)
    bad3.filename_ = str(tmp_path / "nope")
    with pytest.raises(E.EikonalError) as ex:
        bad3.initializeMesh()
    assert ex.value.code == 3


@pytest.mark.skipif(gpu_available(), reason="checks the no-GPU failure path")
def test_solve_without_gpu_fails_loudly(eik, mg):
    xyz, tets = mg.kuhn_cube(4, 0.0)
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    with pytest.raises(eik.EikonalError) as ex:
        e.solveEikonal()
    assert ex.value.code == 4


@pytest.mark.parametrize("dim,nv,k,want", [(2, 1089, 16, 68), (3, 274625, 64, 4292), (2, 10, 64, 2), (3, 7, 64, 2)])
def test_block_count_rule(eik, mg, dim, nv, k, want):
    """METIS wrapper rules: 2D floor(nv/k), 3D ceil(nv/k), at least 2
    (meshFIM2d_eikonal.cu:119-121, meshFIM3dEikonal.cu:160-163)."""
    if dim == 2:
        n = int(round(nv ** 0.5))
        xyz, el = mg.grid2d(n) if n * n == nv else (np.random.default_rng(0).random((nv, 3)).astype(np.float32),
                                                    np.array([[0, 1, 2], [1, 2, 3], [2, 3, 4], [3, 4, 5], [4, 5, 6],
                                                              [5, 6, 7], [6, 7, 8], [7, 8, 9]], np.int32))
    else:
        n = int(round(nv ** (1 / 3)))
        if n ** 3 == nv:
            xyz, el = mg.kuhn_cube(n, 0.2)
        else:
            g = np.load(os.path.join(ROOT, "tests", "golden", "meshes.npz"))
            xyz, el = g["sphere8_xyz"], g["sphere8_tets"]
    e = eik.Eikonal(dim == 2)
    e.set_mesh(xyz, el)
    e.maxVertsPerBlock_ = k
    e.prepare()
    lab, nb = e.getPartition()
    assert nb == want == e.maxBlocks_
    sizes = np.bincount(lab, minlength=nb)
    assert sizes.max() - sizes.min() <= 1  # recursive bisection keeps blocks balanced
    st = e.stats()
    assert st["iterations"] == 0


def test_structured_partition_matches_reference_formula(eik, golden):
    """GraphPartition_Square (meshFIM3dEikonal.cu:239-283) on the 16^3 CubeMesh."""
    xyz, tets = golden["CubeMesh_size16_xyz"], golden["CubeMesh_size16_tets"]
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.isStructured_ = 1
    e.squareBlockLength_ = e.squareBlockWidth_ = e.squareBlockDepth_ = 4
    e.prepare()
    lab, nb = e.getPartition()
    assert nb == 64 == e.maxBlocks_
    idx = np.arange(4096)
    j, i, k = idx % 16, (idx // 16) % 16, idx // 256
    want = (k // 4) * 16 + (i // 4) * 4 + (j // 4)
    assert np.array_equal(lab, want)


def test_file_readers_match_arrays(eik, golden, tmp_path):
    xyz, tets = golden["sphere334_xyz"], golden["sphere334_tets"]
    base = tmp_path / "ball"
    with open(str(base) + ".node", "w") as f:
        f.write(f"{xyz.shape[0]} 3 0 0\n")
        for i, p in enumerate(xyz):
            f.write(f"{i + 1} {float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
    with open(str(base) + ".ele", "w") as f:
        f.write(f"{tets.shape[0]} 4 0\n# comment line\n")
        for i, t in enumerate(tets):
            f.write(f"{i + 1} {t[0] + 1} {t[1] + 1} {t[2] + 1} {t[3] + 1}\n")
    a = eik.Eikonal(False)
    a.filename_ = str(base)
    a.initializeMesh()
    a.prepare()
    b = eik.Eikonal(False)
    b.set_mesh(xyz, tets)
    b.prepare()
    assert a.numVertices() == b.numVertices() == xyz.shape[0]
    assert np.array_equal(a.getPartition()[0], b.getPartition()[0])
    xyz2, faces = golden["sphere_74verts_xyz"], golden["sphere_74verts_faces"]
    ply = tmp_path / "s.ply"
    with open(ply, "w") as f:
        f.write(f"ply\nformat ascii 1.0\nelement vertex {xyz2.shape[0]}\nproperty float x\nproperty float y\n"
                f"property float z\nelement face {faces.shape[0]}\nproperty list uchar int vertex_indices\nend_header\n")
        for p in xyz2:
            f.write(f"{float(p[0])!r} {float(p[1])!r} {float(p[2])!r}\n")
        for t in faces:
            f.write(f"3 {t[0]} {t[1]} {t[2]}\n")
    c = eik.Eikonal(True)
    c.filename_ = str(ply)
    c.initializeMesh()
    d = eik.Eikonal(True)
    d.set_mesh(xyz2, faces)
    fc, oc, vc, wc = c.triPrep()
    fd, od, vd, wd = d.triPrep()
    assert np.array_equal(fc, fd) and np.array_equal(oc, od) and np.array_equal(wc, wd)


def test_batch_rejects_mixed_dimensions_and_empty(eik, mg):
    xyz, faces = mg.icosphere(1)
    a = eik.Eikonal(True)
    a.set_mesh(xyz, faces)
    xyz3, tets = mg.kuhn_cube(5, 0.2, seed=1)
    c = eik.Eikonal(False)
    c.set_mesh(xyz3, tets)
    with pytest.raises(eik.EikonalError):
        eik.EikonalBatch([a, c])
    with pytest.raises(ValueError):
        eik.EikonalBatch([])
    b = eik.EikonalBatch([a, a])
    assert len(b) == 2 and b.numIterations(0) == 0
    with pytest.raises(eik.EikonalError):
        b.getFinalResult(0)  # nothing solved yet


def test_server_host_side_and_no_gpu_failure(eik, mg):
    xyz, faces = mg.icosphere(2)
    a = eik.Eikonal(True)
    a.set_mesh(xyz, faces)
    if not gpu_available():
        # a handle that builds its layout on the device needs the GPU already
        srv = eik.EikonalServer(hbm_budget_bytes=1 << 26)
        with pytest.raises(eik.EikonalError):
            srv.add_mesh(a)
        srv.close()
    a.deviceSetup_ = 0  # host build: adding a mesh is host work
    srv = eik.EikonalServer(hbm_budget_bytes=1 << 26)
    mid = srv.add_mesh(a)
    info = srv.mesh_info(mid)
    assert info["vertices"] == xyz.shape[0] and info["device_bytes"] > 4 * xyz.shape[0]
    with pytest.raises(eik.EikonalError):
        srv.submit(mid, [0], 1.0)  # not started
    if not gpu_available():
        with pytest.raises(eik.EikonalError):
            srv.start()  # no device: fails loudly, no CPU fallback
    srv.close()


def test_invalid_speeds_and_metrics_are_rejected(eik, mg):
    """Host-side fault injection: values the scheme cannot use fail with
    EIK_ERR_ARG before any setup or GPU work."""
    xyz, tets = mg.kuhn_cube(5, 0.2, seed=1)
    nt = tets.shape[0]
    bad = [np.full(nt, -1.0, np.float32), np.full(nt, np.nan, np.float32), np.zeros(nt, np.float32)]
    m6 = np.tile(np.array([1, 0, 0, 1, 0, 1], np.float32), nt)
    m6_bad = m6.copy()
    m6_bad[6 * 3 + 1] = np.nan
    bad.append(m6_bad)
    # an indefinite 6-entry metric is accepted, as the reference's torus fixture needs
    m6_indef = m6.copy()
    m6_indef[6 * 3 + 1] = 2.0
    for vals in bad:
        e = eik.Eikonal(False)
        e.set_mesh(xyz, tets)
        e.initSpeedMtxMultipliers(vals)
        with pytest.raises(eik.EikonalError) as ei:
            e.prepare()
        assert ei.value.code == 1
    for vals in (m6, m6_indef):
        ok = eik.Eikonal(False)
        ok.set_mesh(xyz, tets)
        ok.initSpeedMtxMultipliers(vals)
        ok.prepare()
    fx, faces = mg.grid2d(5)
    t = eik.Eikonal(True)
    t.set_mesh(fx, faces)
    sp = np.ones(faces.shape[0], np.float32)
    sp[2] = np.inf
    t.initSpeedMtxMultipliers(sp)
    with pytest.raises(eik.EikonalError):
        t.prepare()


def test_server_rejects_pool_over_budget(eik, mg):
    xyz, faces = mg.icosphere(3)
    a = eik.Eikonal(True)
    a.set_mesh(xyz, faces)
    a.deviceSetup_ = 0  # host build: the budget check needs no GPU
    srv = eik.EikonalServer(hbm_budget_bytes=1000)
    srv.add_mesh(a)
    with pytest.raises(eik.EikonalError) as ei:
        srv.start()  # fails on the budget before touching a GPU
    assert ei.value.code == 5 and "budget" in str(ei.value)
    srv.close()


@pytest.mark.parametrize("dim", [2, 3])
def test_metis_partition(eik, mg, dim):
    """partitioner = METIS: k-way on the vertex graph (METIS 5 from the CUDA toolkit,
    the reference's partitioner kind).  Every vertex labelled, no empty block, about
    the reference's block count, connected blocks dominate, same labels every time."""
    if dim == 2:
        xyz, el = mg.grid2d(33)
        k = 16
    else:
        xyz, el = mg.kuhn_cube(17, 0.2, seed=3)
        k = 64
    labs = []
    for _ in range(2):
        e = eik.Eikonal(dim == 2)
        e.set_mesh(xyz, el)
        e.maxVertsPerBlock_ = k
        e.partitioner_ = eik.PARTITION_METIS
        e.prepare()
        lab, nb = e.getPartition()
        labs.append(lab.copy())
        want = xyz.shape[0] // k if dim == 2 else -(-xyz.shape[0] // k)
        assert 0.9 * want <= nb <= want and nb == e.maxBlocks_
        sizes = np.bincount(lab, minlength=nb)
        assert sizes.min() > 0 and lab.min() == 0 and lab.max() == nb - 1
        assert sizes.max() <= 1.2 * xyz.shape[0] / nb  # METIS keeps parts within its imbalance
    assert np.array_equal(labs[0], labs[1])
    # RCB stays the default; an unknown partitioner is rejected
    assert eik.Eikonal(dim == 2).partitioner_ == eik.PARTITION_RCB
    e = eik.Eikonal(dim == 2)
    e.set_mesh(xyz, el)
    e.partitioner_ = 7
    with pytest.raises(eik.EikonalError) as ex:
        e.prepare()
    assert ex.value.code == 1


@pytest.mark.parametrize("bad", ["nan", "zero", "negative", "inf_metric6"])
def test_invalid_speeds_rejected_by_both_3d_entry_points(eik, mg, bad):
    """eik_solve and the allocation-free eik_solve3d_noalloc apply the same speed and
    metric checks before any device work (EIK_ERR_ARG = 1)."""
    xyz, tets = mg.kuhn_cube(5, 0.0)
    nt = tets.shape[0]
    if bad == "inf_metric6":
        sp = np.tile(np.array([1, 0, 0, 1, 0, 1], np.float32), nt)
        sp[6 * 3 + 1] = np.inf
    else:
        sp = np.ones(nt, np.float32)
        sp[7] = {"nan": np.nan, "zero": 0.0, "negative": -1.0}[bad]
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.initSpeedMtxMultipliers(sp)
    with pytest.raises(eik.EikonalError) as ex:
        e.prepare()
    assert ex.value.code == 1
    with pytest.raises(eik.EikonalError) as ex:
        eik.solve3d_noalloc(xyz, tets, sp, [0])
    assert ex.value.code == 1
    assert "tet" in str(ex.value)
