"""The product's host set-up pinned against the reference's own host code.

The reference's 2D mesh preparation (meshFIM2dEikonal::SetMesh: orient, across-edge
map, face edge lengths, inverse speeds and the obtuse-corner unfolding into virtual
faces, src/core2d/include/meshFIM2d_eikonal.h:40-72, TriMesh.h:191-313,
TriMesh_connectivity.cu:54-75,206-278, TriMesh_stats.cu:46-70, filter.cc:369-452)
and its 3D metric set-up (TetMesh::init, tetmesh.cu:9-80; gettetmem,
meshFIM3dEikonal.cu:650-678) are compiled from its sources into oracle/_ref/ by
oracle/build_oracle.py.  Where those builds are present the product's set-up must
equal them bit for bit on the reference's fixtures and on stress meshes; everywhere
it must equal the committed outputs of those builds (tests/golden/ref_host_setup.npz,
written by tests/golden/make_golden.py --ref-host).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, bits_equal


def _ours_2d(eik, xyz, faces, speeds):
    e = eik.Eikonal(True)
    e.set_mesh(xyz, faces)
    if speeds is not None:
        e.initSpeedMtxMultipliers(speeds)
    f, _, off, vfv = e.triPrep()
    ed, si, ved, vsi = e.triPrepValues()
    return {"faces": f, "edges": ed, "speed_inv": si, "vf_count": np.diff(off).astype(np.int32),
            "vf_verts": vfv, "vf_edges": ved, "vf_speed_inv": vsi}


def _ours_3d(eik, xyz, tets, speeds):
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    if speeds is not None:
        e.initSpeedMtxMultipliers(speeds)
    e.prepare()
    return e.tetGram(False)


def _same_2d(got, want, name):
    for k, w in want.items():
        g = got[k]
        if w.dtype == np.float32:
            assert bits_equal(g, w), (name, k)
        else:
            assert g.shape == w.shape and np.array_equal(g, w), (name, k)


def _stress_2d(mg, golden):
    rng = np.random.default_rng(3)
    out = []
    for k in ("sphere_12verts", "sphere_74verts", "sphere_1154verts", "sphere_4610verts"):
        out.append((k, golden[k + "_xyz"], golden[k + "_faces"], None))
    xyz, f = golden["sphere_1154verts_xyz"], golden["sphere_1154verts_faces"]
    out.append(("sphere1154_speed", xyz, f, mg.batch_speed(xyz, f)))
    out.append(("square16", golden["SquareMesh_size16_xyz"], golden["SquareMesh_size16_faces"] - 1, None))
    for eps in (0.0, 1e-7, 1e-5, 0.3):  # right angles, within rounding of 90 degrees, strongly obtuse
        xyz, f = mg.grid2d(41)
        xyz = xyz.copy()
        xyz[:, :2] += rng.uniform(-eps / 40, eps / 40, (xyz.shape[0], 2)).astype(np.float32)
        sp = np.exp(rng.uniform(np.log(0.5), np.log(2), f.shape[0])).astype(np.float32)
        out.append((f"grid41_jitter{eps}", xyz, f, sp))
    xyz, f = mg.icosphere(4)
    xyz = (xyz * (1 + rng.uniform(-0.2, 0.2, (xyz.shape[0], 1)))).astype(np.float32)
    out.append(("icosphere4_bumpy", xyz, f, mg.batch_speed(xyz, f)))
    return out


@pytest.mark.parametrize("idx", range(11))
def test_2d_prep_bitwise_vs_reference_host_build(eik, O, mg, golden, idx):
    if O.ref_host_lib("ref_tri") is None:
        pytest.skip("reference host build not present (oracle/_ref/libref_tri.so, built from the reference tree)")
    name, xyz, f, sp = _stress_2d(mg, golden)[idx]
    want = O.ref_tri_setup(xyz, f, sp)
    _same_2d(_ours_2d(eik, xyz, f, sp), want, name)


def _stress_3d(mg, golden):
    out = [("sphere334", golden["sphere334_xyz"], golden["sphere334_tets"], None),
           ("torus", golden["torus_xyz"], golden["torus_tets"], golden["torus_metric"]),
           ("cube16", golden["CubeMesh_size16_xyz"], golden["CubeMesh_size16_tets"], None)]
    for n in (9, 33):
        xyz, t = mg.kuhn_cube(n, 0.2, seed=1)
        v = mg.log_uniform_speeds(t.shape[0], seed=2)
        out.append((f"cube{n}", xyz, t, (1.0 / v.astype(np.float64) ** 2).astype(np.float32)))
    xyz, t, _ = mg.sliver_cube(13, 0.10, seed=5)
    out.append(("sliver13_aniso", xyz, t, mg.anisotropic_metrics(t.shape[0], seed=6).ravel()))
    return out


@pytest.mark.parametrize("idx", range(6))
def test_3d_gram_bitwise_vs_reference_host_build(eik, O, mg, golden, idx):
    if O.ref_host_lib("ref_host3d") is None:
        pytest.skip("reference host build not present (oracle/_ref/libref_host3d.so, built from the reference tree)")
    name, xyz, t, sp = _stress_3d(mg, golden)[idx]
    _, want = O.ref_tet_gram(xyz, t, sp)
    assert bits_equal(_ours_3d(eik, xyz, t, sp), want), name


def _fixture():
    return np.load(os.path.join(GOLDEN, "ref_host_setup.npz"))


def fixture_cases():
    fx = _fixture()
    names = sorted({k.rsplit("_", 1)[0] for k in fx.files if k.endswith("_xyz")})
    return fx, names


def test_host_setup_equals_reference_fixture(eik):
    """Runs wherever the suite runs: the product's host set-up against the committed
    outputs of the reference's host builds."""
    fx, names = fixture_cases()
    assert len(names) == 9
    for name in names:
        xyz, el = fx[name + "_xyz"], fx[name + "_elems"]
        sp = fx[name + "_speeds"] if name + "_speeds" in fx.files else None
        if el.shape[1] == 3:
            want = {k: fx[name + "_" + k] for k in ("faces", "edges", "speed_inv", "vf_count", "vf_verts", "vf_edges",
                                                    "vf_speed_inv")}
            _same_2d(_ours_2d(eik, xyz, el, sp), want, name)
        else:
            assert bits_equal(_ours_3d(eik, xyz, el, sp), fx[name + "_gram"]), name
