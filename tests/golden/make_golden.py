"""Writes the golden fixtures of the test suite.

  meshes.npz          the reference's own test meshes (src/test/test_data of
                      SCI-Solver_Eikonal): TetGen balls sphere8/13/334, the 16^3
                      CubeMesh, the torus with its per-tet metric file, and the PLY
                      spheres / square used by the 2D tests.  Read from the reference
                      source tree named by REFERENCE_ROOT.
  ref_host_setup.npz  inputs and outputs of the reference's own host set-up compiled
                      here from its sources (oracle/_ref/libref_tri.so: the 2D mesh
                      preparation; oracle/_ref/libref_host3d.so: TetMesh::init +
                      gettetmem) on meshes with obtuse corners, heterogeneous speeds,
                      near-right angles, slivers and anisotropic metrics; written with
                      `python tests/golden/make_golden.py --ref-host`.
  ref_gpu_outputs.npz travel times produced by the reference's own CUDA kernels
                      (oracle/_ref/*.cubin run by oracle/ref_gpu_driver.cpp) on fixed
                      inputs and partitions; written on a GPU machine with
                      `python tests/golden/make_golden.py --ref-gpu`.

    python tests/golden/make_golden.py            # meshes.npz (needs the reference tree)
    python tests/golden/make_golden.py --ref-host # ref_host_setup.npz (needs the reference tree)
    python tests/golden/make_golden.py --ref-gpu  # ref_gpu_outputs.npz (needs a GPU)
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = os.environ.get("REFERENCE_ROOT", "/root/reference")
DATA = os.path.join(REF, "src", "test", "test_data")


def read_tetgen(base):
    rows = [l.split() for l in open(base + ".node") if l.strip() and not l.lstrip().startswith("#")]
    n = int(rows[0][0])
    first = int(rows[1][0])
    xyz = np.zeros((n, 3), np.float32)
    for r in rows[1:n + 1]:
        xyz[int(r[0]) - first] = [np.float32(float(x)) for x in r[1:4]]
    rows = [l.split() for l in open(base + ".ele") if l.strip() and not l.lstrip().startswith("#")]
    m = int(rows[0][0])
    tets = np.array([[int(x) for x in r[1:5]] for r in rows[1:m + 1]], np.int32)
    if tets.min() == 1:
        tets -= 1
    return xyz, tets


def read_ply_ascii(path):
    lines = open(path).read().splitlines()
    nv = nf = 0
    i = 0
    while not lines[i].startswith("end_header"):
        p = lines[i].split()
        if p[:2] == ["element", "vertex"]:
            nv = int(p[2])
        if p[:2] == ["element", "face"]:
            nf = int(p[2])
        i += 1
    i += 1
    body = [l for l in lines[i:] if l.strip()]
    xyz = np.array([[np.float32(float(x)) for x in l.split()[:3]] for l in body[:nv]], np.float32)
    faces = []
    for l in body[nv:nv + nf]:
        p = [int(x) for x in l.split()]
        k = p[0]
        poly = p[1:1 + k]
        for j in range(1, k - 1):
            faces.append([poly[0], poly[j], poly[j + 1]])
    return xyz, np.array(faces, np.int32)


def make_meshes():
    out = {}
    for name in ["sphere8", "sphere13", "sphere334", "CubeMesh_size16", "torus"]:
        xyz, tets = read_tetgen(os.path.join(DATA, name))
        out[name + "_xyz"], out[name + "_tets"] = xyz, tets
    vals = np.array([float(x) for x in open(os.path.join(DATA, "torus_matrices.txt")).read().split()], np.float32)
    out["torus_metric"] = vals
    for name in ["sphere_12verts", "sphere_74verts", "sphere_1154verts", "sphere_4610verts", "SquareMesh_size16"]:
        xyz, faces = read_ply_ascii(os.path.join(DATA, name + ".ply"))
        out[name + "_xyz"], out[name + "_faces"] = xyz, faces
    np.savez_compressed(os.path.join(HERE, "meshes.npz"), **out)
    print("meshes.npz:", {k: v.shape for k, v in out.items()})


def ref_gpu_cases():
    """Fixed inputs for the reference-kernel fixtures: (name, dim, xyz, elems, speeds, labels, nb, seeds)."""
    import importlib
    mg = importlib.import_module("sci-solver_eikonal_gb300.meshgen")
    g = np.load(os.path.join(HERE, "meshes.npz"))
    cases = []
    # 3D: balls and torus with simple deterministic partitions
    for name in ["sphere334", "torus"]:
        xyz, tets = g[name + "_xyz"], g[name + "_tets"]
        nb = max(2, -(-xyz.shape[0] // 64))
        order = np.argsort(xyz[:, 0] + 1e-3 * xyz[:, 1] + 1e-6 * xyz[:, 2], kind="stable")
        lab = np.empty(xyz.shape[0], np.int32)
        lab[order] = np.arange(xyz.shape[0]) * nb // xyz.shape[0]
        sp = g["torus_metric"] if name == "torus" else None
        cases.append((name, 3, xyz, tets, sp, lab, nb, [0]))
    xyz, tets = mg.kuhn_cube(17, 0.2, seed=1)
    sp = (1.0 / mg.log_uniform_speeds(tets.shape[0], seed=2).astype(np.float64) ** 2).astype(np.float32)
    i = np.arange(xyz.shape[0])
    lab = ((i % 17) // 4 + 5 * (((i // 17) % 17) // 4) + 25 * ((i // 289) // 4)).astype(np.int32)
    cases.append(("cube17", 3, xyz, tets, sp, lab, int(lab.max()) + 1, [mg.center_vertex(17)]))
    # 2D
    xyz, faces = mg.grid2d(33)
    lab = (((np.arange(xyz.shape[0]) % 33) // 4) + 9 * ((np.arange(xyz.shape[0]) // 33) // 4)).astype(np.int32)
    cases.append(("grid33", 2, xyz, faces, None, lab, int(lab.max()) + 1, [0]))
    xyz, faces = g["sphere_74verts_xyz"], g["sphere_74verts_faces"]
    lab = (np.argsort(np.argsort(xyz[:, 2], kind="stable"), kind="stable") * 5 // xyz.shape[0]).astype(np.int32)
    cases.append(("sphere74", 2, xyz, faces, None, lab, 5, [0]))
    return cases


def make_ref_gpu():
    import importlib
    from oracle import oracle as O
    E = importlib.import_module("sci-solver_eikonal_gb300")
    out = {}
    for name, dim, xyz, el, sp, lab, nb, seeds in ref_gpu_cases():
        if dim == 3:
            M = O.metrics_from_speeds(el.shape[0], sp)
            r = O.ref_gpu_solve3d(xyz, el, M, lab, nb, seeds, history=True)
        else:
            e = E.Eikonal(True)
            e.set_mesh(xyz, el)
            f, obt, off, vfv = e.triPrep()
            init = np.full(xyz.shape[0], 1e7, np.float32)
            init[seeds] = 0
            r = O.ref_gpu_solve2d(xyz, f, np.ones(f.shape[0], np.float32), obt, off, vfv, lab, nb, seeds, init,
                                  history=True)
        out[name + "_result"] = r["result"]
        out[name + "_history"] = r["history"]
        out[name + "_iterations"] = np.int32(r["iterations"])
        out[name + "_updates"] = np.int64(r["vertex_updates"])
        print(name, r["iterations"], r["vertex_updates"])
    np.savez_compressed(os.path.join(HERE, "ref_gpu_outputs.npz"), **out)


def ref_host_cases():
    """Inputs of the host set-up fixtures: (name, dim, xyz, elems, speeds)."""
    import importlib
    mg = importlib.import_module("sci-solver_eikonal_gb300.meshgen")
    g = np.load(os.path.join(HERE, "meshes.npz"))
    cases = []
    # 2D: obtuse corners (PLY spheres), the same with heterogeneous face speeds,
    # right angles (grid, square), corners within rounding of 90 degrees
    cases.append(("sphere74", 2, g["sphere_74verts_xyz"], g["sphere_74verts_faces"], None))
    xyz, f = g["sphere_1154verts_xyz"], g["sphere_1154verts_faces"]
    cases.append(("sphere1154_speed", 2, xyz, f, mg.batch_speed(xyz, f)))
    xyz, f = mg.grid2d(33)
    cases.append(("grid33", 2, xyz, f, None))
    cases.append(("square16", 2, g["SquareMesh_size16_xyz"], g["SquareMesh_size16_faces"] - 1, None))
    rng = np.random.default_rng(12)
    xyz, f = mg.grid2d(21)
    xyz = xyz.copy()
    xyz[:, :2] += rng.uniform(-1e-7 / 20, 1e-7 / 20, (xyz.shape[0], 2)).astype(np.float32)
    cases.append(("grid21_near_right", 2, xyz, f, np.exp(rng.uniform(np.log(0.5), np.log(2), f.shape[0])).astype(
        np.float32)))
    # 3D: the reference's ball and anisotropic torus, a jittered cube with scalar
    # metrics, slivers with anisotropic 6-entry metrics
    cases.append(("sphere334", 3, g["sphere334_xyz"], g["sphere334_tets"], None))
    cases.append(("torus", 3, g["torus_xyz"], g["torus_tets"], g["torus_metric"]))
    xyz, t = mg.kuhn_cube(9, 0.2, seed=1)
    cases.append(("cube9", 3, xyz, t, (1.0 / mg.log_uniform_speeds(t.shape[0], seed=2).astype(np.float64) ** 2)
                  .astype(np.float32)))
    xyz, t, _ = mg.sliver_cube(9, 0.10, seed=5)
    cases.append(("sliver9_aniso", 3, xyz, t, mg.anisotropic_metrics(t.shape[0], seed=6).ravel()))
    return cases


def make_ref_host():
    from oracle import oracle as O
    if O.ref_host_lib("ref_tri") is None or O.ref_host_lib("ref_host3d") is None:
        raise SystemExit("the reference host builds are missing: run oracle/build_oracle.py with the reference tree")
    out = {}
    for name, dim, xyz, el, sp in ref_host_cases():
        out[name + "_xyz"] = np.asarray(xyz, np.float32)
        out[name + "_elems"] = np.asarray(el, np.int32)
        if sp is not None:
            out[name + "_speeds"] = np.asarray(sp, np.float32)
        if dim == 2:
            r = O.ref_tri_setup(xyz, el, sp)
            for k, v in r.items():
                out[name + "_" + k] = v
            print(name, el.shape[0], "faces", r["vf_verts"].shape[0], "virtual")
        else:
            _, G = O.ref_tet_gram(xyz, el, sp)
            out[name + "_gram"] = G
            print(name, el.shape[0], "tets")
    np.savez_compressed(os.path.join(HERE, "ref_host_setup.npz"), **out)


if __name__ == "__main__":
    if "--ref-gpu" in sys.argv:
        make_ref_gpu()
    elif "--ref-host" in sys.argv:
        make_ref_host()
    else:
        make_meshes()
