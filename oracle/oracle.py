"""ctypes binding of the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
module, and only as the checker.  It wraps liboracle.so (fim_oracle.cpp, the CPU
restatement of the reference scheme) and, where built, the reference's own host
code compiled here from its sources (_ref/: the tet local solver, the 2D mesh
preparation, the 3D metric set-up).
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_FP = ctypes.POINTER(ctypes.c_float)
_IP = ctypes.POINTER(ctypes.c_int)
_UP = ctypes.POINTER(ctypes.c_ubyte)
_LP = ctypes.POINTER(ctypes.c_longlong)

_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            from oracle import build_oracle
            build_oracle.build()
        _lib = ctypes.CDLL(path)
        f = _lib.oracle_tet_update_f32
        f.restype = ctypes.c_float
        f.argtypes = [ctypes.c_float] * 9
        f = _lib.oracle_tet_update_f64
        f.restype = ctypes.c_double
        f.argtypes = [ctypes.c_double] * 9
        f = _lib.oracle_tri_update_f32
        f.restype = ctypes.c_float
        f.argtypes = [ctypes.c_float] * 7
        _lib.oracle3d_solve.restype = ctypes.c_int
        _lib.oracle3d_solve.argtypes = [ctypes.c_int, _FP, ctypes.c_int, _IP, _FP, _IP, ctypes.c_int, _IP,
                                        ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        _FP, _FP, ctypes.c_int, _LP, _IP]
        _lib.oracle2d_solve.restype = ctypes.c_int
        _lib.oracle2d_solve.argtypes = [ctypes.c_int, _FP, ctypes.c_int, _IP, _FP, _UP, _IP, _IP, _FP, _IP,
                                        ctypes.c_int, _IP, ctypes.c_int, _FP, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_int, ctypes.c_int, _FP, _FP, ctypes.c_int, _LP, _IP]
        _lib.oracle_num_threads.restype = ctypes.c_int
        _lib.oracle_tet_group_fused.restype = None
        _lib.oracle_tet_group_fused.argtypes = [_FP, ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong), _FP]
        _lib.oracle_tet_fusion_mismatch.restype = ctypes.c_int
        _lib.oracle_tet_fusion_mismatch.argtypes = [_FP, _FP, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong]
        _lib.oracle_partition_rcb.restype = ctypes.c_int
        _lib.oracle_partition_rcb.argtypes = [ctypes.c_int, _FP, ctypes.c_int, ctypes.c_int, _IP]
        _lib.oracle_last_loop_seconds.restype = ctypes.c_double
        _lib.oracle3d_fp64_candidates.restype = ctypes.c_int
        _lib.oracle3d_fp64_candidates.argtypes = [ctypes.c_int, _FP, ctypes.c_int, _IP, _FP, _FP,
                                                  ctypes.POINTER(ctypes.c_double)]
    return _lib


def ref_lib():
    """The reference's tet local solver compiled for the host, or None."""
    global _ref
    path = os.path.join(HERE, "_ref", "libref_tet.so")
    if _ref is None and os.path.exists(path):
        _ref = ctypes.CDLL(path)
        _ref.ref_tet_local_solver.restype = ctypes.c_float
        _ref.ref_tet_local_solver.argtypes = [ctypes.c_float] * 9
    return _ref


_hostlibs = {}


def ref_host_lib(name):
    """A reference host build from _ref/ (libref_tri.so: the reference's trimesh
    preparation; libref_host3d.so: TetMesh::init + gettetmem), or None."""
    path = os.path.join(HERE, "_ref", f"lib{name}.so")
    if name not in _hostlibs:
        if not os.path.exists(path):
            return None
        lib = ctypes.CDLL(path)
        if name == "ref_tri":
            lib.ref_tri_setup.restype = ctypes.c_int
            lib.ref_tri_setup.argtypes = [ctypes.c_int, _FP, ctypes.c_int, _IP, _FP, ctypes.c_int, _IP, _FP, _FP, _IP,
                                          ctypes.c_int, _IP, _FP, _FP]
        else:
            lib.ref_tet_gram.restype = ctypes.c_int
            lib.ref_tet_gram.argtypes = [ctypes.c_int, _FP, ctypes.c_int, _IP, _FP, ctypes.c_int, _FP, _FP]
        _hostlibs[name] = lib
    return _hostlibs[name]


def ref_tri_setup(xyz, faces, speeds=None):
    """The reference's own 2D mesh preparation (meshFIM2dEikonal::SetMesh on a
    TriMesh, compiled from its sources): oriented faces, edge lengths, inverse
    speeds and virtual faces, as a dict of arrays."""
    lib = ref_host_lib("ref_tri")
    xyz, faces = _f(xyz), _i(faces)
    nv, nf = xyz.shape[0], faces.shape[0]
    sp = None if speeds is None else _f(speeds)
    cap = 8 * nf + 16
    while True:
        fo = np.empty((nf, 3), np.int32)
        eo = np.empty((nf, 3), np.float32)
        so = np.empty(nf, np.float32)
        vc = np.empty(nf, np.int32)
        vv = np.empty((cap, 3), np.int32)
        ve = np.empty((cap, 3), np.float32)
        vs = np.empty(cap, np.float32)
        n = lib.ref_tri_setup(nv, xyz.ctypes.data_as(_FP), nf, faces.ctypes.data_as(_IP),
                              sp.ctypes.data_as(_FP) if sp is not None else None, 0 if sp is None else sp.size,
                              fo.ctypes.data_as(_IP), eo.ctypes.data_as(_FP), so.ctypes.data_as(_FP),
                              vc.ctypes.data_as(_IP), cap, vv.ctypes.data_as(_IP), ve.ctypes.data_as(_FP),
                              vs.ctypes.data_as(_FP))
        if n <= cap:
            return {"faces": fo, "edges": eo, "speed_inv": so, "vf_count": vc, "vf_verts": vv[:n],
                    "vf_edges": ve[:n], "vf_speed_inv": vs[:n]}
        cap = n


def ref_tet_gram(xyz, tets, speeds=None):
    """The reference's own TetMesh::init + gettetmem (compiled from its sources):
    per tet its metric (6 entries) and six metric edge products."""
    lib = ref_host_lib("ref_host3d")
    xyz, tets = _f(xyz), _i(tets)
    nt = tets.shape[0]
    sp = None if speeds is None else _f(speeds)
    M = np.empty((nt, 6), np.float32)
    G = np.empty((nt, 6), np.float32)
    lib.ref_tet_gram(xyz.shape[0], xyz.ctypes.data_as(_FP), nt, tets.ctypes.data_as(_IP),
                     sp.ctypes.data_as(_FP) if sp is not None else None, 0 if sp is None else sp.size,
                     M.ctypes.data_as(_FP), G.ctypes.data_as(_FP))
    return M, G


def _f(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def _i(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def metrics_from_speeds(nt, vals):
    """Per-tet metric entries as TetMesh::init builds them (6*nt / nt / identity)."""
    vals = None if vals is None else np.asarray(vals, dtype=np.float32).ravel()
    M = np.zeros((nt, 6), dtype=np.float32)
    if vals is not None and vals.size == 6 * nt:
        return vals.reshape(nt, 6).copy()
    if vals is not None and vals.size == nt:
        M[:, 0] = M[:, 3] = M[:, 5] = vals
        return M
    M[:, 0] = M[:, 3] = M[:, 5] = 1.0
    return M


def solve3d(xyz, tets, metric6, labels, nblocks, seeds, max_iters=100, nsweeps=2, precision=32,
            nthreads=0, history=False):
    xyz, tets, M, lab, sd = _f(xyz), _i(tets), _f(metric6), _i(labels), _i(seeds)
    nv, nt = xyz.shape[0], tets.shape[0]
    out = np.empty(nv, dtype=np.float32)
    hist = np.empty((max_iters, nv), dtype=np.float32) if history else None
    upd = ctypes.c_longlong()
    mt = ctypes.c_int()
    it = lib().oracle3d_solve(nv, xyz.ctypes.data_as(_FP), nt, tets.ctypes.data_as(_IP), M.ctypes.data_as(_FP),
                              lab.ctypes.data_as(_IP), int(nblocks), sd.ctypes.data_as(_IP), sd.size,
                              int(max_iters), int(nsweeps), int(precision), int(nthreads),
                              out.ctypes.data_as(_FP), hist.ctypes.data_as(_FP) if history else None,
                              int(max_iters) if history else 0, ctypes.byref(upd), ctypes.byref(mt))
    if it < 0:
        raise ValueError("oracle3d_solve rejected its input")
    res = {"result": out, "iterations": it, "vertex_updates": upd.value, "max_tets": mt.value}
    if history:
        res["history"] = hist[:it]
    return res


def solve2d(xyz, faces, speed_inv, obtuse, vf_off, vf_verts, labels, nblocks, seeds, init_vals,
            max_iters=100, nsweeps=7, precision=32, nthreads=0, vf_speed_inv=None, history=False):
    xyz, faces, sinv, lab, sd, iv = _f(xyz), _i(faces), _f(speed_inv), _i(labels), _i(seeds), _f(init_vals)
    obt = np.ascontiguousarray(obtuse, dtype=np.uint8)
    off = _i(vf_off)
    vfv = _i(vf_verts).reshape(-1)
    if vfv.size == 0:
        vfv = np.zeros(3, dtype=np.int32)
    nvf = int(off[-1])
    vsp = _f(np.ones(max(nvf, 1)) if vf_speed_inv is None else vf_speed_inv)
    nv, nf = xyz.shape[0], faces.shape[0]
    out = np.empty(nv, dtype=np.float32)
    hist = np.empty((max_iters, nv), dtype=np.float32) if history else None
    upd = ctypes.c_longlong()
    mf = ctypes.c_int()
    it = lib().oracle2d_solve(nv, xyz.ctypes.data_as(_FP), nf, faces.ctypes.data_as(_IP),
                              sinv.ctypes.data_as(_FP), obt.ctypes.data_as(_UP), off.ctypes.data_as(_IP),
                              vfv.ctypes.data_as(_IP), vsp.ctypes.data_as(_FP), lab.ctypes.data_as(_IP),
                              int(nblocks), sd.ctypes.data_as(_IP), sd.size, iv.ctypes.data_as(_FP),
                              int(max_iters), int(nsweeps), int(precision), int(nthreads),
                              out.ctypes.data_as(_FP), hist.ctypes.data_as(_FP) if history else None,
                              int(max_iters) if history else 0, ctypes.byref(upd), ctypes.byref(mf))
    if it < 0:
        raise ValueError("oracle2d_solve rejected its input")
    res = {"result": out, "iterations": it, "vertex_updates": upd.value, "max_faces": mf.value}
    if history:
        res["history"] = hist[:it]
    return res


def partition_rcb(xyz, verts_per_block, dim=3):
    """Labels and block count of the product's default partition (recursive
    coordinate bisection with the reference's block-count rule), restated."""
    xyz = _f(xyz)
    lab = np.empty(xyz.shape[0], dtype=np.int32)
    nb = lib().oracle_partition_rcb(xyz.shape[0], xyz.ctypes.data_as(_FP), int(verts_per_block), int(dim),
                                    lab.ctypes.data_as(_IP))
    if nb < 0:
        raise ValueError("oracle_partition_rcb rejected its input")
    return lab, nb


def tet_group_fused(inputs10, masks):
    """The CPU model of the reference kernel's four apex updates of a slot with
    the given fused-multiply-add masks (tet_fusion_model.hpp): (n, 4) outputs."""
    a = _f(inputs10).reshape(-1, 10)
    out = np.empty((a.shape[0], 4), dtype=np.float32)
    m = (ctypes.c_ulonglong * 4)(*[int(x) for x in masks])
    lib().oracle_tet_group_fused(a.ctypes.data_as(_FP), a.shape[0], m, out.ctypes.data_as(_FP))
    return out


def tet_fusion_mismatch(inputs10, want4, k, mask):
    a, w = _f(inputs10).reshape(-1, 10), _f(want4).reshape(-1, 4)
    return lib().oracle_tet_fusion_mismatch(a.ctypes.data_as(_FP), w.ctypes.data_as(_FP), a.shape[0], int(k),
                                            ctypes.c_ulonglong(int(mask)))


def fp64_candidates(xyz, tets, metric6, T):
    """Per vertex the smallest FP64 tet update over its incident tets from the
    times T (FP64 edge products of the 6-entry metrics); 1e9 where none is finite."""
    xyz, tets, M, T = _f(xyz), _i(tets), _f(metric6), _f(T)
    out = np.empty(xyz.shape[0], dtype=np.float64)
    rc = lib().oracle3d_fp64_candidates(xyz.shape[0], xyz.ctypes.data_as(_FP), tets.shape[0], tets.ctypes.data_as(_IP),
                                        M.ctypes.data_as(_FP), T.ctypes.data_as(_FP),
                                        out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if rc < 0:
        raise ValueError("oracle3d_fp64_candidates rejected its input")
    return out


def fp64_residual(xyz, tets, metric6, T):
    """FP64 fixed-point residual of T, split by sign, relative to T (seeds and
    unreached vertices left out): "lowerable" = max (T - c) / T where an FP64
    update c lies below T (more FIM updates would lower T there), "below" =
    max (c - T) / T where T lies below every FP64 update of its tets."""
    T = np.asarray(T, dtype=np.float32)
    c = fp64_candidates(xyz, tets, metric6, T)
    t = T.astype(np.float64)
    ok = (t > 0) & (t < 1e9) & (c < 1e9)
    d = (t - c)[ok] / t[ok]
    return {"lowerable": float(max(d.max(initial=0.0), 0.0)), "below": float(max((-d).max(initial=0.0), 0.0)),
            "lowerable_1e-5": int((d > 1e-5).sum()), "below_1e-5": int((d < -1e-5).sum())}


def num_threads():
    return lib().oracle_num_threads()


def last_loop_seconds():
    """Wall time of the outer iterations of the last solve3d (layout set-up excluded)."""
    return lib().oracle_last_loop_seconds()


# ---------------------------------------------------------------------------
# the reference's own kernels (cubins built from the reference tree) driven by
# the restated host loop in ref_gpu_driver.cpp
# ---------------------------------------------------------------------------
_gpu = None
CUBIN3D = os.path.join(HERE, "_ref", "ref3d.cubin")
CUBIN2D = os.path.join(HERE, "_ref", "ref2d.cubin")


def ref_gpu():
    """libref_gpu.so, or None when it or the cubins are missing."""
    global _gpu
    path = os.path.join(HERE, "libref_gpu.so")
    if _gpu is None:
        if not (os.path.exists(path) and os.path.exists(CUBIN3D) and os.path.exists(CUBIN2D)):
            return None
        g = ctypes.CDLL(path)
        g.refgpu_last_error.restype = ctypes.c_char_p
        g.refgpu_last_loop_ms.restype = ctypes.c_double
        g.refgpu_tet_local_solver.restype = ctypes.c_int
        g.refgpu_tet_local_solver.argtypes = [ctypes.c_char_p, _FP, _FP, ctypes.c_int]
        g.refgpu_solve3d.restype = ctypes.c_int
        g.refgpu_solve3d.argtypes = [ctypes.c_char_p, ctypes.c_int, _FP, ctypes.c_int, _IP, _FP, _IP, ctypes.c_int,
                                     _IP, ctypes.c_int, ctypes.c_int, _FP, _FP, ctypes.c_int, _LP, _IP]
        g.refgpu_tet_blocks.restype = ctypes.c_int
        g.refgpu_tet_blocks.argtypes = [ctypes.c_char_p, _FP, ctypes.c_int, _FP]
        g.refgpu_tri_blocks.restype = ctypes.c_int
        g.refgpu_tri_blocks.argtypes = [ctypes.c_char_p, _FP, ctypes.c_int, ctypes.c_int, _FP]
        g.refgpu_solve2d.restype = ctypes.c_int
        g.refgpu_solve2d.argtypes = [ctypes.c_char_p, ctypes.c_int, _FP, ctypes.c_int, _IP, _FP, _UP, _IP, _IP, _FP,
                                     _IP, ctypes.c_int, _IP, ctypes.c_int, _FP, ctypes.c_int, _FP, _FP, ctypes.c_int,
                                     _LP, _IP]
        _gpu = g
    return _gpu


class ReferenceUnavailable(RuntimeError):
    pass


def _gpu_check(rc):
    if rc == -1:
        raise ReferenceUnavailable(ref_gpu().refgpu_last_error().decode())
    if rc < 0:
        raise RuntimeError("reference kernels failed: " + ref_gpu().refgpu_last_error().decode())
    return rc


def ref_gpu_tet_local_solver(inputs9):
    a = _f(inputs9).reshape(-1, 9)
    out = np.empty(a.shape[0], dtype=np.float32)
    _gpu_check(ref_gpu().refgpu_tet_local_solver(CUBIN3D.encode(), a.ctypes.data_as(_FP), out.ctypes.data_as(_FP),
                                                 a.shape[0]))
    return out


def ref_gpu_tet_blocks(inputs10):
    """Single-tet blocks through the reference's 3D FIMCuda, one sweep; inputs
    TA TB TC TD and the six metric edge products; returns the four vertex values
    (each min(T_k, the update of apex k) as FIMCuda computes it)."""
    a = _f(inputs10).reshape(-1, 10)
    out = np.empty((a.shape[0], 4), dtype=np.float32)
    _gpu_check(ref_gpu().refgpu_tet_blocks(CUBIN3D.encode(), a.ctypes.data_as(_FP), a.shape[0],
                                           out.ctypes.data_as(_FP)))
    return out


def ref_gpu_tri_blocks(inputs7, check=False):
    """Single-triangle blocks through the reference's 2D FIMCuda (7 sweeps) or
    run_check_neighbor (1 sweep); inputs T0 T1 T2 e01 e12 e20 speedInv."""
    a = _f(inputs7).reshape(-1, 7)
    out = np.empty((a.shape[0], 3), dtype=np.float32)
    _gpu_check(ref_gpu().refgpu_tri_blocks(CUBIN2D.encode(), a.ctypes.data_as(_FP), a.shape[0], int(bool(check)),
                                           out.ctypes.data_as(_FP)))
    return out


def ref_gpu_solve3d(xyz, tets, metric6, labels, nblocks, seeds, max_iters=100, history=False):
    xyz, tets, M, lab, sd = _f(xyz), _i(tets), _f(metric6), _i(labels), _i(seeds)
    nv = xyz.shape[0]
    out = np.empty(nv, dtype=np.float32)
    hist = np.empty((max_iters, nv), dtype=np.float32) if history else None
    upd, mt = ctypes.c_longlong(), ctypes.c_int()
    it = _gpu_check(ref_gpu().refgpu_solve3d(
        CUBIN3D.encode(), nv, xyz.ctypes.data_as(_FP), tets.shape[0], tets.ctypes.data_as(_IP),
        M.ctypes.data_as(_FP), lab.ctypes.data_as(_IP), int(nblocks), sd.ctypes.data_as(_IP), sd.size,
        int(max_iters), out.ctypes.data_as(_FP), hist.ctypes.data_as(_FP) if history else None,
        int(max_iters) if history else 0, ctypes.byref(upd), ctypes.byref(mt)))
    res = {"result": out, "iterations": it, "vertex_updates": upd.value, "max_tets": mt.value,
           "loop_ms": ref_gpu().refgpu_last_loop_ms()}
    if history:
        res["history"] = hist[:it]
    return res


def ref_gpu_solve2d(xyz, faces, speed_inv, obtuse, vf_off, vf_verts, labels, nblocks, seeds, init_vals,
                    max_iters=100, vf_speed_inv=None, history=False):
    xyz, faces, sinv, lab, sd, iv = _f(xyz), _i(faces), _f(speed_inv), _i(labels), _i(seeds), _f(init_vals)
    obt = np.ascontiguousarray(obtuse, dtype=np.uint8)
    off = _i(vf_off)
    vfv = _i(vf_verts).reshape(-1)
    if vfv.size == 0:
        vfv = np.zeros(3, dtype=np.int32)
    nvf = int(off[-1])
    vsp = _f(np.ones(max(nvf, 1)) if vf_speed_inv is None else vf_speed_inv)
    nv = xyz.shape[0]
    out = np.empty(nv, dtype=np.float32)
    hist = np.empty((max_iters, nv), dtype=np.float32) if history else None
    upd, mf = ctypes.c_longlong(), ctypes.c_int()
    it = _gpu_check(ref_gpu().refgpu_solve2d(
        CUBIN2D.encode(), nv, xyz.ctypes.data_as(_FP), faces.shape[0], faces.ctypes.data_as(_IP),
        sinv.ctypes.data_as(_FP), obt.ctypes.data_as(_UP), off.ctypes.data_as(_IP), vfv.ctypes.data_as(_IP),
        vsp.ctypes.data_as(_FP), lab.ctypes.data_as(_IP), int(nblocks), sd.ctypes.data_as(_IP), sd.size,
        iv.ctypes.data_as(_FP), int(max_iters), out.ctypes.data_as(_FP),
        hist.ctypes.data_as(_FP) if history else None, int(max_iters) if history else 0, ctypes.byref(upd),
        ctypes.byref(mf)))
    res = {"result": out, "iterations": it, "vertex_updates": upd.value, "max_faces": mf.value,
           "loop_ms": ref_gpu().refgpu_last_loop_ms()}
    if history:
        res["history"] = hist[:it]
    return res
