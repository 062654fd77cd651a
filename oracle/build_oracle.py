"""Builds the oracle (test infrastructure only; the product never links it).

  oracle/liboracle.so          CPU restatement of the reference scheme (fim_oracle.cpp),
                               built everywhere (here and on the GPU machine)
  oracle/libref_gpu.so         host loop that drives the reference's kernels from the
                               cubins below (ref_gpu_driver.cpp), built everywhere
  oracle/_ref/libref_tet.so    the reference's own tet local solver compiled for the
                               host from the reference tree (ref_tethost.cpp + refshim/)
  oracle/_ref/ref3d.cubin      the reference's 3D kernels for sm_103a (ref_wrap3d.cu)
  oracle/_ref/ref2d.cubin      the reference's 2D kernels for sm_103a (ref_wrap2d.cu)
  oracle/_ref/libref_tri.so    the reference's 2D mesh preparation (its trimesh sources
                               src/core2d/cuda/TriMesh_*.cu, filter.cc, ... compiled as host
                               C++ with g++, driven by ref_trihost.cpp)
  oracle/_ref/libref_host3d.so the reference's TetMesh::init and gettetmem (tetmesh.cu,
                               meshFIM3dEikonal.cu and CUDA_kernels.cu compiled by nvcc, as
                               its own build compiles them, driven by ref_tethost3d.cu; shims
                               for cusp and metis.h in refshim_nvcc/, cudaThreadSynchronize
                               mapped to cudaDeviceSynchronize)

Host floating point of the reference builds: x86-64's baseline instruction set has
no fused multiply-add, so g++ and nvcc's host pass round every product and sum
separately there, whatever -ffp-contract says; the product's host set-up is built
with -ffp-contract=off to give those bits on every host, including aarch64, where
gcc would otherwise fuse (its default is -ffp-contract=fast).  The pin tests hold
the product's host set-up to these builds bit for bit.

The _ref artefacts need the reference sources (REFERENCE_ROOT, default
/root/reference); where they are absent only liboracle.so is built and whatever
_ref files already exist are kept.  The reference's own CMake build is not used:
it needs METIS and cusp, which are not available offline.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("REFERENCE_ROOT", "/root/reference")
OUT_REF = os.path.join(HERE, "_ref")
NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")


# host sources of the reference's trimesh directory (src/core2d/cuda)
TRI_SOURCES = ["TriMesh_connectivity.cu", "TriMesh_stats.cu", "TriMesh_normals.cu", "TriMesh_tstrips.cu",
               "TriMesh_bounding.cu", "TriMesh_grid.cu", "TriMesh_io.cu", "filter.cc", "TriMesh_curvature.cc",
               "TriMesh_pointareas.cc", "KDtree.cc", "remove.cc", "reorder_verts.cc"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out, srcs):
    return not os.path.exists(out) or any(os.path.getmtime(s) > os.path.getmtime(out) for s in srcs)


def build(force=False):
    built = []
    src = os.path.join(HERE, "fim_oracle.cpp")
    lib = os.path.join(HERE, "liboracle.so")
    hdr = os.path.join(HERE, "oracle_scheme.hpp")
    if force or _stale(lib, [src, hdr, os.path.join(HERE, "tet_fusion_model.hpp")]):
        _run([CXX, "-O2", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", src, "-o", lib])
    built.append(lib)
    # driver that runs the reference's kernels (loaded from _ref/*.cubin at run time)
    drv = os.path.join(HERE, "ref_gpu_driver.cpp")
    glib = os.path.join(HERE, "libref_gpu.so")
    if force or _stale(glib, [drv, hdr]):
        _run([NVCC, "-O2", "-std=c++17", "-x", "cu", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-shared", "--cudart", "static", "-gencode", "arch=compute_103a,code=sm_103a", drv, "-o", glib])
    built.append(glib)
    src3 = os.path.join(REF, "src", "core3d")
    src2 = os.path.join(REF, "src", "core2d")
    if not os.path.isdir(src3):
        return built
    os.makedirs(OUT_REF, exist_ok=True)
    jobs = []
    tet = os.path.join(OUT_REF, "libref_tet.so")
    if force or _stale(tet, [os.path.join(HERE, "ref_tethost.cpp")]):
        jobs.append([CXX, "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared",
                     "-I", os.path.join(HERE, "refshim"), "-I", os.path.join(src3, "include"), "-I", src3,
                     os.path.join(HERE, "ref_tethost.cpp"), "-o", tet])
    for dim, sdir in (("3d", src3), ("2d", src2)):
        wrap = os.path.join(HERE, f"ref_wrap{dim}.cu")
        cub = os.path.join(OUT_REF, f"ref{dim}.cubin")
        if force or _stale(cub, [wrap]):
            # -maxrregcount=64: the reference launches one thread per element slot (up
            # to 1024); without a register cap those launches fail on sm_103a.  The cap
            # changes register allocation only, not the arithmetic.
            jobs.append([NVCC, "-std=c++17", "-O3", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a",
                         "-maxrregcount=64", "-w", "-I", os.path.join(sdir, "include"), "-I", sdir, wrap,
                         "-o", cub])
    # the reference's 2D mesh preparation: every host source of its trimesh
    # directory (they reference each other), plus the driver
    tri = os.path.join(OUT_REF, "libref_tri.so")
    tri_srcs = [os.path.join(src2, "cuda", f) for f in TRI_SOURCES] + [os.path.join(HERE, "ref_trihost.cpp")]
    tri_objs = []
    if force or _stale(tri, tri_srcs):
        objdir = os.path.join(OUT_REF, "tri_obj")
        os.makedirs(objdir, exist_ok=True)
        for src in tri_srcs:
            obj = os.path.join(objdir, os.path.basename(src) + ".o")
            tri_objs.append(obj)
            jobs.append([CXX, "-O2", "-std=c++17", "-w", "-fPIC", "-x", "c++", "-include",
                         os.path.join(HERE, "refshim", "host_minmax.h"), "-I", os.path.join(src2, "include"),
                         "-c", src, "-o", obj])
    h3 = os.path.join(OUT_REF, "libref_host3d.so")
    drv3 = os.path.join(HERE, "ref_tethost3d.cu")
    if force or _stale(h3, [drv3]):
        jobs.append([NVCC, "-std=c++17", "-O2", "-w", "-rdc=true", "-shared", "-Xcompiler", "-fPIC", "--cudart", "static",
                     "-gencode", "arch=compute_103a,code=sm_103a", "-DcudaThreadSynchronize=cudaDeviceSynchronize",
                     "-I", os.path.join(HERE, "refshim_nvcc"), "-I", os.path.join(src3, "include"), "-I", src3, drv3,
                     os.path.join(src3, "cuda", "meshFIM3dEikonal.cu"), os.path.join(src3, "cuda", "tetmesh.cu"),
                     os.path.join(src3, "cuda", "CUDA_kernels.cu"), "-o", h3])
    procs = [subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True) for j in jobs]
    for j, p in zip(jobs, procs):
        out, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("oracle build failed: " + " ".join(j) + "\n" + out + err)
    if tri_objs:
        _run([CXX, "-shared", "-Wl,--no-undefined", "-o", tri, *tri_objs])
    built += [tet, os.path.join(OUT_REF, "ref3d.cubin"), os.path.join(OUT_REF, "ref2d.cubin"), tri, h3]
    return built


if __name__ == "__main__":
    for p in build(force="--force" in sys.argv):
        print(p)
