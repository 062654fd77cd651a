"""Builds libeikonal_gb300.so in this directory (host C++ with g++, CUDA with nvcc
for sm_103a, static CUDA runtime).  Sources are compiled in parallel and skipped
when their object file is newer than every input.

    python sci-solver_eikonal_gb300/build.py          # build if stale
    python sci-solver_eikonal_gb300/build.py --force  # rebuild everything
"""
import glob
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libeikonal_gb300.so")

NVCC = os.environ.get("NVCC", "nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: host float expressions round one operation at a time, as the
# reference's host setup does; device code keeps nvcc's default contraction.
HOST_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wextra"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xcompiler",
              "-ffp-contract=off"]

HOST_SRC = ["setup.cpp", "mesh_io.cpp", "capi.cpp", "serve.cpp"]
CUDA_SRC = ["fim_device.cu", "setup_device.cu"]
HEADERS = ["setup.hpp", "mesh_io.hpp", "device.hpp", "local_update.cuh", "solver_access.hpp"]


def _metis_archive():
    """METIS 5 as the CUDA toolkit ships it (libmetis_static.a), or None."""
    nvcc = shutil.which(NVCC) or NVCC
    homes = [os.environ.get("CUDA_HOME"), os.path.dirname(os.path.dirname(os.path.realpath(nvcc))),
             "/usr/local/cuda"]
    for h in homes:
        if not h:
            continue
        for sub in ("lib64", "lib"):
            cand = os.path.join(h, sub, "libmetis_static.a")
            if os.path.exists(cand):
                return cand
        for cand in sorted(glob.glob(os.path.join(h, "targets", "*", "lib", "libmetis_static.a"))):
            return cand
    return None


def _newer(target, deps):
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r


def build(force=False, verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    metis = _metis_archive()
    host_flags = HOST_FLAGS + (["-DEIK_HAVE_METIS"] if metis else [])
    # a build with and one without METIS must not share objects
    stamp = os.path.join(OBJ, "metis.txt")
    want = metis or "none"
    if not os.path.exists(stamp) or open(stamp).read() != want:
        force = True
        with open(stamp, "w") as fh:
            fh.write(want)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", "eikonal_gb300.h")]
    jobs = []
    objs = []
    for s in HOST_SRC + CUDA_SRC:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s + ".o")
        objs.append(obj)
        if force or not _newer(obj, [src] + hdrs):
            if s.endswith(".cu"):
                cmd = [NVCC, *NVCC_FLAGS, "-c", src, "-o", obj]
            else:
                cmd = [CXX, *host_flags, "-c", src, "-o", obj]
            jobs.append(cmd)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for r in ex.map(_run, jobs):
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
    if force or jobs or not _newer(LIB, objs):
        # METIS is linked in with its symbols kept local, so a caller's own METIS
        # cannot clash with it
        extra = [metis, "-Xlinker", "--exclude-libs,libmetis_static.a", "-lm"] if metis else []
        _run([NVCC, "-shared", *ARCH, "--cudart", "static", "-o", LIB, *objs, *extra, "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
