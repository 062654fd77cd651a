"""Autotuner for the block size and CTA size of batched (and single) solves.

The block-FIM solve has two launch-shape knobs that trade against each other:

  vertices per block   larger blocks mean fewer outer iterations across a mesh and
                       fewer halo copies, but more sweeps wasted on converged parts
                       of a block and more shared memory per visit;
  threads per block    the CTA size of the 3D visit kernels (one thread per element
                       slot gives the shortest visit; fewer threads raise occupancy).
                       The 2D visit kernels run one thread per element slot, so their
                       CTA size follows from the block size.

Neither changes the scheme's arithmetic for a given partition: a different block
size is a different partition (a different, equally valid result, as with the
reference's maxVertsPerBlock_), a different CTA size gives bit-identical results.
The tuner times each candidate on the device (the solve's own CUDA-event time,
median of `reps` solves after one warm-up) and keeps the fastest.
"""
import concurrent.futures as _fut
import os
import time

import numpy as np


def _prepare_all(solvers, workers):
    # ctypes releases the GIL, so host layouts of independent handles build in parallel
    if workers <= 1:
        for e in solvers:
            e.prepare()
        return
    with _fut.ThreadPoolExecutor(max_workers=workers) as ex:
        list(ex.map(lambda e: e.prepare(), solvers))


def default_candidates(dim):
    if dim == 2:
        return (16, 32, 64, 128), (0,)
    return (32, 64, 128), (256, 512, 1024)


class TuneResult:
    def __init__(self, vpb, threads, table):
        self.verts_per_block = vpb
        self.threads_per_block = threads
        self.table = table  # list of dicts: vpb, threads, solve_ms (median), iterations

    def as_dict(self):
        return {"verts_per_block": self.verts_per_block, "threads_per_block": self.threads_per_block,
                "table": self.table}


def tune_batch(solvers, vpb_candidates=None, thread_candidates=None, reps=3, workers=None, log=None):
    """Times every (vertices per block, threads per block) pair on a batch of
    configured Eikonal handles (one dimension) and leaves the handles set to the
    fastest.  Returns (TuneResult, EikonalBatch built with the chosen setting)."""
    from . import EikonalBatch  # the package's batch wrapper

    solvers = list(solvers)
    dim = 2 if solvers[0].isTriMesh_ else 3
    dv, dt = default_candidates(dim)
    vpbs = tuple(vpb_candidates or dv)
    threads = tuple(thread_candidates or dt)
    workers = workers or min(16, os.cpu_count() or 1)
    table = []
    best = None
    best_batch = None
    for vpb in vpbs:
        for e in solvers:
            e.maxVertsPerBlock_ = int(vpb)
        t0 = time.perf_counter()
        _prepare_all(solvers, workers)
        prep_s = time.perf_counter() - t0
        batch = EikonalBatch(solvers)
        for th in threads:
            for e in solvers:
                e.threadsPerBlock_ = int(th)
            try:
                batch.solveEikonal()  # warm-up (uploads the packed layout once)
            except Exception as ex:  # a block too large for shared memory: skip the candidate
                table.append({"verts_per_block": vpb, "threads_per_block": th, "error": str(ex)})
                continue
            ms = []
            for _ in range(reps):
                batch.solveEikonal()
                ms.append(batch.stats()["solve_ms"])
            row = {"verts_per_block": int(vpb), "threads_per_block": int(th),
                   "solve_ms": float(np.median(ms)), "iterations": int(batch.stats()["iterations"]),
                   "host_prepare_s": round(prep_s, 3)}
            table.append(row)
            if log:
                log(row)
            if best is None or row["solve_ms"] < best["solve_ms"]:
                best = row
                best_batch = batch
    if best is None:
        raise RuntimeError("no candidate launch shape could run")
    for e in solvers:
        e.maxVertsPerBlock_ = best["verts_per_block"]
        e.threadsPerBlock_ = best["threads_per_block"]
    if best_batch is not batch:
        _prepare_all(solvers, workers)
        best_batch = EikonalBatch(solvers)
    return TuneResult(best["verts_per_block"], best["threads_per_block"], table), best_batch
