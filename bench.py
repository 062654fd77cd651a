#!/usr/bin/env python3
"""Benchmark of the GB300 block-FIM Eikonal solver (one JSON line on rank 0).

Workload (the plain-FIM-at-scale configuration): a 65^3 vertex grid on the unit
cube, every cube Kuhn-split into 6 tets (274,625 vertices, 1,572,864 tets),
interior vertices jittered by U(-0.2h, 0.2h)^3 (seed 1), per-tet speed
log-uniform in [0.5, 2] (seed 2) given to the solver as the scalar metric 1/v^2,
one seed at the centre vertex, 64 vertices per block.  A step is one complete
solve (seed -> every block converged).

  value  vertex-updates/s of the device-resident solve (mesh, partition and metric
         terms resident in HBM), timed with CUDA events on the solver's stream;
         L2 is flushed (512 MB write) before every timed solve, outside the events
  e2e    the same metric through the C ABI with host buffers: seeds copied in,
         solve, travel times copied out, wall clock per step
  roofline  the block-sweep kernel: algorithmic bytes of its launches / their
         device-timer spans, against the measured HBM copy bandwidth
  cpu_baseline  the CPU restatement of the reference scheme (oracle/) with all
         host threads on a bounded sample of the same solve

  reference_gpu  the reference's own kernels (built from its sources into
         oracle/_ref/ref3d.cubin) under a restatement of its host loop, on the same
         mesh and partition: the outer loop's wall time and rate

--impl reference times that CPU restatement alone (the reference has no CPU
driver of its own, and its CUDA build needs METIS 4 and cusp), with the
partition from the oracle's restatement of the default bisection: that arm loads
no product code.  With N > 1 ranks every rank runs its own replica (no
collective in the solve path); value sums all ranks' updates over the slowest
rank's time.
"""
import argparse
import importlib
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "vertex-updates/s & solves/s, batched vs plain FIM; p50/p99 solve latency"
WORKLOAD = ("plain FIM 3D at scale: 65^3 jittered Kuhn cube (274,625 verts, 1,572,864 tets), "
            "log-uniform per-tet speed [0.5, 2] as metric 1/v^2, seed at the centre vertex, 64 verts/block")
N_GRID = 65
MAX_ITERS = 100  # the reference default (src/Eikonal.cu:19); the workload converges in 81
DRAM_PROFILE = "fim3d_items_dram_c3d.txt"  # per-launch DRAM bytes of the sweep and check kernels over one solve


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--cpu-sample-iters", type=int, default=0, help="0 = choose automatically")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-reference-gpu", action="store_true",
                   help="skip the reference kernels' solve of the headline workload (reference_gpu)")
    p.add_argument("--workload", default="c3d", choices=["c3d", "batch", "serve", "prec"],
                   help="c3d: the 65^3 tet solve (headline); batch: 256 icospheres, batched vs plain; "
                        "serve: Poisson request stream over a resident mesh pool; "
                        "prec: sliver + anisotropic 49^3 mesh, FP32 vs mixed FP32/FP64 vs an FP64 run")
    p.add_argument("--serve-rates", default="50,200,500,1000,2000")
    p.add_argument("--serve-budget-gb", type=float, default=64.0,
                   help="HBM the serving pool may hold (slots per mesh follow from it)")
    p.add_argument("--batch-count", type=int, default=256)
    p.add_argument("--batch-vpb", type=int, default=0, help="batch: vertices per block (0 = autotune)")
    p.add_argument("--no-plain", action="store_true", help="batch: skip the one-at-a-time comparison")
    p.add_argument("--no-patterns", action="store_true",
                   help="c3d only: skip the batched / served / precision summaries added to the line")
    p.add_argument("--launch", default="graph", choices=["graph", "direct"],
                   help="graph: one CUDA-graph launch per solve; direct: kernel by kernel (for ncu)")
    p.add_argument("--prec-modes", default="fp32,mixed", help="prec: which of fp32 / mixed to run")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_meshgen():
    """The synthetic-mesh module, loaded from its file so that importing it does not
    import the product package (the reference arm must not load product code)."""
    import importlib.util
    name = "eikonal_bench_meshgen"
    if name in sys.modules:
        return sys.modules[name]
    spec = importlib.util.spec_from_file_location(name, os.path.join(ROOT, "sci-solver_eikonal_gb300", "meshgen.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules[name] = mod
    spec.loader.exec_module(mod)
    return mod


def bench_config(world):
    """`config` of the headline line, the same dict on both arms."""
    return {"workload": WORKLOAD, "partition": "recursive coordinate bisection", "verts_per_block": 64,
            "max_iterations": MAX_ITERS, "parallelism": f"replicas x{world}",
            "l2": "GPU arm: flushed before every timed solve (512 MB write, outside the timed events); "
                  "CPU arm: the padded block layout (about 170 MB of slot data) exceeds the host caches"}


def build_workload():
    mg = load_meshgen()
    xyz, tets = mg.kuhn_cube(N_GRID, 0.2, seed=1)
    speed = mg.log_uniform_speeds(tets.shape[0], 0.5, 2.0, seed=2)
    metric = (1.0 / (speed.astype(np.float64) ** 2)).astype(np.float32)
    seed = mg.center_vertex(N_GRID)
    return xyz, tets, metric, seed


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"eikonal_clocks_{os.getpid()}_{gpu_index}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        # let nvidia-smi finish its start-up (its first query) before the timed
        # region: a solve that overlapped that start-up once took 60 ms instead of 10
        t0 = time.perf_counter()
        while time.perf_counter() - t0 < 1.5 and self.proc.poll() is None:
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.05)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                rows.append(f)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_sample(xyz, tets, metric, seeds, labels, nb, sample_iters, nthreads=0, precision=32):
    """CPU baseline leg: the oracle (CPU restatement of the reference scheme) on the
    first `sample_iters` outer iterations of the same solve (nthreads 0: every host
    thread).  precision 64 is the FP64 run of the scheme, the error reference."""
    from oracle import oracle as O  # CPU baseline only
    M = O.metrics_from_speeds(tets.shape[0], metric)
    threads = nthreads or O.num_threads()
    sd = list(np.atleast_1d(seeds))
    # the restatement builds its padded block layout on every call (as the
    # reference's solveEikonal does); the rate counts only the outer iterations, as
    # the device rate counts only the solve
    t0 = time.perf_counter()
    r = O.solve3d(xyz, tets, M, labels, nb, sd, max_iters=sample_iters, nthreads=threads, precision=precision)
    dt = time.perf_counter() - t0
    loop = max(O.last_loop_seconds(), 1e-9)
    setup = dt - loop
    return {"value": r["vertex_updates"] / loop, "unit": "vertex-updates/s", "cores": threads, "kind": "port",
            "sample": f"first {r['iterations']} outer iterations of the same solve "
                      f"({r['vertex_updates']} vertex updates in {loop:.2f} s of iterations after "
                      f"{setup:.2f} s of layout set-up, FP{precision})",
            "seconds": dt, "loop_seconds": loop, "setup_seconds": setup, "iterations": r["iterations"],
            "result": r["result"]}


def error_stats(got, ref):
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    rel = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-6)
    return {"max": float(rel.max()), "p99": float(np.percentile(rel, 99)), "mean": float(rel.mean()),
            "vertices_above_1e-5": int((rel > 1e-5).sum())}


def run_reference(args, rank, world):
    if rank != 0:
        return 0
    xyz, tets, metric, seed = build_workload()
    # the same partition as the product's arm (recursive coordinate bisection),
    # from the oracle's restatement of it
    from oracle import oracle as O
    labels, nb = O.partition_rcb(xyz, 64, 3)
    sample_iters = args.cpu_sample_iters or MAX_ITERS
    vals = []
    for i in range(args.warmup + args.steps):
        res = cpu_sample(xyz, tets, metric, seed, labels, nb, sample_iters)
        if i >= args.warmup:
            vals.append(res)
    v = statistics.median(r["value"] for r in vals)
    secs = [r["seconds"] for r in vals]
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "vertex-updates/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.median(secs),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": bench_config(world), "blocks": nb, "step": vals[0]["sample"],
            "cpu_baseline": {"value": v, "unit": "vertex-updates/s", "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"]},
            "e2e": {"value": v, "unit": "vertex-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def aggregate_replicas(torch, total_ms, updates, world, device):
    """Replicas (one independent solve stream per rank, no collective in the solve):
    the job's time is the slowest rank's, its work the sum over ranks."""
    if world <= 1:
        return float(total_ms), float(updates)
    tt = torch.tensor([float(total_ms), float(updates)], dtype=torch.float64, device=device)
    mx = tt.clone()
    torch.distributed.all_reduce(mx, op=torch.distributed.ReduceOp.MAX)
    sm = tt.clone()
    torch.distributed.all_reduce(sm, op=torch.distributed.ReduceOp.SUM)
    return float(mx[0]), float(sm[1])


BATCH_WORKLOAD = ("batching: 256 unit icospheres, subdivision level U{2..6} (162-40,962 verts; seed 3), "
                  "1-8 random seeds each (seed 4), per-triangle speed 1 + 0.5 sin(3x) cos(2y) sin(z)")


def bench_batch(args, E, torch, world, local):
    """Batched vs plain (one solve at a time) on the icosphere batch.  Block size
    and CTA size from the autotuner; plain solves use the same partitions, so the
    batched results must equal them bit for bit (checked)."""
    mg = importlib.import_module("sci-solver_eikonal_gb300.meshgen")
    tune = importlib.import_module("sci-solver_eikonal_gb300.autotune")
    work = mg.batch_workload(args.batch_count)
    solvers = []
    for xyz, faces, speed, seeds in work:
        e = E.Eikonal(True)
        e.set_mesh(xyz, faces)
        e.initSpeedMtxMultipliers(speed)
        e.setSeeds(seeds)
        e.maxIterations_ = MAX_ITERS
        e.directLaunch_ = 1 if args.launch == "direct" else 0
        solvers.append(e)
    nv_total = sum(w[0].shape[0] for w in work)
    t0 = time.perf_counter()
    if args.batch_vpb > 0:
        tuned, batch = tune.tune_batch(solvers, vpb_candidates=(args.batch_vpb,), reps=1)
    else:
        tuned, batch = tune.tune_batch(solvers, reps=2)
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.ExternalStream(batch.stream())

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # batched: device-resident (events around the solve on the batch's stream)
    for _ in range(args.warmup):
        batch.solveEikonal()
    sampler = ClockSampler(local)
    sampler.start()
    barrier()
    times, upd, iters, fim_ms, fim_bytes = [], 0, [], 0.0, 0
    for _ in range(args.steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        batch.solveEikonal()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
        st = batch.stats()
        upd += st["vertex_updates"]
        iters.append(st["iterations"])
        fim_ms += st["fim_kernel_ms"]
        # 2D sweep visit: per slot 3 edge lengths + inverse speed (16 B) + corner ids (8 B)
        fim_bytes += (24 * st["fim_slots"] + 4 * (st["fim_owned"] + st["fim_halo"]) + 4 * st["fim_owned"]
                      + 4 * st["fim_visits"])
    barrier()
    clocks = sampler.stop()
    batched_ms = statistics.median(times)
    n = len(solvers)
    # batched end to end: seeds in, solve, every travel time out (into pinned memory)
    e2e = []
    res_buf = torch.empty(nv_total, dtype=torch.float32, pin_memory=True).numpy()
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        for e, w in zip(solvers, work):
            e.setSeeds(w[3])
        batch.solveEikonal()
        res = batch.getFinalResults(out=res_buf)
        if i >= args.warmup:
            e2e.append(time.perf_counter() - t)
    # plain: the same solves one at a time (same partitions, each its own handle)
    plain_ms, plain_upd, plain_wall = [], 0, []
    mismatch = 0
    for k, e in enumerate([] if args.no_plain else solvers):
        e.solveEikonal()  # upload + graph build
        t = time.perf_counter()
        e.solveEikonal()
        r = e.getFinalResult()
        plain_wall.append(time.perf_counter() - t)
        plain_ms.append(e.stats()["solve_ms"])
        plain_upd += e.stats()["vertex_updates"]
        if not np.array_equal(r.view(np.uint32), res[k].view(np.uint32)):
            mismatch += 1
    plain_total_ms = sum(plain_ms) if plain_ms else float("nan")
    lat = sorted(times)
    peak, peak_src = measured_hbm_peak()
    achieved = fim_bytes / (fim_ms * 1e-3) / 1e9 if fim_ms > 0 else 0.0
    # error against the FP64 run of the same scheme (same partition), on instances
    # spread over the sizes
    from oracle import oracle as O
    order = sorted(range(n), key=lambda k: work[k][0].shape[0])
    err = []
    for k in sorted({order[0], order[n // 3], order[(2 * n) // 3], order[-1]}):
        xyz, faces, speed, seeds = work[k]
        f, obt, off, vfv = solvers[k].triPrep()
        lab, nb = solvers[k].getPartition()
        init = np.full(xyz.shape[0], 1e7, np.float32)
        init[list(seeds)] = 0
        r64 = O.solve2d(xyz, f, (np.float32(1) / speed).astype(np.float32), obt, off, vfv, lab, nb, list(seeds),
                        init, max_iters=MAX_ITERS, precision=64)
        err.append(dict(error_stats(res[k], r64["result"]), vertices=int(xyz.shape[0])))
    return {
        "metric": METRIC, "value": n / (batched_ms * 1e-3), "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": batched_ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": BATCH_WORKLOAD, "instances": n, "vertices": nv_total,
                   "verts_per_block": tuned.verts_per_block, "threads_per_block": tuned.threads_per_block,
                   "iterations_per_step": iters[0], "l2": "inputs resident; results 11 MB",
                   "autotune_s": round(tune_s, 2), "autotune": tuned.table},
        "vertex_updates_per_s": (upd / args.steps) / (batched_ms * 1e-3),
        "plain": {"solves_per_s": n / (plain_total_ms * 1e-3), "ms_total": plain_total_ms,
                  "vertex_updates_per_s": plain_upd / (plain_total_ms * 1e-3),
                  "e2e_solves_per_s": n / sum(plain_wall) if plain_wall else float("nan")},
        "batched_over_plain": (n / (batched_ms * 1e-3)) / (n / (plain_total_ms * 1e-3)),
        "bitwise_mismatches_vs_plain": mismatch,
        "error_vs_fp64_sample": err,
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "e2e": {"value": n / statistics.median(e2e), "unit": "solves/s",
                "h2d_bytes_per_step": int(batch.stats()["h2d_bytes"]), "d2h_bytes_per_step": 4 * nv_total},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_source": peak_src,
                     "kernel": "k_visit2d_slot<false,7> (block sweeps)",
                     "kernel_ms_per_step": fim_ms / args.steps},
        "clocks": clocks,
        # start + 4 kernels per iteration, the graph body running 4 iterations a pass
        "gpu_launches": int(sum(1 + 4 * 4 * ((i + 3) // 4) for i in iters)),
    }


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        return json.load(open(path))["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def launch_dram(name):
    """DRAM bytes (read + write) per launch of the sweep and check kernels over one
    solve, by outer iteration, from a committed ncu summary (data lines
    `iteration sweep_bytes check_bytes`); None when the summary is absent."""
    path = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(path):
        return None
    rows = {}
    for line in open(path):
        f = line.split()
        if len(f) >= 3 and f[0].isdigit():
            rows[int(f[0])] = (float(f[1]), float(f[2]))
    return rows or None


def sweep_bytes(it):
    """Algorithmic bytes of one sweep-kernel launch from its iteration's counters
    (Eikonal.iterationStats columns): per slot 6 float metric terms + 4 u16 corner
    ids (32 B), its sweep memo read and written (16 B each) and its four fp16 apex
    bounds (8 B), owned + halo travel times read (4 B each), owned times written
    (4 B), one block flag (4 B) per visit."""
    return 72 * it[3] + 4 * (it[5] + it[4]) + 4 * it[5] + 4 * it[2]


def check_bytes(it):
    """Algorithmic bytes of one check-kernel launch: per slot the metric terms and
    ids (32 B), its check memo (16 B) and apex bounds (8 B), owned + halo times read,
    one list entry."""
    return 56 * it[7] + 4 * (it[9] + it[8]) + 4 * it[6]


def launch_bytes(its, fused):
    """Algorithmic bytes of every sweep launch and every check launch of one solve,
    by outer iteration.  With the checks inside the sweep kernel (fused), the sweep
    launch of iteration k also runs the checks of iteration k - 1 (row k - 1's check
    columns) and there is no check launch; a block that its check activated is
    swept in the same visit, so its metric terms, ids and bounds (40 B per slot) and
    its owned + halo times are read once (columns 12-15 count those visits)."""
    n = len(its)
    sweep = [sweep_bytes(its[i]) for i in range(n)]
    check = [check_bytes(its[i]) for i in range(n)]
    if fused:
        once = [40 * its[i][13] + 4 * (its[i][14] + its[i][15]) if len(its[i]) > 15 else 0 for i in range(n)]
        return [sweep[i] + (check[i - 1] if i > 0 else 0) - once[i] for i in range(n)], [0] * n
    return sweep, check


def traffic_vs_algorithmic(its, profile, fused):
    """Mean DRAM bytes per launch from the capture beside the mean algorithmic bytes
    of the same launches (same iterations of the same deterministic solve) in this
    run, for the sweep and the check kernel."""
    rows = launch_dram(profile)
    out = {}
    per_launch = launch_bytes(its, fused)
    for k, (col, name) in enumerate(((0, "sweep"), (1, "check"))):
        alg = per_launch[k]
        if rows:
            common = [i for i in sorted(rows) if i < len(its) and rows[i][col] > 0]
            if common:
                dram = sum(rows[i][col] for i in common) / len(common)
                a = sum(alg[i] for i in common) / len(common)
                out[name] = {"traffic": dram, "algorithmic": a, "traffic_over_algorithmic": dram / a if a else None,
                             "launches": len(common)}
                continue
        out[name] = {"traffic": None, "algorithmic": sum(alg) / max(1, sum(1 for x in alg if x > 0)),
                     "traffic_over_algorithmic": None, "launches": 0}
    return out


SERVE_WORKLOAD = ("serving: resident pool of icospheres L5, L6, L7 and L6 with other speeds (2D) and jittered "
                  "Kuhn cubes 33^3, 49^3, 65^3, 97^3 (3D); Poisson arrivals (seed 7), each request a uniform "
                  "pool mesh, 1-16 random seeds and a global speed scale U[0.5, 2]")


def serve_pool(E, mg):
    """The eight pool meshes as configured handles."""
    pool = []
    for lv, phase in ((5, 0.0), (6, 0.0), (7, 0.0), (6, 1.0)):
        xyz, faces = mg.icosphere(lv)
        c = xyz[faces].mean(axis=1).astype(np.float64)
        sp = (1.0 + 0.5 * np.sin(3 * c[:, 0] + phase) * np.cos(2 * c[:, 1]) * np.sin(c[:, 2])).astype(np.float32)
        e = E.Eikonal(True)
        e.set_mesh(xyz, faces)
        e.initSpeedMtxMultipliers(sp)
        e.maxVertsPerBlock_ = 64
        e.maxIterations_ = 1000
        pool.append((e, xyz.shape[0]))
    for k, n in enumerate((33, 49, 65, 97)):
        xyz, tets = mg.kuhn_cube(n, 0.2, seed=20 + k)
        v = mg.log_uniform_speeds(tets.shape[0], 0.5, 2.0, seed=30 + k)
        e = E.Eikonal(False)
        e.set_mesh(xyz, tets)
        e.initSpeedMtxMultipliers((1.0 / (v.astype(np.float64) ** 2)).astype(np.float32))
        e.maxVertsPerBlock_ = 64
        e.maxIterations_ = 1000
        pool.append((e, xyz.shape[0]))
    return pool


def serve_stream(srv, ids, sizes, rate, count, rng):
    """Submits `count` Poisson arrivals at `rate`/s, waits for all, returns the
    completion records."""
    gaps = rng.exponential(1.0 / rate, size=count)
    reqs = []
    for _ in range(count):
        m = int(rng.integers(len(ids)))
        seeds = rng.choice(sizes[m], size=int(rng.integers(1, 17)), replace=False).astype(np.int32)
        reqs.append((m, seeds, float(rng.uniform(0.5, 2.0))))
    t0 = time.perf_counter()
    due = t0
    for (m, seeds, s), g in zip(reqs, gaps):
        due += g
        while True:
            now = time.perf_counter()
            if now >= due:
                break
            time.sleep(min(due - now, 0.001))
        srv.submit(ids[m], seeds, s)
    srv.drain()
    out = []
    while True:
        got = srv.poll(max_items=4096)
        if not got:
            break
        out += got
    return out


def bench_serve(args, E, torch):
    mg = importlib.import_module("sci-solver_eikonal_gb300.meshgen")
    pool = serve_pool(E, mg)
    sizes = [n for _, n in pool]
    rates = [float(r) for r in args.serve_rates.split(",")]
    res = {"metric": METRIC, "unit": "solves/s", "n_gpus": 1, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic", "steps": args.steps, "warmup": args.warmup,
           "config": {"workload": SERVE_WORKLOAD, "rates_per_s": rates, "hbm_budget_gb": args.serve_budget_gb}}
    # server start (pool layouts, arena, graph) and each pool mesh's first request,
    # with the pool meshes' layouts built on the device and on the host (fresh
    # handles each); the first requests' results must be the same bits
    startup, firsts = {}, {}
    for build, dev in (("host_setup", 0), ("device_setup", 1)):
        fresh = serve_pool(E, mg)
        for e, _ in fresh:
            e.deviceSetup_ = dev
        srv = E.EikonalServer(hbm_budget_bytes=int(args.serve_budget_gb * (1 << 30)), keep_results=True)
        t0 = time.perf_counter()
        ids = [srv.add_mesh(e) for e, _ in fresh]
        srv.start()
        start_s = time.perf_counter() - t0
        lat, outs = [], []
        for i in ids:
            t = time.perf_counter()
            rid = srv.submit(i, [0], 1.0)
            srv.drain()
            lat.append(round(1e3 * (time.perf_counter() - t), 3))
            srv.poll(max_items=16)
            outs.append(srv.result(rid, i))
        srv.close()
        firsts[build] = outs
        startup[build] = {"start_s": round(start_s, 3), "first_request_ms_by_mesh": lat}
    startup["bitwise_equal"] = all(np.array_equal(a.view(np.uint32), b.view(np.uint32))
                                   for a, b in zip(firsts["host_setup"], firsts["device_setup"]))
    res["startup"] = startup
    modes = {}
    for mode, inflight in (("served", 0), ("plain", 1)):
        srv = E.EikonalServer(hbm_budget_bytes=int(args.serve_budget_gb * (1 << 30)), max_inflight=inflight)
        t0 = time.perf_counter()
        ids = [srv.add_mesh(e) for e, _ in pool]
        srv.start()
        setup_s = time.perf_counter() - t0
        info = [srv.mesh_info(i) for i in ids]
        rng = np.random.Generator(np.random.PCG64(7))
        # warm-up: one request per pool mesh
        for i in ids:
            srv.submit(i, [0], 1.0)
        srv.drain()
        srv.poll(max_items=4096)
        per_rate = []
        for rate in rates:
            count = int(min(300, max(100, 2 * rate)))
            comp = serve_stream(srv, ids, sizes, rate, count, rng)
            lat = sorted(1e3 * (c["done_s"] - c["submit_s"]) for c in comp)
            span = max(c["done_s"] for c in comp) - min(c["submit_s"] for c in comp)
            per_rate.append({"rate_per_s": rate, "requests": len(comp), "solves_per_s": len(comp) / span,
                             "p50_ms": lat[len(lat) // 2], "p99_ms": lat[min(len(lat) - 1, int(0.99 * len(lat)))],
                             "errors": sum(1 for c in comp if c["status"] != 0)})
            if rate == rates[0]:
                # per pool mesh: median latency at the lowest rate (little queueing)
                per_rate[-1]["p50_ms_by_mesh"] = [
                    statistics.median([1e3 * (c["done_s"] - c["submit_s"]) for c in comp if c["mesh"] == i] or [0.0])
                    for i in ids]
        st = srv.stats()
        srv.close()
        modes[mode] = {"per_rate": per_rate, "setup_s": round(setup_s, 2), "device_bytes": st["device_bytes"],
                       "slots": [x["slots"] for x in info], "device_loops": st["device_loops"],
                       "arena_busy_s": st["busy_s"], "arena_vertex_updates": st["vertex_updates"],
                       "arena_vertex_updates_per_busy_s": [u / b if b > 0 else 0.0
                                                           for u, b in zip(st["vertex_updates"], st["busy_s"])]}
    top = modes["served"]["per_rate"][-1]
    res["value"] = top["solves_per_s"]
    res["ms_per_step"] = 1e3 / top["solves_per_s"]
    res["latency_ms"] = {"p50": top["p50_ms"], "p99": top["p99_ms"]}
    res["served"] = modes["served"]
    res["plain"] = modes["plain"]
    res["served_over_plain"] = top["solves_per_s"] / modes["plain"]["per_rate"][-1]["solves_per_s"]
    res["served_over_plain_per_rate"] = [
        {"rate_per_s": a["rate_per_s"], "ratio": a["solves_per_s"] / b["solves_per_s"]}
        for a, b in zip(modes["served"]["per_rate"], modes["plain"]["per_rate"])]
    res["e2e"] = {"value": top["solves_per_s"], "unit": "solves/s", "note": "requests submitted from the host, "
                  "travel times copied back to pinned host memory before completion"}
    return res


PREC_WORKLOAD = ("precision: 49^3 jittered Kuhn cube with sliver tets (min dihedral < 5 deg, vertices moved "
                 "toward opposite faces, seed 5), per-tet metric R diag(1, a, b) R^T with a, b log-uniform in "
                 "[1, 100] (seed 6), 4 random seeds (seed 9), 64 verts/block")


def bench_prec(args, E, torch):
    mg = importlib.import_module("sci-solver_eikonal_gb300.meshgen")
    t0 = time.perf_counter()
    xyz, tets, sl = mg.sliver_cube(49, 0.10, seed=5)
    M6 = mg.anisotropic_metrics(tets.shape[0], seed=6)
    seeds = np.random.Generator(np.random.PCG64(9)).choice(xyz.shape[0], 4, replace=False).astype(np.int32)
    gen_s = time.perf_counter() - t0
    runs = {}
    modes = [m for m in ("fp32", "mixed") if m in args.prec_modes.split(",")]
    for name in modes:
        e = E.Eikonal(False)
        e.set_mesh(xyz, tets)
        e.initSpeedMtxMultipliers(M6.ravel())
        e.setSeeds(seeds)
        e.maxIterations_ = 1000
        e.keepHistory_ = 0
        e.precisionMode_ = 1 if name == "mixed" else 0
        e.directLaunch_ = 1 if args.launch == "direct" else 0
        e.solveEikonal()
        for _ in range(args.warmup):
            e.solveEikonal()
        ms = []
        for _ in range(args.steps):
            e.solveEikonal()
            ms.append(e.stats()["solve_ms"])
        st = e.stats()
        runs[name] = {"e": e, "ms": statistics.median(ms), "stats": st, "result": e.getFinalResult()}
    lab, nb = runs[modes[0]]["e"].getPartition()
    # CPU baseline leg: the FP64 run of the same scheme, which is also the error reference
    c64 = cpu_sample(xyz, tets, M6.ravel(), seeds, lab, nb, 1000, precision=64)
    ref = c64["result"]

    def err(r):
        return error_stats(r, ref)

    out = {"metric": METRIC, "unit": "vertex-updates/s", "n_gpus": 1, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
           "steps": args.steps, "warmup": args.warmup,
           "config": {"workload": PREC_WORKLOAD, "vertices": int(xyz.shape[0]), "tets": int(tets.shape[0]),
                      "sliver_fraction": float(sl.mean()), "mesh_generation_s": round(gen_s, 1),
                      "kappa_threshold": 1e4}}
    for name in modes:
        r = runs[name]
        st = r["stats"]
        out[name] = {"solve_ms": r["ms"], "iterations": st["iterations"],
                     "vertex_updates_per_s": st["vertex_updates"] / (r["ms"] * 1e-3),
                     "error_vs_fp64": err(r["result"]), "flagged_tets": st["flagged_tets"],
                     "residual_max_rel": st["residual_max_rel"], "residual_vertices": st["residual_vertices"],
                     "residual_below_rel": st["residual_below_rel"], "polish_rounds": st["polish_rounds"],
                     "polish_blocks": st["polish_blocks"]}
    out["value"] = out[modes[-1]]["vertex_updates_per_s"]
    out["ms_per_step"] = runs[modes[-1]]["ms"]
    from oracle import oracle as O  # the FP64 run's own residual, beside the device's
    res64 = O.fp64_residual(xyz, tets, O.metrics_from_speeds(tets.shape[0], M6.ravel()), ref)
    out["fp64_oracle"] = {"seconds": c64["seconds"], "iterations": c64["iterations"], "threads": c64["cores"],
                          "residual_max_rel": res64["lowerable"], "residual_below_rel": res64["below"]}
    out["cpu_baseline"] = {k: c64[k] for k in ("value", "unit", "cores", "kind", "sample")}
    out["e2e"] = None
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    E = importlib.import_module("sci-solver_eikonal_gb300")
    if args.workload == "batch":
        res = bench_batch(args, E, torch, world, local)
        if rank == 0:
            print(json.dumps(res), flush=True)
        return 0
    if args.workload == "prec":
        res = bench_prec(args, E, torch)
        print(json.dumps(res), flush=True)
        return 0
    if args.workload == "serve":
        res = bench_serve(args, E, torch)
        if rank == 0:
            print(json.dumps(res), flush=True)
        return 0
    xyz, tets, metric, seed = build_workload()
    # load the library's kernels once (a small solve), so the first solve below
    # times this mesh's setup rather than the process's module loading
    mg = importlib.import_module("sci-solver_eikonal_gb300.meshgen")
    for dev_setup in (1, 0):
        wx, wt = mg.kuhn_cube(9, 0.2, seed=1)
        w = E.Eikonal(False)
        w.set_mesh(wx, wt)
        w.setSeeds([0])
        w.keepHistory_ = 0
        w.deviceSetup_ = dev_setup
        w.directLaunch_ = 1 if args.launch == "direct" else 0
        w.solveEikonal()
        del w
    e = E.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.initSpeedMtxMultipliers(metric)
    e.setSeeds([seed])
    e.maxVertsPerBlock_ = 64
    e.maxIterations_ = MAX_ITERS
    e.keepHistory_ = 0
    e.directLaunch_ = 1 if args.launch == "direct" else 0
    t0 = time.perf_counter()
    e.solveEikonal()  # partition, layout built on the device, graph build, first solve
    setup_s = time.perf_counter() - t0
    # the same first solve with the block layout built on the host
    eh = E.Eikonal(False)
    eh.set_mesh(xyz, tets)
    eh.initSpeedMtxMultipliers(metric)
    eh.setSeeds([seed])
    eh.maxVertsPerBlock_ = 64
    eh.maxIterations_ = MAX_ITERS
    eh.keepHistory_ = 0
    eh.deviceSetup_ = 0
    t0 = time.perf_counter()
    eh.solveEikonal()
    setup_host_s = time.perf_counter() - t0
    same_as_host = bool(np.array_equal(eh.getFinalResult().view(np.uint32), e.getFinalResult().view(np.uint32)))
    del eh
    st0 = e.stats()
    stream = torch.cuda.ExternalStream(e.stream())
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    # the timed solves record no per-launch telemetry (it costs about 1.5%); the same
    # solve with it, right after, gives the sweep kernel's launch spans and each
    # launch's visit counts (same bits, same launches) for the roofline
    e.telemetry_ = 0
    for _ in range(args.warmup):
        e.solveEikonal()
    sampler = ClockSampler(local)
    sampler.start()
    times, upd, iters = [], 0, []
    barrier()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        e.solveEikonal()
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b))
        st = e.stats()
        upd += st["vertex_updates"]
        iters.append(st["iterations"])
    barrier()
    clocks = sampler.stop()
    e.telemetry_ = 1
    flush.zero_()
    torch.cuda.synchronize()
    e.solveEikonal()
    st = e.stats()
    its = e.iterationStats()
    # the checks run inside the sweep kernel: no check launches, check visits counted
    fused = st["check_launches"] == 0 and st["check_visits"] > 0
    fim_ms, chk_ms = st["fim_kernel_ms"] * args.steps, st["check_kernel_ms"] * args.steps
    fim_bytes = sum(launch_bytes(its, fused)[0]) * args.steps
    # the state initialisation (k_init_state, k_seed_state), the graph's start node,
    # then 3 kernels (sweep with checks, commit, close) or 4 per iteration, the graph
    # body running 4 iterations a pass (loop iterations = sweep launches)
    launches = args.steps * (3 + (3 if fused else 4) * 4 * ((st["fim_launches"] + 3) // 4))
    e.telemetry_ = 0
    total_ms, upd_all = aggregate_replicas(torch, sum(times), upd, world, "cuda")
    value = upd_all / (total_ms * 1e-3)

    # end to end through the C ABI with host buffers
    nv = xyz.shape[0]
    # the travel times come back into pinned host memory (a direct copy, no staging)
    out = torch.empty(nv, dtype=torch.float32, pin_memory=True).numpy()
    seeds = np.array([seed], dtype=np.int32)
    e2e_times = []
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        e.setSeeds(seeds)
        e.solveEikonal()
        e.getFinalResult(out=out)
        dt = time.perf_counter() - t
        if i >= args.warmup:
            e2e_times.append(dt)
    st = e.stats()
    e2e_value = st["vertex_updates"] * len(e2e_times) / sum(e2e_times)
    h2d = st["h2d_bytes"] + seeds.nbytes
    # results, the per-iteration telemetry (12 words per iteration) and the control block
    d2h = 4 * nv + 8 * 12 * (MAX_ITERS + 1) + 256

    if rank != 0:
        return 0
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak = json.load(open(peaks_path))["hbm_gbs"]
        peak_src = "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    achieved = fim_bytes / (fim_ms * 1e-3) / 1e9 if fim_ms > 0 else 0.0
    tva = traffic_vs_algorithmic(its, DRAM_PROFILE, fused)
    lat = sorted(times)
    res = {
        "metric": METRIC, "value": value, "unit": "vertex-updates/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(world),
        "blocks": st0["num_blocks"], "iterations_per_solve": iters[0], "vertex_updates_per_solve": upd // args.steps,
        "launch": args.launch,
        "solves_per_s": world * args.steps / (total_ms * 1e-3),
        "latency_ms": {"p50": lat[len(lat) // 2], "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))]},
        "setup_s": setup_s,
        "first_solve_s": {"device_setup": setup_s, "host_setup": setup_host_s,
                          "bitwise_equal": same_as_host,
                          "note": "first solve of this mesh (partition, layout, upload, graph, solve) in a "
                                  "process whose kernels are loaded"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": tva["sweep"]["traffic"], "peak_source": peak_src,
                     "kernel": ("k_sweep3d (block sweeps and the previous iteration's neighbour checks)"
                                if fused else "k_sweep3d (block sweeps)"),
                     "kernel_ms_per_step": fim_ms / args.steps,
                     "kernel_ms_source": "device-timer span of every sweep launch of one solve with telemetry "
                                         "on, run right after the timed solves (same launches and bits)",
                     "algorithmic_bytes_per_launch": tva["sweep"]["algorithmic"],
                     "traffic_over_algorithmic": tva["sweep"]["traffic_over_algorithmic"],
                     "check_kernel": (None if fused else dict(tva["check"], kernel_ms_per_step=chk_ms / args.steps)),
                     "traffic_source": f"profiles/{DRAM_PROFILE}: ncu dram__bytes_read.sum + dram__bytes_write.sum "
                                       "of every sweep launch of one solve of this workload (kernel by kernel; cold "
                                       "caches), set beside this run's algorithmic bytes of the same launches",
                     "note": "the sweep kernel is bound by CTA barriers and instruction latency in the tet local "
                             "solver, not by HBM",
                     # compute side, from the committed full capture of one sweep launch (outer
                     # iteration 40 of the same solve, kernel-by-kernel mode)
                     "compute": {"bound": "issue", "issue_active_pct": 50.5, "ipc_per_sm": 2.05,
                                 "fma_pipe_pct": 16.0, "alu_pipe_pct": 30.9, "xu_pipe_pct": 7.3,
                                 "top_stall": "barrier",
                                 "source": "ncu --set full capture of one k_sweep3d launch (outer iteration 40) "
                                           "of this workload, summarised under profiles/"}},
        "e2e": {"value": e2e_value, "unit": "vertex-updates/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "ms_per_step": 1e3 * statistics.median(e2e_times),
                "note": "each step re-solves the resident mesh through the C ABI: seeds copied in, the solve, the "
                        "travel times copied out into pinned host memory; the partition and block layout built by the first solve "
                        "(first_solve_s) are kept, whereas the reference's solveEikonal rebuilds them on every "
                        "call"},
        "clocks": clocks,
        "gpu_launches": launches,
    }
    if not args.no_cpu_baseline and world == 1:
        labels, nb = e.getPartition()
        base = cpu_sample(xyz, tets, metric, seed, labels, nb, args.cpu_sample_iters or MAX_ITERS)
        res["cpu_baseline"] = {k: v for k, v in base.items() if k in ("value", "unit", "cores", "kind", "sample")}
        # one host thread, on the first 20 iterations (a bounded sample)
        res["cpu_baseline_1thread"] = {k: v for k, v in cpu_sample(xyz, tets, metric, seed, labels, nb, 20,
                                                                   nthreads=1).items()
                                       if k in ("value", "unit", "cores", "kind", "sample")}
        # the result's error against the FP64 run of the same scheme (same partition)
        f64 = cpu_sample(xyz, tets, metric, seed, labels, nb, MAX_ITERS, precision=64)
        res["error_vs_fp64"] = error_stats(out, f64["result"])
        res["error_vs_fp64"]["fp64_run_s"] = round(f64["seconds"], 2)
    if world == 1 and not args.no_reference_gpu:
        labels, nb = e.getPartition()
        res["reference_gpu"] = reference_gpu_summary(xyz, tets, metric, seed, labels, nb, out)
    if world == 1 and not args.no_patterns:
        res.update(pattern_summaries(args, E, torch, local))
    print(json.dumps(res), flush=True)
    return 0


def reference_gpu_summary(xyz, tets, metric, seed, labels, nb, ours):
    """The reference's own kernels (FIMCuda, CopyOutBack, run_check_neghbor,
    run_reduction built from its sources) under a restatement of its host loop
    (meshFIM3dEikonal.cu:411-542) on the same mesh, metric, seed and partition: one
    solve, its outer loop timed on the host clock (kernels plus the reference's
    per-iteration host round trips; the padded layout set-up timed apart)."""
    from oracle import oracle as O  # reference baseline only
    if O.ref_gpu() is None:
        return {"unavailable": "the reference's kernels were not built (oracle/_ref/ref3d.cubin)"}
    M = O.metrics_from_speeds(tets.shape[0], metric)
    t0 = time.perf_counter()
    r = O.ref_gpu_solve3d(xyz, tets, M, labels, nb, [seed], max_iters=MAX_ITERS)
    total = time.perf_counter() - t0
    loop_s = r["loop_ms"] * 1e-3
    return {"ms_per_solve": r["loop_ms"], "solves_per_s": 1.0 / loop_s,
            "vertex_updates_per_s": r["vertex_updates"] / loop_s, "vertex_updates": r["vertex_updates"],
            "iterations": r["iterations"], "layout_setup_s": round(total - loop_s, 3),
            "bitwise_equal_to_ours": bool(np.array_equal(np.asarray(r["result"]).view(np.uint32),
                                                         np.asarray(ours, np.float32).view(np.uint32))),
            "what": "the reference's CUDA kernels compiled from its sources for sm_103a, one CUDA block per active "
                    "mesh block with one thread per element slot, host round trips every iteration"}


C2D_WORKLOAD = ("plain FIM 2D: 33x33 vertex grid on the unit square, cells split along one diagonal "
                "(1089 verts, 2048 tris), uniform speed 1, seed at vertex 0, 16 verts/block")


def c2d_summary(E):
    """The reference's small 2D case: device solve time, and the result's error
    against the FP64 run of the same scheme (same partition) and against the exact
    Euclidean distance to the seed."""
    from oracle import oracle as O
    mg = importlib.import_module("sci-solver_eikonal_gb300.meshgen")
    xyz, faces = mg.grid2d(33)
    e = E.Eikonal(True)
    e.set_mesh(xyz, faces)
    e.maxVertsPerBlock_ = 16
    e.setSeeds([0])
    e.keepHistory_ = 0
    e.solveEikonal()
    ms = []
    for _ in range(20):
        e.solveEikonal()
        ms.append(e.stats()["solve_ms"])
    got = e.getFinalResult()
    lab, nb = e.getPartition()
    ff, obt, off, vfv = e.triPrep()
    init = np.full(xyz.shape[0], 1e7, np.float32)
    init[0] = 0
    r64 = O.solve2d(xyz, ff, np.ones(ff.shape[0], np.float32), obt, off, vfv, lab, nb, [0], init, precision=64)
    dist = np.linalg.norm(xyz.astype(np.float64) - xyz[0].astype(np.float64), axis=1)
    out = {"workload": C2D_WORKLOAD, "solve_ms_p50": statistics.median(ms), "iterations": e.numIterations(),
           "blocks": int(nb), "error_vs_fp64": error_stats(got, r64["result"]),
           "error_vs_exact_distance": error_stats(got, dist)}
    # the reference's own 2D kernels (FIMCuda, run_check_neighbor, run_reduction built
    # from its sources) under the restatement of its host loop (meshFIM2d_eikonal.cu:
    # 683-816), same mesh, seed and partition (reference baseline only)
    if O.ref_gpu() is None:
        out["reference_gpu"] = {"unavailable": "the reference's kernels were not built (oracle/_ref/ref2d.cubin)"}
    else:
        loops = []
        for _ in range(5):
            r = O.ref_gpu_solve2d(xyz, ff, np.ones(ff.shape[0], np.float32), obt, off, vfv, lab, nb, [0], init,
                                  max_iters=MAX_ITERS)
            loops.append(r["loop_ms"])
        out["reference_gpu"] = {
            "ms_per_solve": statistics.median(loops), "iterations": r["iterations"],
            "bitwise_equal_to_ours": bool(np.array_equal(np.asarray(r["result"], np.float32).view(np.uint32),
                                                         np.asarray(got, np.float32).view(np.uint32))),
            "what": "outer loop of the reference's CUDA kernels compiled from its sources for sm_103a, host round "
                    "trips every iteration, median of 5 solves"}
    return out


def first_solve_2d(E, batch_count=256, vpb=128):
    """First-solve latency of 2D meshes with the layout built on the device and on
    the host: one icosphere of level 7 (163,842 vertices) and the icosphere batch
    (one batch solve over all instances), each on fresh handles in a process whose
    kernels are loaded.  The triangle preparation of set_mesh (orientation, obtuse
    corners, virtual faces; host work in both builds) is timed apart.  The two
    builds must give the same bits."""
    mg = importlib.import_module("sci-solver_eikonal_gb300.meshgen")
    xyz, faces = mg.icosphere(7)
    sp = mg.batch_speed(xyz, faces)
    work = mg.batch_workload(batch_count)
    warm = E.Eikonal(True)
    wx, wf = mg.icosphere(2)
    warm.set_mesh(wx, wf)
    for dev in (1, 0):
        warm.deviceSetup_ = dev
        warm.solveEikonal()
        E.EikonalBatch([warm]).solveEikonal()
    out = {"workload": "icosphere level 7 (163,842 vertices, per-triangle speed 1 + 0.5 sin(3x) cos(2y) sin(z), "
                       f"seed vertex 0) and the batch of {batch_count} icospheres, {vpb} verts/block"}
    res = {}
    for name, dev in (("device_setup", 1), ("host_setup", 0)):
        t0 = time.perf_counter()
        e = E.Eikonal(True)
        e.set_mesh(xyz, faces)
        prep_s = time.perf_counter() - t0
        e.initSpeedMtxMultipliers(sp)
        e.setSeeds([0])
        e.maxVertsPerBlock_ = vpb
        e.deviceSetup_ = dev
        t0 = time.perf_counter()
        e.solveEikonal()
        r = e.getFinalResult()
        one_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        solvers = []
        for wxyz, wfaces, wsp, wseeds in work:
            h = E.Eikonal(True)
            h.set_mesh(wxyz, wfaces)
            h.initSpeedMtxMultipliers(wsp)
            h.setSeeds(wseeds)
            h.maxVertsPerBlock_ = vpb
            h.deviceSetup_ = dev
            solvers.append(h)
        bprep_s = time.perf_counter() - t0
        t0 = time.perf_counter()
        b = E.EikonalBatch(solvers)
        b.solveEikonal()
        rb = b.getFinalResults()
        batch_s = time.perf_counter() - t0
        res[name] = (r, rb)
        out[name] = {"single_first_solve_s": round(one_s, 4), "single_triangle_prep_s": round(prep_s, 4),
                     "single_solve_ms": e.stats()["solve_ms"], "batch_first_solve_s": round(batch_s, 4),
                     "batch_triangle_prep_s": round(bprep_s, 3), "batch_solve_ms": b.stats()["solve_ms"]}
    a, h = res["device_setup"], res["host_setup"]
    out["bitwise_equal"] = bool(np.array_equal(a[0].view(np.uint32), h[0].view(np.uint32)) and all(
        np.array_equal(x.view(np.uint32), y.view(np.uint32)) for x, y in zip(a[1], h[1])))
    out["note"] = ("first solve = partition, block layout, upload, graph and solve (results copied back); "
                   "the triangle preparation is host work in both builds")
    return out


def metis_summary(E, torch):
    """The headline workload on a METIS k-way partition (the reference's partitioner
    kind; the headline uses coordinate bisection): partition time, device solve
    time, vertex updates, and the error against the FP64 run of the scheme on that
    partition."""
    xyz, tets, metric, seed = build_workload()
    e = E.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.initSpeedMtxMultipliers(metric)
    e.setSeeds([seed])
    e.maxVertsPerBlock_ = 64
    e.maxIterations_ = MAX_ITERS
    e.keepHistory_ = 0
    e.partitioner_ = E.PARTITION_METIS
    t0 = time.perf_counter()
    e.solveEikonal()  # METIS on the host, layout on the device, first solve
    first_s = time.perf_counter() - t0
    for _ in range(3):  # the CTA-size choice
        e.solveEikonal()
    ms = []
    for _ in range(10):
        e.solveEikonal()
        ms.append(e.stats()["solve_ms"])
    st = e.stats()
    med = statistics.median(ms)
    lab, nb = e.getPartition()
    f64 = cpu_sample(xyz, tets, metric, seed, lab, nb, MAX_ITERS, precision=64)
    return {"partition": "METIS 5 k-way on the vertex graph", "first_solve_s": round(first_s, 2),
            "solve_ms": med, "solves_per_s": 1e3 / med, "vertex_updates": st["vertex_updates"],
            "vertex_updates_per_s": st["vertex_updates"] / (med * 1e-3), "iterations": st["iterations"],
            "mean_slots_per_block": st["mean_slots_per_block"], "mean_halo_per_block": st["mean_halo_per_block"],
            "error_vs_fp64": error_stats(e.getFinalResult(), f64["result"])}


def pattern_summaries(args, E, torch, local):
    """The batched, served and precision workloads, the small 2D case and the
    headline on a METIS partition, summarised on the same line."""
    out = {}
    try:
        out["metis_partition"] = metis_summary(E, torch)
    except Exception as ex:  # keep the headline line even if a pattern fails
        out["metis_partition"] = {"error": repr(ex)}
    try:
        out["plain_2d"] = c2d_summary(E)
    except Exception as ex:
        out["plain_2d"] = {"error": repr(ex)}
    try:
        out["first_solve_2d"] = first_solve_2d(E)
    except Exception as ex:  # keep the headline line even if a pattern fails
        out["first_solve_2d"] = {"error": repr(ex)}
    try:
        b = bench_batch(args, E, torch, 1, local)
        out["batched"] = {"workload": BATCH_WORKLOAD, "solves_per_s": b["value"],
                          "plain_solves_per_s": b["plain"]["solves_per_s"], "ratio": b["batched_over_plain"],
                          "vertex_updates_per_s": b["vertex_updates_per_s"], "ms_per_batch": b["ms_per_step"],
                          "latency_ms": b["latency_ms"], "e2e_solves_per_s": b["e2e"]["value"],
                          "bitwise_mismatches_vs_plain": b["bitwise_mismatches_vs_plain"],
                          "error_vs_fp64_sample": b["error_vs_fp64_sample"],
                          "verts_per_block": b["config"]["verts_per_block"], "clocks": b["clocks"]}
    except Exception as ex:  # keep the headline line even if a pattern fails
        out["batched"] = {"error": repr(ex)}
    try:
        sv = bench_serve(args, E, torch)
        out["served"] = {"workload": SERVE_WORKLOAD,
                         "per_rate": [{k: r[k] for k in ("rate_per_s", "solves_per_s", "p50_ms", "p99_ms")}
                                      for r in sv["served"]["per_rate"]],
                         "plain_per_rate": [{k: r[k] for k in ("rate_per_s", "solves_per_s", "p50_ms", "p99_ms")}
                                            for r in sv["plain"]["per_rate"]],
                         "ratio_at_top_rate": sv["served_over_plain"],
                         "ratio_per_rate": sv["served_over_plain_per_rate"], "slots": sv["served"]["slots"],
                         "device_bytes": sv["served"]["device_bytes"], "hbm_budget_gb": args.serve_budget_gb,
                         "setup_s": sv["served"]["setup_s"], "startup": sv["startup"],
                         "device_loops": {m: sv[m]["device_loops"] for m in ("served", "plain")},
                         "arena_busy_s": {m: sv[m]["arena_busy_s"] for m in ("served", "plain")},
                         "arena_vertex_updates_per_busy_s": {m: sv[m]["arena_vertex_updates_per_busy_s"]
                                                             for m in ("served", "plain")}}
    except Exception as ex:
        out["served"] = {"error": repr(ex)}
    try:
        pr = bench_prec(args, E, torch)
        out["precision"] = {"workload": PREC_WORKLOAD, "sliver_fraction": pr["config"]["sliver_fraction"],
                            "fp32": {k: pr["fp32"][k] for k in ("solve_ms", "error_vs_fp64")},
                            "mixed": {k: pr["mixed"][k] for k in ("solve_ms", "error_vs_fp64", "flagged_tets",
                                                                  "residual_max_rel", "residual_below_rel",
                                                                  "polish_rounds", "polish_blocks")},
                            "fp64_oracle": pr["fp64_oracle"]}
    except Exception as ex:
        out["precision"] = {"error": repr(ex)}
    return out


if __name__ == "__main__":
    sys.exit(main())
