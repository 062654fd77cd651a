"""Request server (eik_server_*): results in the mix equal results alone, and both
equal a plain solve of the same request (speeds / metric scaled the same way).
The server has no counterpart in the reference; the plain solve it is held to is
the one the other GPU tests pin against the reference's kernels."""
import time

import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


def _pool(eik, mg):
    """Two 2D icospheres and two 3D jittered cubes, each as a configured handle
    plus what a plain solve needs to rebuild a request."""
    pool = []
    for lv in (3, 4):
        xyz, faces = mg.icosphere(lv)
        sp = mg.batch_speed(xyz, faces)
        e = eik.Eikonal(True)
        e.set_mesh(xyz, faces)
        e.initSpeedMtxMultipliers(sp)
        e.maxVertsPerBlock_ = 32
        pool.append({"dim": 2, "solver": e, "xyz": xyz, "elems": faces, "coef": sp, "vpb": 32})
    for n, sd in ((9, 1), (13, 2)):
        xyz, tets = mg.kuhn_cube(n, 0.2, seed=sd)
        v = mg.log_uniform_speeds(tets.shape[0], seed=sd + 10)
        metric = (1.0 / v.astype(np.float64) ** 2).astype(np.float32)
        e = eik.Eikonal(False)
        e.set_mesh(xyz, tets)
        e.initSpeedMtxMultipliers(metric)
        e.maxVertsPerBlock_ = 64
        pool.append({"dim": 3, "solver": e, "xyz": xyz, "elems": tets, "coef": metric, "vpb": 64})
    return pool


def _plain(eik, p, seeds, scale):
    e = eik.Eikonal(p["dim"] == 2)
    e.set_mesh(p["xyz"], p["elems"])
    if p["dim"] == 2:
        e.initSpeedMtxMultipliers(p["coef"] * np.float32(scale))
    else:
        k = np.float32(1.0 / (float(np.float32(scale)) ** 2))
        e.initSpeedMtxMultipliers(p["coef"] * k)
    e.maxVertsPerBlock_ = p["vpb"]
    e.setSeeds(seeds)
    e.solveEikonal()
    return e.getFinalResult(), e.numIterations()


def _requests(pool, count, seed):
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(count):
        m = int(rng.integers(len(pool)))
        nv = pool[m]["xyz"].shape[0]
        seeds = rng.choice(nv, size=int(rng.integers(1, 17)), replace=False).astype(np.int32)
        reqs.append((m, seeds, float(np.float32(rng.uniform(0.5, 2.0)))))
    return reqs


def _serve(eik, pool, reqs, max_inflight, slots=0, stagger_s=0.0):
    srv = eik.EikonalServer(hbm_budget_bytes=1 << 30, max_inflight=max_inflight, keep_results=True)
    ids = [srv.add_mesh(p["solver"], slots=slots) for p in pool]
    srv.start()
    rid = []
    for k, (m, seeds, s) in enumerate(reqs):
        rid.append(srv.submit(ids[m], seeds, s))
        if stagger_s and k % 3 == 2:
            time.sleep(stagger_s)
    srv.drain(timeout_ms=120000)
    comp = {}
    while True:
        got = srv.poll(wait_ms=0)
        if not got:
            break
        for c in got:
            comp[c["id"]] = c
    out = []
    for r, (m, _, _) in zip(rid, reqs):
        assert comp[r]["status"] == 0
        out.append((srv.result(r, ids[m]), comp[r]["iterations"]))
    st = srv.stats()
    srv.close()
    return out, st


def test_mix_equals_alone_equals_plain(need_gpu, eik, mg):
    pool = _pool(eik, mg)
    reqs = _requests(pool, 24, seed=7)
    mix, st = _serve(eik, pool, reqs, max_inflight=0)
    assert st["completed"] == len(reqs) and st["queued"] == 0 and st["running"] == 0
    alone, st1 = _serve(eik, pool, reqs, max_inflight=1)
    for i, ((rm, im), (ra, ia)) in enumerate(zip(mix, alone)):
        assert im == ia, i
        assert bits_equal(rm, ra), i
    # the plain drop-in solve of the same request (first few of each dimension)
    for i, (m, seeds, s) in enumerate(reqs[:12]):
        want, it = _plain(eik, pool[m], seeds, s)
        assert it == mix[i][1], (i, it, mix[i][1])
        assert bits_equal(mix[i][0], want), i


def test_staggered_arrivals_and_single_slots(need_gpu, eik, mg):
    """Requests arriving while others run, with one slot per mesh (queueing)."""
    pool = _pool(eik, mg)
    reqs = _requests(pool, 15, seed=8)
    got, st = _serve(eik, pool, reqs, max_inflight=0, slots=1, stagger_s=0.002)
    assert st["slots_2d"] == 2 and st["slots_3d"] == 2
    for i, (m, seeds, s) in enumerate(reqs):
        want, it = _plain(eik, pool[m], seeds, s)
        assert got[i][1] == it, i
        assert bits_equal(got[i][0], want), i


def test_submit_rejects_bad_requests(need_gpu, eik, mg):
    pool = _pool(eik, mg)[:1]
    srv = eik.EikonalServer(hbm_budget_bytes=1 << 28, keep_results=True)
    mid = srv.add_mesh(pool[0]["solver"])
    srv.start()
    with pytest.raises(eik.EikonalError):
        srv.submit(mid, [], 1.0)
    with pytest.raises(eik.EikonalError):
        srv.submit(mid, [10 ** 7], 1.0)
    with pytest.raises(eik.EikonalError):
        srv.submit(mid, [0], -1.0)
    with pytest.raises(eik.EikonalError):
        srv.submit(mid + 1, [0], 1.0)
    r = srv.submit(mid, [0], 1.0)
    srv.drain(timeout_ms=60000)
    c = srv.poll()
    assert len(c) == 1 and c[0]["id"] == r and c[0]["status"] == 0
    srv.close()


def test_device_and_host_built_arenas_agree(need_gpu, eik, mg):
    """Pool meshes whose handles build on the device are replicated into the arena
    on the device; host-built ones are concatenated on the host; an arena holding
    both brings the device-built ones back to the host first.  All three give the
    same slot sizes and the same bits."""
    reqs = None
    runs = []
    for mode in ("device", "host", "mixed"):
        pool = _pool(eik, mg)
        for k, p in enumerate(pool):
            p["solver"].deviceSetup_ = {"device": 1, "host": 0, "mixed": k % 2}[mode]
        if reqs is None:
            reqs = _requests(pool, 16, seed=9)
        srv = eik.EikonalServer(hbm_budget_bytes=1 << 30)
        ids = [srv.add_mesh(p["solver"]) for p in pool]
        info = [srv.mesh_info(i) for i in ids]
        srv.close()
        out, st = _serve(eik, pool, reqs, max_inflight=0)
        runs.append((info, out))
    for info, out in runs[1:]:
        assert [x["device_bytes"] for x in info] == [x["device_bytes"] for x in runs[0][0]]
        for i, ((ra, ia), (rb, ib)) in enumerate(zip(runs[0][1], out)):
            assert ia == ib, i
            assert bits_equal(ra, rb), i
