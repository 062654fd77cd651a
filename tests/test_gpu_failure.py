"""Failure paths on the GPU without faulting it: a bounded device wait that gives
up and reports, and server requests cancelled while queued or running.  The
injected faults are host-side or a wait for a copy that is never issued; no test
here traps, faults or hangs a GPU."""
import time

import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_the_context_stays_usable(need_gpu, eik, golden):
    t0 = time.perf_counter()
    rc, waited_ms = eik.selftest_wait_timeout()
    wall = time.perf_counter() - t0
    assert rc == 6, rc  # EIK_ERR_DEVICE: the wait expired and said so
    assert 900.0 <= waited_ms <= 5000.0, waited_ms
    assert wall < 30.0
    # the same process still solves: the reference's 8-tet ball known answer
    e = eik.Eikonal(False)
    e.set_mesh(golden["sphere8_xyz"], golden["sphere8_tets"])
    e.maxBlocks_ = 100
    e.solveEikonal()
    r = e.getFinalResult()
    assert r[0] == 0.0 and np.all(np.abs(r[1:] - np.float32(19.58)) <= 4 * np.spacing(np.float32(19.58)))


def _cube(eik, mg, n, seed):
    xyz, tets = mg.kuhn_cube(n, 0.2, seed=seed)
    v = mg.log_uniform_speeds(tets.shape[0], seed=seed + 1)
    metric = (1.0 / v.astype(np.float64) ** 2).astype(np.float32)
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.initSpeedMtxMultipliers(metric)
    e.maxIterations_ = 1000
    return e, xyz, tets, metric


def test_server_cancels_queued_and_running_requests(need_gpu, eik, mg):
    e, xyz, tets, metric = _cube(eik, mg, 33, 5)
    srv = eik.EikonalServer(hbm_budget_bytes=1 << 30, keep_results=True)
    mid = srv.add_mesh(e, slots=1)  # one slot: later requests queue behind the first
    srv.start()
    r_run = srv.submit(mid, [0], 1.0)
    r_q1 = srv.submit(mid, [5], 1.0)
    r_q2 = srv.submit(mid, [77], 1.0)
    srv.cancel(r_q1)                 # still queued
    srv.cancel(r_run)                # running (or just finished: either completes it)
    with pytest.raises(eik.EikonalError):
        srv.cancel(10 ** 9)          # unknown id
    srv.drain(timeout_ms=120000)
    done = {c["id"]: c for c in srv.poll()}
    assert done[r_q1]["status"] == 8          # EIK_ERR_CANCELLED
    assert done[r_run]["status"] in (0, 8)
    assert done[r_q2]["status"] == 0
    # the slot freed by the cancellations serves the next request correctly
    got = srv.result(r_q2, mid)
    plain = eik.Eikonal(False)
    plain.set_mesh(xyz, tets)
    plain.initSpeedMtxMultipliers(metric)
    plain.maxIterations_ = 1000
    plain.setSeeds([77])
    plain.solveEikonal()
    assert bits_equal(got, plain.getFinalResult())
    r_after = srv.submit(mid, [1000], 1.5)
    srv.drain(timeout_ms=120000)
    assert srv.poll()[0]["status"] == 0
    plain.initSpeedMtxMultipliers(metric * np.float32(1.0 / (float(np.float32(1.5)) ** 2)))
    plain.setSeeds([1000])
    plain.solveEikonal()
    assert bits_equal(srv.result(r_after, mid), plain.getFinalResult())
    srv.close()
