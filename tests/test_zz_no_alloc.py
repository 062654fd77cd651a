"""The allocation-free 3D entry point (eik_solve3d_noalloc).

It exists for callers that cannot call cudaMalloc (code running during another
component's stream capture, hosts that reserve all device memory up front,
plugins whose application owns the device memory pool).  It must give the same
travel times as the regular entry point (eik_set_mesh ... eik_solve ...
eik_get_result) with the same partition rule: the tests here ask for identical
bits, which is tighter than the 1e-5 relative the parity tests allow for
floating point.  Two calls run back to back to show that the shared scratch array
is cleared between calls.  This file is collected last on purpose.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _regular(eik, xyz, tets, speeds, seeds):
    e = eik.Eikonal(False)
    e.set_mesh(xyz, tets)
    e.initSpeedMtxMultipliers(speeds)
    e.setSeeds(seeds)
    e.maxVertsPerBlock_ = 64
    e.keepHistory_ = 0
    e.solveEikonal()
    return e.getFinalResult(), e.numIterations()


def test_noalloc_matches_regular_entry_point_twice(need_gpu, eik, mg):
    xyz, tets = mg.kuhn_cube(17, 0.2, seed=1)
    s1 = (1.0 / mg.log_uniform_speeds(tets.shape[0], seed=2).astype(np.float64) ** 2).astype(np.float32)
    s2 = (1.0 / mg.log_uniform_speeds(tets.shape[0], seed=9).astype(np.float64) ** 2).astype(np.float32)
    runs = [(s1, [mg.center_vertex(17)]), (s2, [0, xyz.shape[0] - 1])]
    for speeds, seeds in runs:
        got, it = eik.solve3d_noalloc(xyz, tets, speeds, seeds)
        want, it_want = _regular(eik, xyz, tets, speeds, seeds)
        assert it == it_want
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
        assert np.abs(got.astype(np.float64) - want).max() <= 1e-5 * np.abs(want).max()


def test_noalloc_rejects_meshes_beyond_the_scratch_size(need_gpu, eik, mg):
    xyz, tets = mg.kuhn_cube(65, 0.2, seed=1)
    with pytest.raises(eik.EikonalError) as ex:
        eik.solve3d_noalloc(xyz, tets)
    assert ex.value.code == 5
    assert "too large" in str(ex.value)


def _case(mg):
    xyz, tets = mg.kuhn_cube(13, 0.2, seed=1)
    sp = (1.0 / mg.log_uniform_speeds(tets.shape[0], seed=2).astype(np.float64) ** 2).astype(np.float32)
    return xyz, tets, sp, [mg.center_vertex(13)]


def test_noalloc_call_allocates_no_device_memory(need_gpu, eik, mg):
    """After a first call (which loads the kernels and looks up the array's
    address), a call leaves the device's free memory exactly as it found it."""
    import torch
    xyz, tets, sp, seeds = _case(mg)
    want, _ = eik.solve3d_noalloc(xyz, tets, sp, seeds)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    got, _ = eik.solve3d_noalloc(xyz, tets, sp, seeds)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_noalloc_runs_while_another_stream_is_captured(need_gpu, eik, mg):
    """The use the entry point exists for: a component is capturing its stream into
    a CUDA graph (thread-local capture mode) while this library solves on a
    non-blocking stream of its own from another thread.  The capture must survive
    (a cudaMalloc or a legacy-stream operation would break it) and the solve must
    give the same bits as outside the capture."""
    import threading
    import torch
    xyz, tets, sp, seeds = _case(mg)
    want, it_want = eik.solve3d_noalloc(xyz, tets, sp, seeds)  # first call: before any capture
    side = torch.cuda.Stream()  # PyTorch creates its streams non-blocking
    cap = torch.cuda.Stream()
    x = torch.zeros(64, device="cuda")
    torch.cuda.synchronize()
    result = {}

    def worker():
        try:
            result["out"] = eik.solve3d_noalloc(xyz, tets, sp, seeds, stream=side.cuda_stream)
        except Exception as ex:  # reported below
            result["err"] = ex

    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=cap, capture_error_mode="thread_local"):
        x.add_(1.0)
        t = threading.Thread(target=worker)
        t.start()
        t.join()
        still_capturing = torch.cuda.is_current_stream_capturing()
        x.mul_(3.0)
    g.replay()
    torch.cuda.synchronize()
    assert "err" not in result, result.get("err")
    assert still_capturing
    assert torch.all(x == 3.0)
    got, it = result["out"]
    assert it == it_want
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
