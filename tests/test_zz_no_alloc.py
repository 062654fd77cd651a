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
