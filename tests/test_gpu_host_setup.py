"""Set-up on the GPU machine against the reference's own host code.

tests/golden/ref_host_setup.npz holds the outputs of the reference's host set-up
compiled from its sources (2D: meshFIM2dEikonal::SetMesh's mesh preparation; 3D:
TetMesh::init + gettetmem; see tests/test_host_setup_pin.py).  Here the values
the solver actually uses must equal them bit for bit:
  * 3D: the metric edge products in the device's block layout, built on the
    device and built on this machine's host (an aarch64 host, where gcc's default
    would fuse the products the reference's x86-64 build rounds separately);
  * 2D: the mesh preparation on this machine's host, the one the 2D layout uses.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, bits_equal

pytestmark = pytest.mark.gpu


def _fx():
    return np.load(os.path.join(GOLDEN, "ref_host_setup.npz"))


def _names(fx, dim):
    names = sorted({k.rsplit("_", 1)[0] for k in fx.files if k.endswith("_xyz")})
    return [n for n in names if fx[n + "_elems"].shape[1] == dim + 1]


@pytest.mark.parametrize("device_setup", [1, 0])
def test_device_layout_gram_equals_reference_host_build(need_gpu, eik, device_setup):
    fx = _fx()
    names = _names(fx, 3)
    assert len(names) == 4
    for name in names:
        e = eik.Eikonal(False)
        e.set_mesh(fx[name + "_xyz"], fx[name + "_elems"])
        if name + "_speeds" in fx.files:
            e.initSpeedMtxMultipliers(fx[name + "_speeds"])
        e.deviceSetup_ = device_setup
        e.maxIterations_ = 3
        e.solveEikonal()
        assert bits_equal(e.tetGram(from_device=True), fx[name + "_gram"]), name


def test_2d_prep_on_this_host_equals_reference_host_build(need_gpu, eik):
    fx = _fx()
    names = _names(fx, 2)
    assert len(names) == 5
    for name in names:
        e = eik.Eikonal(True)
        e.set_mesh(fx[name + "_xyz"], fx[name + "_elems"])
        if name + "_speeds" in fx.files:
            e.initSpeedMtxMultipliers(fx[name + "_speeds"])
        e.maxIterations_ = 3
        e.solveEikonal()
        f, _, off, vfv = e.triPrep()
        ed, si, ved, vsi = e.triPrepValues()
        assert np.array_equal(f, fx[name + "_faces"]), name
        assert np.array_equal(np.diff(off), fx[name + "_vf_count"]), name
        assert np.array_equal(vfv, fx[name + "_vf_verts"]), name
        for got, key in ((ed, "edges"), (si, "speed_inv"), (ved, "vf_edges"), (vsi, "vf_speed_inv")):
            assert bits_equal(got, fx[name + "_" + key]), (name, key)
