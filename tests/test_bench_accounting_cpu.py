"""bench.py's algorithmic bytes per launch (the numerator of roofline.achieved),
checked on hand-made iteration rows (Eikonal.iterationStats columns)."""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _row(fim=(0, 0, 0, 0), chk=(0, 0, 0, 0), fused=(0, 0, 0, 0)):
    # fim_ns, check_ns, sweep visits/slots/halo/owned, check visits/slots/halo/owned,
    # fim_start_ns, check_start_ns, fused visits/slots/halo/owned
    return [0, 0, *fim, *chk, 0, -1, *fused]


def test_sweep_and_check_bytes_per_visit():
    sys.path.insert(0, ROOT)
    import bench
    it = _row(fim=(2, 100, 30, 10), chk=(3, 50, 20, 5))
    # sweeps: 72 B per slot, 4 B per owned and halo time read, 4 B per owned time
    # written, 4 B per visit
    assert bench.sweep_bytes(it) == 72 * 100 + 4 * (10 + 30) + 4 * 10 + 4 * 2
    # checks: 56 B per slot, 4 B per owned and halo time, 4 B per visit
    assert bench.check_bytes(it) == 56 * 50 + 4 * (5 + 20) + 4 * 3


def test_fused_launch_bytes():
    sys.path.insert(0, ROOT)
    import bench
    its = np.array([_row(fim=(1, 10, 4, 2), chk=(2, 8, 3, 1)),
                    _row(fim=(3, 30, 9, 6), chk=(1, 5, 2, 1), fused=(1, 7, 3, 2))], dtype=np.int64)
    sweep, check = bench.launch_bytes(its, fused=False)
    assert sweep == [bench.sweep_bytes(its[0]), bench.sweep_bytes(its[1])]
    assert check == [bench.check_bytes(its[0]), bench.check_bytes(its[1])]
    sweep, check = bench.launch_bytes(its, fused=True)
    # launch k runs the sweeps of iteration k and the checks of iteration k - 1; a
    # block swept after its own check is read once (40 B per slot and its times)
    assert sweep[0] == bench.sweep_bytes(its[0])
    assert sweep[1] == bench.sweep_bytes(its[1]) + bench.check_bytes(its[0]) - (40 * 7 + 4 * (3 + 2))
    assert check == [0, 0]
