"""Fits the fused-multiply-add masks of the reference kernel's tet update
(TEST INFRASTRUCTURE; the product's tet_update_x takes the masks it prints).

    python oracle/fit_tet_fusion.py --collect out.npz   # on a GPU machine: run the
        # reference's FIMCuda on single-tet blocks (oracle/_ref/ref3d.cubin) and save
        # the inputs and outputs
    python oracle/fit_tet_fusion.py out.npz             # fit and print the masks

The CPU model (tet_fusion_model.hpp) has one switch per sum or difference of two
products (which product nvcc fused).  Starting from all-zero masks, every switch
is flipped in turn and kept when it lowers the number of outputs that differ from
the reference kernel's, until a pass changes nothing; then each switch is flipped
once more to report the ones the data leave undetermined.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
NSITES = 51


def collect(path, n=200000, seed=2024):
    import importlib
    from oracle import oracle as O
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "tests"))
    mg = importlib.import_module("sci-solver_eikonal_gb300.meshgen")
    from test_gpu_parity import _tet_block_cases
    inp = _tet_block_cases(np.random.default_rng(seed), mg, n)
    out = O.ref_gpu_tet_blocks(inp)
    np.savez_compressed(path, inp=inp, out=out)
    print(f"{inp.shape[0]} cases, {np.mean(out < inp[:, :4]):.3f} of the vertices lowered")


def fit(path):
    from oracle import oracle as O
    d = np.load(path)
    inp, out = d["inp"], d["out"]
    masks = []
    for k in range(4):
        m = 0
        best = O.tet_fusion_mismatch(inp, out, k, m)
        changed = True
        while changed and best:
            changed = False
            for s in range(NSITES):
                c = O.tet_fusion_mismatch(inp, out, k, m ^ (1 << s))
                if c < best:
                    m, best, changed = m ^ (1 << s), c, True
        loose = [s for s in range(NSITES) if O.tet_fusion_mismatch(inp, out, k, m ^ (1 << s)) == best]
        print(f"apex {'ABCD'[k]}: mask {m:#x}, {best} of {inp.shape[0]} outputs differ; "
              f"sites the data leave open: {loose}")
        masks.append(m)
    return masks


if __name__ == "__main__":
    if len(sys.argv) > 2 and sys.argv[1] == "--collect":
        collect(sys.argv[2])
    elif len(sys.argv) > 1:
        fit(sys.argv[1])
    else:
        print(__doc__)
