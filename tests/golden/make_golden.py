"""Writes the committed summary of the reference's golden Orszag-Tang state.

Source: tests/mhd_tests/final_state_orszag_tang.npz of leo1200/astronomix
0.5.1 (the FP64 final state of tests/mhd_tests/orszag_tang.py: 200^2 cells on
[0, 2 pi]^2, HLL, MINMOD, C_cfl 0.4, t = 3).  The summary keeps the shape, the
per-row sums, minima and maxima, and the density on every 8th cell in each
direction, small enough to commit.  Run from the repository root with the
reference's source tree as the argument (or in AMX_REFERENCE_PATH):

    python tests/golden/make_golden.py /path/to/astronomix-checkout
"""
import json
import os
import sys

import numpy as np


def main(ref_root):
    g = np.load(os.path.join(ref_root, "tests", "mhd_tests", "final_state_orszag_tang.npz"))["final_state"]
    out = {
        "source": "tests/mhd_tests/final_state_orszag_tang.npz",
        "shape": list(g.shape),
        "sum_rho": float(g[0].sum()),
        "row_sums": [float(v) for v in g.reshape(g.shape[0], -1).sum(1)],
        "row_min": [float(v) for v in g.reshape(g.shape[0], -1).min(1)],
        "row_max": [float(v) for v in g.reshape(g.shape[0], -1).max(1)],
        "rho_every_8": g[0][::8, ::8].tolist(),
    }
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "orszag_tang_200_t3_summary.json"), "w") as f:
        json.dump(out, f)


if __name__ == "__main__":
    path = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("AMX_REFERENCE_PATH")
    if not path:
        sys.exit("usage: make_golden.py <reference source tree>")
    main(path)
