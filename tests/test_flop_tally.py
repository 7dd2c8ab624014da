"""The algorithmic FLOP count the benchmark divides by (recorded in the FP64
stage-kernel profile summary) is the oracle's current operation tally."""
import ctypes as C
import os

import numpy as np

from oracle import oracle_py

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def tally(flux=0, limiter=3, rk=3):
    lib = oracle_py.load(False)
    lib.hco_flop_tally.argtypes = [C.c_int, C.c_int, C.c_int, np.ctypeslib.ndpointer(np.float64, flags="C")]
    out = np.zeros(8)
    lib.hco_flop_tally(flux, limiter, rk, out)
    return out


def test_recorded_flops_match_oracle_tally():
    rec = None
    for line in open(os.path.join(ROOT, "profiles", "stage_kernel_fp64_ogrid.md")):
        if line.startswith("algorithmic_flops_per_cell_stage:"):
            rec = float(line.split(":", 1)[1].split()[0])
    assert rec is not None
    out = tally()
    assert abs(out[0] - rec) < 0.05, (out[0], rec)
    assert abs(out[1] + out[2] + out[3] + out[4] + out[5] - out[0]) < 1e-9


def test_tally_orders_fluxes():
    roe, rus = tally(0)[0], tally(4)[0]
    assert roe > rus > 0
