"""The steps either side of the path, host side: the contribution list of the time-series
injection matrix (restated from the reference's build_sbus_matrix) and the oracle's
_fill_sbus reproduce the reference's own output bit for bit (golden_sbus.npz, made by
tests/golden/make_golden_sbus.py from the reference's p3s/timeseries.py)."""

import os

import numpy as np

from oracle.postproc import fill_sbus
from p3s_gb300.timeseries import contributions

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "golden_sbus.npz")


def golden_inputs():
    d = np.load(GOLDEN)
    elements = {}
    for k in d.files:
        if "__" in k and not k.startswith("ts__"):
            name, col = k.split("__")
            elements.setdefault(name, {})[col] = d[k]
    ts = {(k.split("__")[1], k.split("__")[2]): d[k] for k in d.files if k.startswith("ts__")}
    return d, elements, ts


def test_oracle_sbus_matches_the_reference_bit_for_bit():
    d, elements, ts = golden_inputs()
    T, ptr, row, coef, base, imag, series = contributions(len(d["s0"]), elements, ts, float(d["sn_mva"]))
    assert T == d["Sbus"].shape[1] == 48  # the shortest series sets T
    assert ptr[-1] == len(row) and (np.diff(ptr) >= 0).all()
    S = fill_sbus(d["s0"], ptr, row, coef, base, imag, series)
    assert np.array_equal(S, d["Sbus"])
    # an out-of-service load injects nothing whatever its series says
    load = elements["load"]
    off = np.nonzero(~load["in_service"].astype(bool) & (load["bus"] >= 0))[0]
    assert len(off) > 0
