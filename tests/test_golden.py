"""The oracle against the committed closed-form fixtures (tests/golden)."""
from oracle import p3dfft_oracle as orc

import golden_cases


class _Oracle:
    def __init__(self, nx, ny, nz):
        self.p = orc.OraclePlan(nx, ny, nz)

    def ftran(self, a, op):
        return self.p.ftran_r2c(a, op)

    def btran(self, c, op):
        return self.p.btran_c2r(c, op)

    def cheby(self, a, lz):
        return self.p.cheby(a, lz)


def test_oracle_matches_golden_fixtures():
    golden_cases.check_all(_Oracle, 1e-13)


def test_fixtures_are_current():
    # the committed file is what make_golden.py writes
    import importlib.util
    import os

    import numpy as np
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(golden_cases.GOLDEN), "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = golden_cases.load()
    a, b = mg.sine(14, 26, 38)
    assert np.array_equal(g["sine_14x26x38_in"], a) and np.array_equal(g["sine_14x26x38_out"], b)
    a, b = mg.dct(12, 8, 17, 5)
    assert np.array_equal(g["dct_12x8x17_m5_in"], a) and np.array_equal(g["dct_12x8x17_m5_out"], b)
