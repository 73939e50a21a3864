"""The oracle against its committed golden results (tests/golden/make_golden.py):
one remap interval at ne=2 with 2 tracers.  Inputs come from numpy's libm, which may
differ in the last bit between hosts, hence a 1e-11 relative bound rather than bit
equality."""
import os

import numpy as np

import hxtest as H

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "oracle_ne2_q2.npz")


def test_oracle_matches_golden(oracle_path):
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "make_golden", os.path.join(os.path.dirname(GOLDEN), "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    got = mg.run_case()
    ref = np.load(GOLDEN)
    assert set(ref.files) == set(got)
    for k in ref.files:
        a, b = got[k], ref[k]
        den = max(float(np.max(np.abs(b))), 1e-300)
        assert float(np.max(np.abs(a - b))) / den < 1e-11, k
