"""The oracle reproduces the committed golden vectors (tests/golden/*.npz, written by
tests/golden/make_golden.py from the same oracle).  Catches any drift of the CPU restatement;
relative L2 <= 1e-13 per field (compiler contraction of a*b + c may differ between builds)."""
import os

import numpy as np
import pytest

from conftest import ROOT

GOLD = os.path.join(ROOT, "tests", "golden")


def _mg():
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLD, "make_golden.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


@pytest.mark.parametrize("name", ["heve_C1_3x3x3", "hevi_C1_3x3x3", "hevi_C2_2x2x2", "trc_T1_4x4x3"])
def test_oracle_matches_golden(name):
    mg = _mg()
    ref = np.load(os.path.join(GOLD, name + ".npz"))
    got = mg.oracle_outputs(mg.golden_cases()[name])
    assert sorted(got) == sorted(ref.files)
    for k in ref.files:
        r, g = ref[k], got[k]
        assert r.shape == g.shape
        if k == "q":  # per variable; DDENS/DRHOT are deviations of size 1e-3..1e-1 of the totals
            for v in range(5):
                assert np.linalg.norm(g[v] - r[v]) <= 1e-13 * max(np.linalg.norm(r[v]), 1e-300) + 1e-15, (k, v)
        else:
            assert np.linalg.norm(g - r) <= 1e-13 * np.linalg.norm(r), k
