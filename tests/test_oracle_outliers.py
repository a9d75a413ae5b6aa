"""The oracle's restatement of isOutlier (CPU)."""
import os

import numpy as np

import oracle_py as O
import plume


def test_far_ions_are_outliers_and_plume_ions_are_not():
    s = plume.make_plume(4001, 1e-6, 11)
    s["x"][[5, 17]] += [[0.0, 0.0, 4e-6], [0.0, 3e-7, 0.0]]
    s["status"][100] = 0
    s["status"][101] = -1
    f, c = O.outliers(s)
    assert c == 2 and f[5] == 1 and f[17] == 1
    assert f[100] == -1 and f[101] == -1
    assert np.count_nonzero(f == 0) == 4001 - 4


def test_true_median_rule():
    # even count: the median is the mean of the two middle values; MAD of the
    # deviations the same way; x = 10 is then 3.4 scaled deviations away
    x = np.array([0.0, 1.0, 2.0, 3.0, 4.0, 10.0])
    s = {"x": np.stack([x, np.zeros(6), np.zeros(6)], 1), "status": np.ones(6, np.int32)}
    f, c = O.outliers(s)
    med = 2.5
    dev = np.abs(x - med)
    mad = 1.482602218505602 * np.median(dev)
    expect = ((dev / mad) >= 3).astype(np.int32)
    np.testing.assert_array_equal(f, expect)
    assert c == 1 and f[5] == 1


def test_matches_reference_isoutlier_fixture(golden_dir):
    """Flags of the reference's own DomainBoundsFunction::isOutlier, run by
    tests/golden/make_golden.py, odd and even particle counts."""
    d = np.load(os.path.join(golden_dir, "outliers.npz"))
    for key in ("n2001", "n2000"):
        st = plume.from_ref32(d[f"{key}_pos4"], d[f"{key}_vel4"], d[f"{key}_acc4"], d[f"{key}_tinj"])
        f, c = O.outliers(st)
        np.testing.assert_array_equal(f, d[f"{key}_flags"])
        assert c == int(d[f"{key}_count"])
