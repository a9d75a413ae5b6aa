"""FMM variants of the reference's FmmType (structures.h:283-288): treecode
(multipoles evaluated at the particles) and the outlier variants (outliers
found by the median-absolute-deviation rule of isOutlier and summed
directly).  Forces against the oracle's FP64 direct sum, outlier flags
against the oracle's restatement of isOutlier."""
import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv

pytestmark = pytest.mark.gpu

EPS20 = 1e-20


def fmm(**kw):
    base = dict(softening2=EPS20, method=sv.FMM, fmm_order=8, fmm_ws=2)
    base.update(kw)
    return sv.ForceMethod(**base)


def with_outliers(n, seed):
    s = plume.make_plume(n, 1e-6, seed)
    rng = np.random.default_rng(seed)
    # a handful of ions far off the plume (several plume lengths away)
    k = 7
    s["x"][:k] += rng.normal(size=(k, 3)) * 20e-6
    s["status"][3] = 2
    return s


@pytest.mark.parametrize("sym", [sv.SYM_NONE, sv.SYM_ROTATIONAL])
def test_treecode_matches_fp64_direct(sym):
    s = plume.make_plume(16384, 1e-6, 5100 + sym)
    with fmm(fmm_type=sv.TREECODE, symmetry=sym) as f:
        f.upload(s)
        a = f.accel()
    ref = O.direct_f64(s, EPS20, sym=sym)
    err = O.rel_l2(a, ref, s["status"])[0]
    assert err <= 2e-5, err


def test_treecode_agrees_with_fmm():
    s = plume.make_plume(20000, 2e-6, 5200)
    with fmm(fmm_type=sv.TREECODE) as t, fmm() as f:
        t.upload(s)
        f.upload(s)
        at, af = t.accel(), f.accel()
    ref = O.direct_f64(s, EPS20)
    et, ef = O.rel_l2(at, ref)[0], O.rel_l2(af, ref)[0]
    # the treecode skips the local-expansion truncation: never worse than the FMM
    assert et <= 1.5 * ef + 1e-7, (et, ef)


@pytest.mark.parametrize("ftype", [sv.FMM_OUTLIERS, sv.TREECODE_OUTLIERS])
def test_outlier_variants(ftype):
    s = with_outliers(12000, 5300 + ftype)
    with fmm(fmm_type=ftype) as f:
        f.upload(s)
        a = f.accel()
        flags, cnt = f.outliers()
    ref_flags, ref_cnt = O.outliers(s)
    np.testing.assert_array_equal(flags, ref_flags)
    assert cnt == ref_cnt >= 7
    ref = O.direct_f64(s, EPS20)
    err = O.rel_l2(a, ref, s["status"])[0]
    assert err <= 2e-5, err
    # the outliers themselves are summed directly in FP64
    o = np.nonzero((flags == 1) & (s["status"] == 1))[0]
    np.testing.assert_allclose(a[o], ref[o], rtol=1e-12, atol=0)


def test_outliers_keep_the_tree_fine():
    """One ion 1 m away stretches the Morton cube; the plain FMM then packs the
    plume into few boxes, the outlier variant keeps its normal depth."""
    s = plume.make_plume(20000, 2e-6, 5400)
    s["x"][0] = (1.0, 0.0, 0.0)
    with fmm(fmm_type=sv.FMM_OUTLIERS) as f:
        f.upload(s)
        a = f.accel()
        st = f.stats()
        _, cnt = f.outliers()
    assert cnt == 1 and st.levels >= 4
    ref = O.direct_f64(s, EPS20)
    assert O.rel_l2(a, ref, s["status"])[0] <= 2e-5


def test_outlier_variant_limits():
    s = with_outliers(3000, 5500)
    with fmm(fmm_type=sv.FMM_OUTLIERS, symmetry=sv.SYM_ROTATIONAL) as f:
        f.upload(s)
        with pytest.raises(sv.SolveitError):
            f.accel()
    with fmm() as f:
        f.upload(s)
        f.accel()
        with pytest.raises(sv.SolveitError):
            f.outliers()  # no outlier-variant evaluation yet
    with fmm(fmm_type=sv.TREECODE) as f:
        with pytest.raises(sv.SolveitError):
            f.upload_batch([s], [sv.FMM], [0])


def test_outlier_flags_match_reference_fixture(golden_dir):
    """GPU outlier detection on the reference's own state (FP32 vec4 arrays)
    against the flags of the reference's isOutlier."""
    import os

    d = np.load(os.path.join(golden_dir, "outliers.npz"))
    for key in ("n2001", "n2000"):
        with fmm(fmm_type=sv.FMM_OUTLIERS) as f:
            f.upload_ref32(d[f"{key}_pos4"], d[f"{key}_vel4"], d[f"{key}_acc4"], d[f"{key}_tinj"])
            f.accel(out=False)
            flags, cnt = f.outliers()
        np.testing.assert_array_equal(flags, d[f"{key}_flags"])
        assert cnt == int(d[f"{key}_count"])
