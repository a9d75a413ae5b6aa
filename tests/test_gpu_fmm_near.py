"""The trimmed near field of separation 2 (sv_params.fmm_near = 2): the
(2,2,1)- and (2,2,2)-type boxes of the 5^3 near cube are M2L entries instead
of direct pairs.

Checked against the FP64 direct sum (the oracle) on plumes resolved in three
dimensions, where those boxes are occupied:
  p 8: relative-L2 force error <= 1e-5 (the workload's bound), with fewer
      pairs and fewer M2L translations than the full cube;
  the tensor-core and rotation-kernel M2L agree in the trimmed mode;
  a batch's forest with the trimmed near field matches the oracle per plume
      at the batch's p 6 bound (2.5e-4);
  a 5-step leapfrog tracks the FP64 direct leapfrog;
  at separation 1 the option changes nothing.
"""
import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv
from gpu_util import rel_l2

pytestmark = pytest.mark.gpu

EPS20 = 1e-20


def _eval(st, **kw):
    with sv.ForceMethod(softening2=EPS20, method=sv.FMM, **kw) as fm:
        fm.upload(st)
        fm.accel()  # the tensor-core room is sized by the first evaluation
        a = fm.accel()
        return a, fm.stats()


def test_trimmed_ball_p8_meets_1e5_with_less_work():
    st = plume.make_ball(65536, 200e-9, 9100)
    tg = np.arange(0, 65536, 64)
    ref = O.direct_f64(st, EPS20, targets=tg)
    a1, s1 = _eval(st, fmm_order=8, fmm_ws=2, fmm_near=1)
    a2, s2 = _eval(st, fmm_order=8, fmm_ws=2, fmm_near=2)
    e1 = rel_l2(a1[tg], ref, st["status"][tg])
    e2 = rel_l2(a2[tg], ref, st["status"][tg])
    assert e2 <= 1e-5, e2
    assert e1 <= e2, (e1, e2)
    assert s2.pair_interactions < 0.9 * s1.pair_interactions, (s1.pair_interactions, s2.pair_interactions)
    assert s2.cell_interactions < s1.cell_interactions, (s1.cell_interactions, s2.cell_interactions)


def test_trimmed_tensor_cores_match_rotation_kernel():
    st = plume.make_ball(32768, 150e-9, 9200)
    tg = np.arange(0, 32768, 32)
    ref = O.direct_f64(st, EPS20, targets=tg)
    a_tc, s_tc = _eval(st, fmm_order=8, fmm_ws=2, fmm_near=2, fmm_m2l_tc=1)
    a_rot, s_rot = _eval(st, fmm_order=8, fmm_ws=2, fmm_near=2, fmm_m2l_tc=-1)
    assert s_tc.m2l_tc == 1 and s_rot.m2l_tc == 0
    e_tc = rel_l2(a_tc[tg], ref, st["status"][tg])
    e_rot = rel_l2(a_rot[tg], ref, st["status"][tg])
    assert e_tc <= 1.05 * e_rot + 1e-7, (e_tc, e_rot)
    assert rel_l2(a_tc, a_rot, st["status"]) < 3e-6


def test_trimmed_forest_matches_oracle():
    sizes = (9000, 14000, 20000)
    states = [plume.make_ball(n, 120e-9, 9300 + i) for i, n in enumerate(sizes)]
    methods, syms = [sv.FMM] * 3, [sv.SYM_NONE, sv.SYM_ROTATIONAL, sv.SYM_NONE]
    with sv.ForceMethod(softening2=EPS20, fmm_order=6, fmm_ws=2, fmm_near=2) as fm:
        fm.upload_batch(states, methods, syms)
        fm.accel()
        a = fm.accel()
    o = 0
    for s, sy in zip(states, syms):
        k = s["x"].shape[0]
        ref = O.direct_f64(s, EPS20, sym=sy)
        e = rel_l2(a[o:o + k], ref, s["status"])
        assert e <= 2.5e-4, (k, sy, e)
        o += k


def test_trimmed_leapfrog_tracks_direct():
    st = plume.make_ball(8192, 80e-9, 9400)
    ef = (0.0, 0.0, 1e8)
    _, vr, _ = O.leapfrog_f64(st, 5, 1e-13, EPS20, ef)
    with sv.ForceMethod(softening2=EPS20, method=sv.FMM, fmm_order=8, fmm_ws=2, fmm_near=2, efield=ef) as fm:
        fm.upload(st)
        fm.leapfrog(5, 1e-13)
        _, v, _ = fm.download()
    dv = np.linalg.norm(v - vr, axis=1) / np.linalg.norm(vr - st["v"], axis=1)
    assert np.sqrt(np.mean(dv ** 2)) < 1e-5


@pytest.mark.parametrize("sym", [1, 2])
def test_trimmed_symmetry_images(sym):
    """Rotational (4 quadrant images) and translational (81 images) variants
    with the trimmed near field: the image copies join the tree as sources,
    so their boxes at trimmed offsets are M2L sources too."""
    st = plume.make_ball(4096, 150e-9, 9600 + sym)
    st["x"][:, 0] += 3e-7
    img = O.trans_images(2, (1, 1, 0)) * np.array([1e-6, 1e-6, 0.0]) if sym == 2 else None
    ref = O.direct_f64(st, EPS20, sym=sym, img_off=img)
    kw = dict(fmm_order=8, fmm_ws=2, symmetry=sym, sym_axes=(1, 1, 0), sym_levels=2, domain_size=(1e-6, 1e-6, 0.0))
    a2, s2 = _eval(st, fmm_near=2, **kw)
    a1, s1 = _eval(st, fmm_near=1, **kw)
    assert rel_l2(a2, ref, st["status"]) < 1e-5
    assert s2.pair_interactions < s1.pair_interactions


@pytest.mark.parametrize("ftype", [sv.TREECODE, sv.FMM_OUTLIERS])
def test_trimmed_treecode_and_outlier_types(ftype):
    """The treecode evaluates interaction-list entries by M2P, the outlier
    variant leaves outliers out of the tree: both take the trimmed lists."""
    st = plume.make_ball(16384, 120e-9, 9700)
    if ftype == sv.FMM_OUTLIERS:
        st["x"][:16] *= 40.0  # a few ions far outside the ball
    ref = O.direct_f64(st, EPS20)
    a, _ = _eval(st, fmm_order=8, fmm_ws=2, fmm_near=2, fmm_type=ftype)
    assert rel_l2(a, ref, st["status"]) < 2e-5


def test_near_option_ignored_at_separation_1():
    st = plume.make_ball(16384, 100e-9, 9500)
    a1, _ = _eval(st, fmm_order=8, fmm_ws=1, fmm_near=1)
    a2, _ = _eval(st, fmm_order=8, fmm_ws=1, fmm_near=2)
    assert np.array_equal(a1, a2)


def test_near_option_validated():
    with pytest.raises(sv.SolveitError):
        with sv.ForceMethod(softening2=EPS20, method=sv.FMM, fmm_near=3) as fm:
            fm.upload(plume.make_plume(256, 1e-7, 1))
            fm.accel()
