"""The M2L on the tensor cores (fmm_m2l_tc = 1) against the oracle and
against the FP32 rotation M2L (fmm_m2l_tc = -1) on the same tree.

The tensor-core path contracts each offset class's translations with a dense
operator built in FP64 (TF32 high / low split of both operands, three
products, FP32 accumulation), so its error against the FP64 direct sum must
stay at the rotation kernel's: per-particle relative L2 below 1e-5 at p = 8,
ws = 2 (the workload bound), and within 5 % (plus 1e-7) of the rotation
kernel's own error at the other orders and at ws = 1; the two paths' far
fields agree to 2e-6 of the acceleration.
"""
import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv
from gpu_util import rel_l2, run_accel

pytestmark = pytest.mark.gpu

EPS20 = 1e-20


def _both(st, **kw):
    a_tc, s_tc = run_accel(st, softening2=EPS20, method=sv.FMM, fmm_m2l_tc=1, **kw)
    a_rot, s_rot = run_accel(st, softening2=EPS20, method=sv.FMM, fmm_m2l_tc=-1, **kw)
    return a_tc, s_tc, a_rot, s_rot


def test_tc_p8_ws2_meets_1e5_and_matches_rotation():
    n = 65536
    st = plume.make_plume(n, 10e-6, 7001)
    tg = np.arange(0, n, 32)
    ref = O.direct_f64(st, EPS20, targets=tg)
    a_tc, s_tc, a_rot, s_rot = _both(st, fmm_order=8, fmm_ws=2)
    assert s_tc.m2l_tc == 1 and s_rot.m2l_tc == 0
    assert s_tc.cell_interactions == s_rot.cell_interactions > 0
    e_tc = rel_l2(a_tc[tg], ref, st["status"][tg])
    e_rot = rel_l2(a_rot[tg], ref, st["status"][tg])
    assert e_tc < 1e-5 and e_tc < 1.05 * e_rot + 1e-7, (e_tc, e_rot)
    assert rel_l2(a_tc, a_rot, st["status"]) < 2e-6


@pytest.mark.parametrize("p,ws", [(4, 2), (6, 2), (10, 2), (8, 1), (6, 1)])
def test_tc_orders_and_separations(p, ws):
    n = 20000
    st = plume.make_plume(n, 2e-6, 7100 + 10 * p + ws)
    ref = O.direct_f64(st, EPS20)
    a_tc, s_tc, a_rot, _ = _both(st, fmm_order=p, fmm_ws=ws)
    assert s_tc.m2l_tc == 1
    e_tc, e_rot = rel_l2(a_tc, ref, st["status"]), rel_l2(a_rot, ref, st["status"])
    assert e_tc < 1.05 * e_rot + 1e-7, (e_tc, e_rot)


def test_tc_cube_overflow_falls_back_then_grows():
    """A 3D cube's lists are long (up to 875 entries per box at ws 2): the
    first evaluation may exceed the reserved room and run the rotation
    kernel instead; the room then grows and the next evaluation runs on the
    tensor cores.  Both meet the bound."""
    n = 40000
    rng = np.random.default_rng(7200)
    st = plume.make_plume(n, 1e-6, 7201)
    st["x"][:] = rng.random((n, 3)) * 2e-7
    st["q"][:] = rng.choice([1.0, 2.0], n)
    st["status"][::97] = 2
    tg = np.arange(0, n, 16)
    ref = O.direct_f64(st, EPS20, targets=tg)
    with sv.ForceMethod(softening2=EPS20, method=sv.FMM, fmm_order=8, fmm_ws=2, fmm_m2l_tc=1) as fm:
        fm.upload(st)
        paths = []
        for _ in range(3):
            a = fm.accel()
            paths.append(fm.stats().m2l_tc)
            assert rel_l2(a[tg], ref, st["status"][tg]) < 1e-5
    assert paths[-1] == 1, paths


def test_tc_leapfrog_and_symmetry_images():
    """Rotational and translational images join the tree as sources; the
    tensor-core M2L handles their boxes as any other."""
    st = plume.make_plume(4096, 1e-6, 7300)
    st["x"][:, 0] += 3e-8
    for sym in (1, 2):
        img = O.trans_images(2, (1, 1, 0)) * np.array([2e-6, 2e-6, 0.0]) if sym == 2 else None
        ref = O.direct_f64(st, EPS20, sym=sym, img_off=img)
        a, s = run_accel(st, softening2=EPS20, method=sv.FMM, fmm_order=8, fmm_ws=2, fmm_m2l_tc=1, symmetry=sym,
                         sym_axes=(1, 1, 0), sym_levels=2, domain_size=(2e-6, 2e-6, 0.0))
        assert rel_l2(a, ref, st["status"]) < 1e-5
    ef = (0.0, 0.0, 1e8)
    xr, vr, _ = O.leapfrog_f64(st, 5, 1e-13, EPS20, ef)
    with sv.ForceMethod(softening2=EPS20, method=sv.FMM, fmm_order=8, fmm_ws=2, fmm_m2l_tc=1, efield=ef) as fm:
        fm.upload(st)
        fm.leapfrog(5, 1e-13)
        x, v, _ = fm.download()
    dv = np.linalg.norm(v - vr, axis=1) / np.linalg.norm(vr - st["v"], axis=1)
    assert np.sqrt(np.mean(dv ** 2)) < 1e-5


@pytest.mark.parametrize("p", [6, 8])
def test_tc_forest_of_plumes(p):
    """A batch's FMM forest (several plumes, one root each, rotational images
    on one of them): the tensor-core M2L against the oracle and against the
    rotation kernel, over two evaluations (the first may run out of room and
    fall back, the plan then grows it)."""
    sizes = (9000, 14000, 20000)
    states = [plume.make_plume(n, 1e-6, 7400 + i) for i, n in enumerate(sizes)]
    methods, syms = [sv.FMM] * 3, [sv.SYM_NONE, sv.SYM_ROTATIONAL, sv.SYM_NONE]
    out = {}
    for tc in (1, -1):
        with sv.ForceMethod(softening2=EPS20, fmm_order=p, fmm_ws=2, fmm_m2l_tc=tc) as fm:
            fm.upload_batch(states, methods, syms)
            fm.accel()
            out[tc] = fm.accel()
    o = 0
    for s, sy in zip(states, syms):
        k = s["x"].shape[0]
        ref = O.direct_f64(s, EPS20, sym=sy)
        e_tc = rel_l2(out[1][o:o + k], ref, s["status"])
        e_rot = rel_l2(out[-1][o:o + k], ref, s["status"])
        assert e_tc < 1.05 * e_rot + 1e-7, (p, e_tc, e_rot)
        o += k
