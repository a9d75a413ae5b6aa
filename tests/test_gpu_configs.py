"""Parity at the benchmark configurations' own sizes, against the CPU oracle.

Each test runs one of the workloads at its configured size and compares with
the oracle's FP64 direct sum (oracle/sv_oracle.c, pinned to the reference's
own outputs by tests/test_oracle_golden.py) or, for trajectories longer than
the oracle finishes in seconds, with the GPU FP64 direct leapfrog, which the
C0 test here and tests/test_gpu_direct.py pin to the oracle.

Tolerances (per-particle relative L2 of the acceleration, the reference's
compareAcceleration metric, unless stated):
  C2   FMM p 8, ws 2, N = 1,048,576, z in [0, 50] um: < 1e-5 on 512 sampled
       targets against the oracle, at the initial state and after 50 steps;
       the same with the translational-periodic images (2 um in x and y, 81
       images) at the initial state and after 10 steps.
  C0   FP64 direct, N = 4096, 100 leapfrog steps: positions and velocities
       within 1e-9 of their change over the run, energy within 1e-10.
  FMM trajectory, N = 65,536, 50 steps: velocity change within 1e-5 (RMS
       over particles) and energy change within 1e-4 of the FP64 direct run.
  C1   Barnes-Hut theta 0.5, leaf 16, N = 65,536: error below the
       reference's own Barnes-Hut error on the same plume (fixture), and a
       200-step trajectory whose velocity change stays within 2e-2 (RMS) of
       the FP64 direct run.
"""
import os

import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv
from gpu_util import rel_l2

pytestmark = pytest.mark.gpu

EPS20 = 1e-20
DT = 1e-13
EF = (0.0, 0.0, 1e8)
THREADS = os.cpu_count() or 1


def _targets(n, k, seed):
    return np.sort(np.random.default_rng(seed).choice(n, k, replace=False))


def _cur(st, x, v, s):
    return dict(st, x=x, v=v, status=s)


def _fmm(**kw):
    return sv.ForceMethod(softening2=EPS20, method=sv.FMM, precision=sv.MIXED, fmm_order=8, fmm_ws=2,
                          fmm_leaf_target=32, efield=EF, **kw)


def test_c2_fmm_n1m_initial_and_after_50_steps():
    n = 1 << 20
    st = plume.make_plume(n, 50e-6, 2000 * 1000)
    with _fmm() as fm:
        fm.upload(st)
        fm.fmm_tune()
        a0 = fm.accel()
        fm.leapfrog(50, DT, 0.0)
        x, v, s = fm.download()
        a1 = fm.accel()
    tg = _targets(n, 512, 1)
    ref0 = O.direct_f64(st, EPS20, targets=tg, threads=THREADS)
    e0, m0, _, _ = O.rel_l2(a0[tg], ref0, st["status"][tg])
    assert e0 < 1e-5, (e0, m0)
    cur = _cur(st, x, v, s)
    assert np.all(s == 1) and np.all(np.isfinite(x))
    ref1 = O.direct_f64(cur, EPS20, targets=tg, threads=THREADS)
    e1, m1, _, _ = O.rel_l2(a1[tg], ref1, s[tg])
    assert e1 < 1e-5, (e1, m1)


def test_c2_fmm_n1m_translational_periodic():
    """81 periodic images (x and y period 2 um, two lattice levels): the
    images enter the tree as source-only copies."""
    n = 1 << 20
    st = plume.make_plume(n, 50e-6, 2000 * 1000 + 1)
    sym = dict(symmetry=sv.SYM_TRANSLATIONAL, sym_axes=(1, 1, 0), sym_levels=2, domain_size=(2e-6, 2e-6, 0.0))
    with _fmm(**sym) as fm:
        fm.upload(st)
        a0 = fm.accel()
        fm.leapfrog(10, DT, 0.0)
        x, v, s = fm.download()
        a1 = fm.accel()
    img = O.trans_images(2, (1, 1, 0)) * np.array([2e-6, 2e-6, 0.0])
    assert img.shape == (81, 3)
    tg = _targets(n, 512, 2)
    ref0 = O.direct_f64(st, EPS20, sym=2, img_off=img, targets=tg, threads=THREADS)
    e0, m0, _, _ = O.rel_l2(a0[tg], ref0, st["status"][tg])
    assert e0 < 1e-5, (e0, m0)
    tg1 = tg[::2]
    ref1 = O.direct_f64(_cur(st, x, v, s), EPS20, sym=2, img_off=img, targets=tg1, threads=THREADS)
    e1, m1, _, _ = O.rel_l2(a1[tg1], ref1, s[tg1])
    assert e1 < 1e-5, (e1, m1)


def test_c0_direct_fp64_100_steps_against_oracle():
    n = 4096
    st = plume.make_plume(n, 1e-6, 0)
    xr, vr, _ = O.leapfrog_f64(st, 100, DT, EPS20, EF, threads=THREADS)
    with sv.ForceMethod(softening2=EPS20, method=sv.DIRECT, precision=sv.FP64, efield=EF) as fm:
        fm.upload(st)
        ke0, pe0 = fm.energy()
        fm.leapfrog(100, DT, 0.0)
        x, v, s = fm.download()
        ke1, pe1 = fm.energy()
    dx = np.abs(x - xr).max() / np.abs(xr - st["x"]).max()
    dv = np.abs(v - vr).max() / np.abs(vr - st["v"]).max()
    assert dx < 1e-9 and dv < 1e-9, (dx, dv)
    oke0, ope0 = O.energy_f64(st, EPS20, threads=THREADS)
    oke1, ope1 = O.energy_f64(_cur(st, xr, vr, s), EPS20, threads=THREADS)
    for g, o in ((ke0, oke0), (pe0, ope0), (ke1, oke1), (pe1, ope1)):
        assert abs(g - o) <= 1e-10 * abs(o), (g, o)
    # the energy change over the run (field work plus Coulomb expansion)
    d_gpu, d_orc = (ke1 + pe1) - (ke0 + pe0), (oke1 + ope1) - (oke0 + ope0)
    assert abs(d_gpu - d_orc) <= 1e-8 * abs(d_orc), (d_gpu, d_orc)


def test_direct_fp64_trajectory_n16384_against_oracle():
    """The GPU FP64 direct leapfrog, the trajectory reference of the tests
    below, against the oracle at the adjoint workload's size over its 50
    steps."""
    n = 16384
    st = plume.make_plume(n, 1e-6, 4000)
    xr, vr, _ = O.leapfrog_f64(st, 50, DT, EPS20, EF, threads=THREADS)
    with sv.ForceMethod(softening2=EPS20, method=sv.DIRECT, precision=sv.FP64, efield=EF) as fm:
        fm.upload(st)
        fm.leapfrog(50, DT, 0.0)
        x, v, _ = fm.download()
    assert np.abs(x - xr).max() / np.abs(xr - st["x"]).max() < 1e-9
    assert np.abs(v - vr).max() / np.abs(vr - st["v"]).max() < 1e-9


def _trajectory(st, nsteps, **kw):
    with sv.ForceMethod(softening2=EPS20, efield=EF, **kw) as fm:
        fm.upload(st)
        e0 = sum(fm.energy())
        fm.leapfrog(nsteps, DT, 0.0)
        x, v, s = fm.download()
        e1 = sum(fm.energy())
    return x, v, s, e0, e1


def _rms_rel(a, ar, a0):
    d = np.linalg.norm(a - ar, axis=1) / np.linalg.norm(ar - a0, axis=1)
    return float(np.sqrt(np.mean(d ** 2)))


def test_fmm_trajectory_n65536_50_steps():
    n = 65536
    st = plume.make_plume(n, 10e-6, 2000 * 1000 + 2)
    xr, vr, _, er0, er1 = _trajectory(st, 50, method=sv.DIRECT, precision=sv.FP64)
    x, v, _, e0, e1 = _trajectory(st, 50, method=sv.FMM, precision=sv.MIXED, fmm_order=8, fmm_ws=2)
    assert abs(e0 - er0) <= 1e-12 * abs(er0)
    assert _rms_rel(v, vr, st["v"]) < 1e-5
    assert _rms_rel(x, xr, st["x"]) < 1e-5
    assert abs((e1 - e0) - (er1 - er0)) <= 1e-4 * abs(er1 - er0), (e1 - e0, er1 - er0)


def test_c1_barnes_hut_against_reference_envelope(golden_dir):
    g = dict(np.load(os.path.join(golden_dir, "bh_n65536_sampled.npz")))
    n, tg = int(g["n"]), g["targets"]
    st = plume.make_plume(n, float(g["length"]), int(g["seed"]))
    assert np.array_equal(plume.to_ref32(st)[0][tg], g["pos4_targets"])
    ref = O.direct_f64(st, EPS20, targets=tg, threads=THREADS)
    err_ref = rel_l2(g["acc_ref"].astype(np.float64), ref, st["status"][tg])
    with sv.ForceMethod(softening2=EPS20, method=sv.BARNES_HUT, theta=float(g["theta"]), leaf_size=16) as fm:
        fm.upload(st)
        a = fm.accel()
    err = rel_l2(a[tg], ref, st["status"][tg])
    assert err < err_ref, (err, err_ref)


def test_c1_barnes_hut_200_steps():
    n = 65536
    st = plume.make_plume(n, 10e-6, 1000)
    xr, vr, _, _, _ = _trajectory(st, 200, method=sv.DIRECT, precision=sv.FP64)
    x, v, s, _, _ = _trajectory(st, 200, method=sv.BARNES_HUT, precision=sv.MIXED, theta=0.5, leaf_size=16)
    assert np.all(s == 1) and np.all(np.isfinite(x))
    assert _rms_rel(v, vr, st["v"]) < 2e-2


def test_c2_reference_fmm_envelope_at_65536(golden_dir):
    """The long plume at the largest size the reference's FMM runs: the GPU
    FMM (ws 2) is more accurate than the reference's (ws 1) on the same
    particles, and within the workload's 1e-5."""
    g = dict(np.load(os.path.join(golden_dir, "fmm_n65536_z50_sampled.npz")))
    n, tg = int(g["n"]), g["targets"]
    st = plume.make_plume(n, float(g["length"]), int(g["seed"]))
    ref = O.direct_f64(st, EPS20, targets=tg, threads=THREADS)
    err_ref = rel_l2(g["acc_ref"].astype(np.float64), ref, st["status"][tg])
    with _fmm() as fm:
        fm.upload(st)
        a = fm.accel()
    err = rel_l2(a[tg], ref, st["status"][tg])
    assert err < 1e-5 and err < err_ref / 10, (err, err_ref)


@pytest.mark.parametrize("method", [sv.DIRECT, sv.FMM])
def test_compare_accel_window_against_oracle_metric(method):
    """sv_compare_accel on the device over the last evaluation's [first,
    last) window equals the oracle's metric on that window (the terms in
    FP64: largest term and its index exactly, the mean to rounding)."""
    n, first, last = 6000, 700, 5100
    st = plume.make_plume(n, 1e-6, 6100 + method)
    st["status"][800:820] = 2
    st["status"][900:910] = 0
    win = dict(st, status=np.where((np.arange(n) >= first) & (np.arange(n) < last), st["status"], 0)
               .astype(np.int32))
    ref = O.direct_f64(win, EPS20, threads=THREADS)
    ref_full = ref.copy()
    ref_full[:first] = 1.0  # outside the window: must not count
    ref_full[last:] = -1.0
    kw = dict(fmm_order=8, fmm_ws=2) if method == sv.FMM else {}
    with sv.ForceMethod(softening2=EPS20, method=method, precision=sv.MIXED, **kw) as fm:
        fm.upload(st)
        a = fm.accel(first=first, last=last)
        l2, mx, am = fm.compare(ref_full)
    ol2, omx, oam, _ = O.rel_l2(a[first:last], ref[first:last], st["status"][first:last])
    assert l2 > 0 and abs(l2 - ol2) <= 1e-12 * ol2, (l2, ol2)
    assert mx == omx and am == oam + first, (mx, omx, am, oam)
    # after a leapfrog step the window is the whole plume
    with sv.ForceMethod(softening2=EPS20, method=method, precision=sv.MIXED, **kw) as fm:
        fm.upload(st)
        fm.leapfrog(1, DT)
        x, v, s = fm.download()
        a2 = fm.accel()
        ref2 = O.direct_f64(_cur(st, x, v, s), EPS20, threads=THREADS)
        l2b, mxb, amb = fm.compare(ref2)
    ol2b, omxb, oamb, _ = O.rel_l2(a2, ref2, s)
    assert abs(l2b - ol2b) <= 1e-12 * ol2b and mxb == omxb and amb == oamb
