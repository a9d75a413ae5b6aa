"""Batched plumes: many independent plumes in one context.

Each plume's acceleration from the batch is checked against the FP64 oracle
direct sum of that plume alone (with its own symmetry variant), against a
single-plume context running the same method, and the batched leapfrog
(CUDA-graph replays) against the oracle's FP64 leapfrog per plume.
"""
import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv

pytestmark = pytest.mark.gpu

EPS20 = 1e-20
# per-plume relative-L2 force error bounds against the FP64 direct sum
TOL_DIRECT = 2e-6
TOL_FMM_P6 = 2.5e-4


def small_batch(seed=3100):
    sizes = [1500, 3000, 9000, 12000, 2000, 20000, 700]
    methods = [sv.DIRECT, sv.DIRECT, sv.FMM, sv.FMM, sv.DIRECT, sv.FMM, sv.FMM]
    syms = [sv.SYM_NONE, sv.SYM_ROTATIONAL, sv.SYM_NONE, sv.SYM_ROTATIONAL, sv.SYM_ROTATIONAL, sv.SYM_NONE,
            sv.SYM_ROTATIONAL]
    states = [plume.make_plume(n, 1e-6, seed + i) for i, n in enumerate(sizes)]
    return states, methods, syms


def split(a, states):
    out, o = [], 0
    for s in states:
        n = s["x"].shape[0]
        out.append(a[o:o + n])
        o += n
    return out


def batch_ctx(**kw):
    return sv.ForceMethod(softening2=EPS20, fmm_order=6, fmm_ws=2, **kw)


def test_batch_accel_matches_oracle():
    states, methods, syms = small_batch()
    # a few particles that are sources only or ignored
    states[1]["status"][:50] = 2
    states[2]["status"][10:40] = 0
    states[5]["status"][::97] = -1
    with batch_ctx() as fm:
        fm.upload_batch(states, methods, syms)
        a = fm.accel()
        info = fm.batch_info()
    assert info.nplumes == len(states) and info.fmm_plumes == 4
    assert info.leaf_level >= 2 and info.graph_kernels_accel > 10
    for s, ap, meth, sym in zip(states, split(a, states), methods, syms):
        ref = O.direct_f64(s, EPS20, sym=sym)
        err = O.rel_l2(ap, ref, s["status"])[0]
        tol = TOL_DIRECT if meth == sv.DIRECT else TOL_FMM_P6
        assert err <= tol, (meth, sym, s["x"].shape[0], err)
        nt = s["status"] != 1
        assert np.all(ap[nt] == 0.0)


def test_batch_matches_single_plume_contexts():
    states, methods, syms = small_batch(seed=3200)
    with batch_ctx() as fm:
        fm.upload_batch(states, methods, syms)
        a = split(fm.accel(), states)
    for s, ab, meth, sym in zip(states, a, methods, syms):
        with batch_ctx(method=meth, symmetry=sym) as one:
            one.upload(s)
            a1 = one.accel()
        ref = O.direct_f64(s, EPS20, sym=sym)
        d = O.rel_l2(ab, a1, s["status"])[0]
        # the direct sums agree to FP32 rounding; the two FMM trees differ
        # (per-plume cube scaling), so their errors against the FP64 sum do
        bound = 2 * TOL_DIRECT if meth == sv.DIRECT else 2 * TOL_FMM_P6
        assert d <= bound, (meth, sym, d)
        assert O.rel_l2(a1, ref, s["status"])[0] <= (TOL_DIRECT if meth == sv.DIRECT else TOL_FMM_P6)


def test_batch_leapfrog_matches_oracle():
    states, methods, syms = small_batch(seed=3300)
    dt, nsteps, t0 = 1e-13, 6, 2e-13
    ez = (0.0, 0.0, 1e8)
    # staggered injection times exercise the clamps of the drift and kick
    for i, s in enumerate(states):
        s["t_inj"][:] = t0 + dt * (np.arange(s["x"].shape[0]) % 4) * 0.75
    with batch_ctx(efield=ez) as fm:
        fm.upload_batch(states, methods, syms)
        fm.leapfrog(3, dt, t0)
        fm.leapfrog(nsteps - 3, dt, t0 + 3 * dt)  # a second call continues the clock
        x, v, st = fm.download()
    xs, vs = split(x, states), split(v, states)
    for s, xb, vb, meth, sym in zip(states, xs, vs, methods, syms):
        xr, vr, _ = O.leapfrog_f64(s, nsteps, dt, EPS20, ez, t0=t0, sym=sym)
        # the force moves a particle ~1e-11 m in these steps against ~1e-8 m
        # of drift, so the FMM's force error shows as ~1e-7 of the displacement
        disp = np.linalg.norm(xr - s["x"])
        tol_x = 2e-7 if meth == sv.DIRECT else 5e-6
        assert np.linalg.norm(xb - xr) <= tol_x * disp, (meth, sym, np.linalg.norm(xb - xr) / disp)
        dv = np.linalg.norm(vr - s["v"])
        tol = 1e-5 if meth == sv.DIRECT else 1e-3
        assert np.linalg.norm(vb - vr) <= tol * dv, (meth, sym, np.linalg.norm(vb - vr) / dv)


def test_batch_tune_and_cache(tmp_path):
    states, methods, syms = small_batch(seed=3400)
    cache = tmp_path / "tune.txt"
    with batch_ctx() as fm:
        fm.upload_batch(states, methods, syms)
        ms = fm.tune(cache)
        info = fm.batch_info()
        a = split(fm.accel(), states)
    assert ms > 0 and info.tuned_ms == pytest.approx(ms)
    assert info.m2l_weight in (100, 200, 400, 800, 1600, 3200)
    assert info.direct_chunk in (1024, 2048, 4096, 8192)
    lines = cache.read_text().split()
    # key, leaf target, direct chunk, ms, order and near field (0: not tuned)
    assert len(lines) == 6 and int(lines[1]) == info.m2l_weight and lines[4:] == ["0", "0"]
    # a new context with the same shape reads the cached choice
    with batch_ctx() as fm2:
        fm2.upload_batch(states, methods, syms)
        fm2.tune(cache)
        i2 = fm2.batch_info()
    assert (i2.m2l_weight, i2.direct_chunk) == (info.m2l_weight, info.direct_chunk)
    assert len(cache.read_text().split()) == 6
    for s, ap, meth, sym in zip(states, a, methods, syms):
        ref = O.direct_f64(s, EPS20, sym=sym)
        assert O.rel_l2(ap, ref, s["status"])[0] <= (TOL_DIRECT if meth == sv.DIRECT else TOL_FMM_P6)


def test_batch_tune_chooses_order_under_error_bound(tmp_path):
    """With fmm_tune_err the batch tuner also picks the forest's order and
    near field: the kept choice meets the bound on every FMM plume against
    the oracle (1.5x margin: the tuner samples 64 targets on up to four
    plumes), a looser bound keeps a choice at least as fast, and a cached
    choice is restored in a new context."""
    sizes = [9000, 14000, 20000, 3000]
    states = [plume.make_ball(n, 100e-9, 3500 + i) for i, n in enumerate(sizes)]
    methods = [sv.FMM, sv.FMM, sv.FMM, sv.DIRECT]
    syms = [sv.SYM_NONE, sv.SYM_ROTATIONAL, sv.SYM_NONE, sv.SYM_NONE]
    cache = tmp_path / "tune.txt"
    kept = {}
    for bound in (1e-5, 3e-4):
        with sv.ForceMethod(softening2=EPS20, fmm_order=6, fmm_ws=2, fmm_tune_err=bound) as fm:
            fm.upload_batch(states, methods, syms)
            fm.tune(cache)
            info = fm.batch_info()
            a = split(fm.accel(), states)
        assert info.fmm_order in (4, 6, 8) and info.fmm_near in (1, 2)
        for s, ap, meth, sym in zip(states, a, methods, syms):
            if meth == sv.FMM:
                e = O.rel_l2(ap, O.direct_f64(s, EPS20, sym=sym), s["status"])[0]
                assert e <= 1.5 * bound, (bound, info.fmm_order, info.fmm_near, sym, e)
        kept[bound] = (info.fmm_order, info.fmm_near, info.tuned_ms)
    # the looser bound's choice is at least as fast (within timing noise)
    assert kept[3e-4][2] <= 1.15 * kept[1e-5][2], kept
    with sv.ForceMethod(softening2=EPS20, fmm_order=6, fmm_ws=2, fmm_tune_err=1e-5) as fm:
        fm.upload_batch(states, methods, syms)
        fm.tune(cache)
        i2 = fm.batch_info()
    assert (i2.fmm_order, i2.fmm_near) == kept[1e-5][:2]


def test_batch_edge_cases():
    a = plume.make_plume(0, 1e-6, 1)
    b = plume.make_plume(1, 1e-6, 2)
    c = plume.make_plume(2500, 1e-6, 3)
    d = plume.make_plume(9000, 1e-6, 4)
    d["status"][:] = 2  # sources only: no target in the whole plume
    states = [a, b, c, d]
    with batch_ctx() as fm:
        fm.upload_batch(states, [sv.FMM, sv.DIRECT, sv.FMM, sv.FMM], [0, 1, 0, 1])
        acc = split(fm.accel(), states)
        with pytest.raises(sv.SolveitError):
            fm.energy()
    # a lone particle feels only its own rotated images; a plume without targets gets nothing
    np.testing.assert_allclose(acc[1], O.direct_f64(b, EPS20, sym=1), rtol=1e-6)
    assert np.all(acc[3] == 0.0)
    ref = O.direct_f64(c, EPS20)
    assert O.rel_l2(acc[2], ref, c["status"])[0] <= TOL_FMM_P6
    with batch_ctx() as fm:
        with pytest.raises(sv.SolveitError):
            fm.upload_batch([c], [sv.BARNES_HUT], [0])


def test_batch_sampled_c3_workload():
    """32 plumes of the batched workload's distribution; 64 sampled targets
    per plume against the FP64 oracle."""
    states, methods, syms = plume.make_batch(32)
    with batch_ctx() as fm:
        fm.upload_batch(states, methods, syms)
        a = split(fm.accel(), states)
    rng = np.random.default_rng(0)
    for s, ap, meth, sym in zip(states, a, methods, syms):
        t = np.sort(rng.choice(s["x"].shape[0], 64, replace=False))
        ref = O.direct_f64(s, EPS20, sym=sym, targets=t, threads=8)
        err = O.rel_l2(ap[t], ref)[0]
        assert err <= (TOL_DIRECT if meth == sv.DIRECT else TOL_FMM_P6), (meth, sym, s["x"].shape[0], err)
