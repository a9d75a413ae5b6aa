"""Parity of the GPU direct sum and leapfrog with the oracle (FP64 restatement,
itself pinned bit-exact to the reference) and with the reference's golden
outputs.  Tolerances: FP64 path 1e-12 relative (rounding only); mixed path
1e-5 per-particle relative L2 (the workload's force-error bound) against the
FP64 direct sum."""
import os

import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv
from gpu_util import rel_l2, run_accel

pytestmark = pytest.mark.gpu

EPS20 = 1e-20


def golden(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, name)))


@pytest.mark.parametrize("prec,tol", [(sv.MIXED, 2e-6), (sv.FP64, 1e-12)])
@pytest.mark.parametrize("n,length", [(1, 1e-6), (2, 1e-9), (257, 1e-7), (4096, 1e-6)])
def test_direct_vs_f64_oracle(prec, tol, n, length):
    st = plume.make_plume(n, length, 100 + n)
    ref = O.direct_f64(st, EPS20)
    a, _ = run_accel(st, softening2=EPS20, precision=prec)
    if n == 1:
        assert np.all(a == 0.0)
        return
    assert rel_l2(a, ref, st["status"]) < tol


def test_direct_long_plume_mixed_precision():
    # 50 um plume: FP32 absolute coordinates would lose ~1e-3 on close pairs;
    # block-relative FP32 coordinates on Morton-sorted targets keep 1e-6.
    st = plume.make_plume(32768, 50e-6, 7)
    tg = np.arange(0, 32768, 97)
    ref = O.direct_f64(st, EPS20, targets=tg)
    a, _ = run_accel(st, softening2=EPS20, precision=sv.MIXED)
    assert rel_l2(a[tg], ref, st["status"][tg]) < 1e-5


@pytest.mark.parametrize("sym", [0, 1, 2])
def test_direct_matches_reference_golden(golden_dir, sym):
    g = golden(golden_dir, "direct_n512.npz")
    with sv.ForceMethod(softening2=float(g["eps"]), symmetry=sym, precision=sv.FP64, sym_axes=(1, 1, 0),
                        sym_levels=2, domain_size=tuple(float(d) for d in g["domain"])) as fm:
        fm.upload_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
        fm.accel(out=False)
        acc = g["acc4"].copy()
        fm.add_accel_ref32(acc)
    ref = g[f"acc_sym{sym}"]
    st = g["acc4"][:, 3].astype(np.int32)
    # the reference forms coordinate differences in FP32 and stores FP32
    assert rel_l2(acc[:, :3].astype(np.float64), ref[:, :3].astype(np.float64), st) < 2e-6
    # status handling: source-only / out-of-bounds / crashed receive nothing
    for i in (5, 7, 9):
        assert np.all(acc[i, :3] == 0.0)


@pytest.mark.parametrize("sym", [1, 2])
@pytest.mark.parametrize("prec,tol", [(sv.MIXED, 2e-6), (sv.FP64, 1e-12)])
def test_direct_symmetry_vs_f64_oracle(sym, prec, tol):
    st = plume.make_plume(1024, 1e-6, 55)
    st["x"][:, 0] += 3e-8  # move off the rotation axis
    img = O.trans_images(2, (1, 1, 0)) * np.array([2e-6, 2e-6, 0.0]) if sym == 2 else None
    ref = O.direct_f64(st, EPS20, sym=sym, img_off=img)
    a, _ = run_accel(st, softening2=EPS20, precision=prec, symmetry=sym, sym_axes=(1, 1, 0), sym_levels=2,
                     domain_size=(2e-6, 2e-6, 0.0))
    assert rel_l2(a, ref, st["status"]) < tol


def test_status_and_target_range():
    st = plume.make_plume(600, 1e-7, 3)
    st["status"][10:20] = 2
    st["status"][20:30] = 0
    st["status"][30:40] = -1
    ref = O.direct_f64(st, EPS20)
    with sv.ForceMethod(softening2=EPS20, precision=sv.FP64) as fm:
        fm.upload(st)
        a = fm.accel()
        assert np.all(a[10:40] == 0.0)
        assert rel_l2(a, ref, st["status"]) < 1e-12
        a2 = fm.accel(first=100, last=200)
    # the reference's [firstParticle, lastParticle) bounds the sources too
    # (direct_force_method.cpp:374-377)
    win = dict(st, status=np.where((np.arange(600) >= 100) & (np.arange(600) < 200), st["status"], 0).astype(np.int32))
    ref_w = O.direct_f64(win, EPS20)
    assert np.all(a2[:100] == 0.0) and np.all(a2[200:] == 0.0)
    np.testing.assert_allclose(a2[100:200], ref_w[100:200], rtol=1e-11, atol=0)
    assert np.max(np.abs(ref_w[100:200] - ref[100:200])) > 1e-3 * np.max(np.abs(ref[100:200]))


def test_empty_plume():
    st = plume.make_plume(0, 1e-6, 1)
    with sv.ForceMethod(softening2=EPS20) as fm:
        fm.upload(st)
        a = fm.accel()
        assert a.shape == (0, 3)
        fm.leapfrog(2, 1e-13)


def test_leapfrog_vs_oracle():
    st = plume.make_plume(512, 1e-6, 21)
    st["t_inj"][:50] = 2.5e-13  # injected during the run: exercises the clamps
    nsteps, dt, ef = 10, 1e-13, (0.0, 0.0, 1e8)
    xr, vr, _ = O.leapfrog_f64(st, nsteps, dt, EPS20, ef)
    with sv.ForceMethod(softening2=EPS20, precision=sv.FP64, efield=ef) as fm:
        fm.upload(st)
        fm.leapfrog(nsteps, dt)
        x, v, _ = fm.download()
    assert np.max(np.abs(x - xr)) < 1e-20 + 1e-13 * np.max(np.abs(xr))
    assert np.max(np.abs(v - vr)) / np.max(np.abs(vr)) < 1e-11


def test_leapfrog_matches_reference_golden(golden_dir):
    g = golden(golden_dir, "dkd_n256.npz")
    with sv.ForceMethod(softening2=float(g["eps"]), precision=sv.FP64, efield=(0.0, 0.0, float(g["ez"]))) as fm:
        fm.upload_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
        fm.leapfrog(int(g["steps"]), float(g["dt"]))
        x, v, _ = fm.download()
    vr = g["vel4_out"][:, :3].astype(np.float64)
    xr = g["pos4_out"][:, :3].astype(np.float64)
    # the reference integrates in FP32
    assert np.max(np.abs(v - vr) / np.linalg.norm(vr, axis=1)[:, None]) < 1e-5
    assert np.max(np.abs(x - xr)) < 1e-12


def test_energy_vs_oracle():
    st = plume.make_plume(3000, 1e-6, 77)
    ke_r, pe_r = O.energy_f64(st, EPS20)
    with sv.ForceMethod(softening2=EPS20) as fm:
        fm.upload(st)
        ke, pe = fm.energy()
    assert abs(ke - ke_r) / ke_r < 1e-12
    assert abs(pe - pe_r) / pe_r < 1e-12


def test_mixed_accumulation_large_n_property():
    # N = 262144 over a 10 um plume: checksum property on a sample of targets
    st = plume.make_plume(1 << 18, 10e-6, 8)
    tg = np.random.default_rng(0).choice(1 << 18, 256, replace=False)
    ref = O.direct_f64(st, EPS20, targets=tg)
    a, s = run_accel(st, softening2=EPS20, precision=sv.MIXED)
    assert rel_l2(a[tg], ref, st["status"][tg]) < 1e-5
    assert s.pair_interactions > 0


def test_page_locked_upload_and_download_match_pageable():
    """Page-locked host arrays (the end-to-end bench's buffers, copied
    asynchronously): an upload / download round trip returns the input
    exactly, and a leapfrog from either kind of buffer agrees to round-off
    (the direct sum's split accumulation is not bit-reproducible)."""
    torch = pytest.importorskip("torch")
    import ctypes as C

    st = plume.make_plume(5000, 1e-6, 61)
    st["t_inj"][:] = np.linspace(0.0, 2e-13, 5000)
    st["status"][::7] = 2
    pin = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory() for k in ("x", "v", "q", "m", "status",
                                                                                  "t_inj")}
    ptr = {k: C.c_void_p(t.data_ptr()) for k, t in pin.items()}
    L = sv.load()

    def download_pinned(fm):
        xo = torch.zeros((5000, 3), dtype=torch.float64).pin_memory()
        vo = torch.zeros((5000, 3), dtype=torch.float64).pin_memory()
        so = torch.zeros(5000, dtype=torch.int32).pin_memory()
        assert L.sv_download(fm.h, C.c_void_p(xo.data_ptr()), C.c_void_p(vo.data_ptr()),
                             C.c_void_p(so.data_ptr())) == 0
        return xo.numpy().copy(), vo.numpy().copy(), so.numpy().copy()

    with sv.ForceMethod(softening2=EPS20, efield=(0.0, 0.0, 1e8)) as fm:
        assert L.sv_upload(fm.h, 5000, ptr["x"], ptr["v"], ptr["q"], ptr["m"], ptr["status"], ptr["t_inj"]) == 0
        x, v, s = download_pinned(fm)
        assert np.array_equal(x, st["x"]) and np.array_equal(v, st["v"]) and np.array_equal(s, st["status"])
        fm.leapfrog(3, 1e-13)
        xp, vp, sp = download_pinned(fm)
    with sv.ForceMethod(softening2=EPS20, efield=(0.0, 0.0, 1e8)) as fm:
        fm.upload(st)
        fm.leapfrog(3, 1e-13)
        xr, vr, sr = fm.download()
    assert np.array_equal(sp, sr)
    assert np.max(np.abs(xp - xr)) <= 1e-13 * np.max(np.abs(xr))
    assert np.max(np.abs(vp - vr)) <= 1e-10 * np.max(np.abs(vr))
