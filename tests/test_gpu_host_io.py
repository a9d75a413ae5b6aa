"""Host state arrays in pinned, mapped memory are read and written in place
by kernels (no staging copy); pageable arrays go by copies.  Both paths must
move identical bits, and a call whose arrays mix the two kinds takes the
copies.  Each comparison isolates the transfer: uploads are compared by an
immediate download, downloads of one context's state by both paths, and the
accelerations of one FMM evaluation (the FMM is deterministic run to run)."""
import ctypes as C

import numpy as np
import pytest
import torch

import plume
import solveit_gpu as sv

pytestmark = pytest.mark.gpu

EPS20 = 1e-20
N = 5000


def _pinned(a):
    t = torch.empty(a.shape, dtype=torch.float64 if a.dtype == np.float64 else torch.int32, pin_memory=True)
    t.numpy()[...] = a
    return t


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else None


def _upload_pinned(L, f, pin, v=None):
    v = _p(pin["v"]) if v is None else v
    assert L.sv_upload(f.h, N, _p(pin["x"]), v, _p(pin["q"]), _p(pin["m"]), _p(pin["status"]),
                       _p(pin["t_inj"])) == 0
    f.n = N


def test_pinned_and_pageable_paths_agree():
    st = plume.make_plume(N, 1e-6, 11)
    st["status"][::7] = 2
    kw = dict(softening2=EPS20, method=sv.FMM, efield=(0.0, 0.0, 1e8))
    L = sv.load()
    pin = {k: _pinned(np.ascontiguousarray(st[k])) for k in ("x", "v", "q", "m", "status", "t_inj")}
    with sv.ForceMethod(**kw) as fa, sv.ForceMethod(**kw) as fb:
        # uploads: pageable vs pinned, read back by the same (pageable) download
        fa.upload(st)
        _upload_pinned(L, fb, pin)
        for u, w in zip(fa.download(), fb.download()):
            assert np.array_equal(u, w)
        # downloads of one context's state after three steps: pageable vs pinned
        fa.leapfrog(3, 1e-13)
        xa, va, sa = fa.download()
        out = {k: _pinned(np.zeros_like(st[k])) for k in ("x", "v", "status")}
        assert L.sv_download(fa.h, _p(out["x"]), _p(out["v"]), _p(out["status"])) == 0
        assert np.array_equal(out["x"].numpy(), xa)
        assert np.array_equal(out["v"].numpy(), va)
        assert np.array_equal(out["status"].numpy(), sa)
        # accelerations of the same state: pageable vs pinned output
        aa = fa.accel()
        ab = _pinned(np.zeros((N, 3)))
        assert L.sv_compute_accel(fa.h, 0, -1, _p(ab)) == 0
        assert np.array_equal(ab.numpy(), aa)
        assert np.all(aa[st["status"] != 1] == 0.0)
        # pinned positions with pageable velocities: the copy path, same bits
        v_page = np.ascontiguousarray(st["v"])
        _upload_pinned(L, fb, pin, v=v_page.ctypes.data_as(C.c_void_p))
        fa.upload(st)
        xb = _pinned(np.zeros((N, 3)))
        assert L.sv_download(fb.h, _p(xb), None, None) == 0
        assert np.array_equal(xb.numpy(), fa.download()[0])


def test_update_state_continues_a_run():
    """sv_update_state with the downloaded state (pinned or pageable arrays)
    changes nothing: one step, update, two steps equals three steps, bit for
    bit (the FMM is deterministic); the wrong count and a state-less context
    are refused."""
    st = plume.make_plume(N, 1e-6, 13)
    kw = dict(softening2=EPS20, method=sv.FMM, efield=(0.0, 0.0, 1e8))
    L = sv.load()
    with sv.ForceMethod(**kw) as fa:
        fa.upload(st)
        fa.leapfrog(3, 1e-13, 0.0)
        xa, va, sa = fa.download()
    for pinned in (False, True):
        with sv.ForceMethod(**kw) as fb:
            fb.upload(st)
            fb.leapfrog(1, 1e-13, 0.0)
            x, v, s = fb.download()
            if pinned:
                px, pv, ps = _pinned(x), _pinned(v), _pinned(s)
                assert L.sv_update_state(fb.h, N, _p(px), _p(pv), _p(ps)) == 0
            else:
                fb.update_state(x, v, s)
            fb.leapfrog(2, 1e-13, 1e-13)
            xb, vb, sb = fb.download()
        assert np.array_equal(xb, xa) and np.array_equal(vb, va) and np.array_equal(sb, sa)
    with sv.ForceMethod(**kw) as fc:
        with pytest.raises(sv.SolveitError):
            fc.update_state(st["x"])
        fc.upload(st)
        with pytest.raises(sv.SolveitError):
            fc.update_state(st["x"][:10])
        # positions only: velocities and statuses stay
        fc.update_state(st["x"] + 1e-9)
        x, v, s = fc.download()
        assert np.array_equal(x, st["x"] + 1e-9) and np.array_equal(v, st["v"]) and np.array_equal(s, st["status"])


def test_adapter_add_accel_uses_the_context_buffer():
    """sv_add_accel_ref32 adds the last acceleration into the reference's
    float4 array through the context's own pinned buffer."""
    st = plume.make_plume(N, 1e-6, 12)
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    with sv.ForceMethod(softening2=EPS20, method=sv.FMM) as f:
        f.upload_ref32(pos4, vel4, acc4, tinj)
        a = f.accel()
        acc = acc4.copy()
        acc[:, :3] = 0.0
        f.add_accel_ref32(acc)
    inb = acc4[:, 3] == 1.0
    assert np.array_equal(acc[inb, :3], a[inb].astype(np.float32))
    assert np.all(acc[~inb, :3] == 0.0)
