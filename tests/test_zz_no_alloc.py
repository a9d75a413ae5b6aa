"""The allocation-free direct-sum entry point, through the C ABI.

sv_direct_accel_noalloc serves callers that cannot allocate device memory
(an allocator owned by a host framework, real-time loops that must not call
cudaMalloc / cudaFree): they pass device buffers they already own and the
library works in one static device array.  This test owns its buffers (torch
allocates them here, outside the call), calls the entry point twice in a row
on different plumes, and checks each result against the regular entry point
(sv_compute_accel, direct method, mixed precision) within 1e-12 relative per
particle: both run the same sorted FP32 tile kernel and differ only in the
order of FP64 atomic additions.  The second call must not change the amount
of free device memory (the first call on a device is its set-up call: it
loads the array).  Each result is also held to the oracle's FP64 direct sum
on sampled targets within 2e-6 per-particle relative L2, the bound of the
mixed-precision direct sum in tests/test_gpu_direct.py, and one call runs at
the stated maximum size, where the array must hold the sort's temporary
storage too.
"""
import ctypes as C
import os

import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv

pytestmark = pytest.mark.gpu

EPS20 = 1e-20


def _regular(state):
    with sv.ForceMethod(softening2=EPS20, method=sv.DIRECT, precision=sv.MIXED) as fm:
        fm.upload(state)
        return fm.accel()


def _noalloc(L, torch, state, a3_dev):
    n = state["x"].shape[0]
    dev = torch.device("cuda:0")
    x3 = torch.as_tensor(state["x"], device=dev).contiguous()
    q = torch.as_tensor(state["q"], device=dev).contiguous()
    m = torch.as_tensor(state["m"], device=dev).contiguous()
    st = torch.as_tensor(state["status"], device=dev).contiguous()
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info(0)[0]
    rc = L.sv_direct_accel_noalloc(C.c_int64(n), C.c_void_p(x3.data_ptr()), C.c_void_p(q.data_ptr()),
                                   C.c_void_p(m.data_ptr()), C.c_void_p(st.data_ptr()), C.c_double(EPS20),
                                   C.c_double(sv.default_params().k_const), C.c_void_p(a3_dev.data_ptr()),
                                   C.c_void_p(torch.cuda.current_stream(0).cuda_stream))
    torch.cuda.synchronize()
    free_after = torch.cuda.mem_get_info(0)[0]
    return rc, a3_dev[:n].cpu().numpy(), free_before, free_after


def _assert_close(a, ref):
    nrm = np.linalg.norm(ref, axis=1)
    live = nrm > 0
    rel = np.linalg.norm(a - ref, axis=1)[live] / nrm[live]
    assert rel.max() < 1e-12, rel.max()
    assert np.all(a[~live] == 0.0)


def _assert_oracle(a, state, k=512):
    n = state["x"].shape[0]
    tg = np.sort(np.random.default_rng(n).choice(n, min(n, k), replace=False))
    ref = O.direct_f64(state, EPS20, targets=tg, threads=os.cpu_count() or 1)
    assert O.rel_l2(a[tg], ref, state["status"][tg])[0] < 2e-6


def test_noalloc_matches_regular_entry_point_twice():
    torch = pytest.importorskip("torch")
    L = sv.load()
    L.sv_direct_accel_noalloc.restype = C.c_int
    n1, n2 = 20000, 12345
    s1 = plume.make_plume(n1, 2e-6, 501)
    s2 = plume.make_plume(n2, 5e-6, 502)
    s2["status"][:300] = 2
    s2["status"][300:400] = 0
    a3_dev = torch.empty((max(n1, n2), 3), dtype=torch.float64, device="cuda:0")

    rc, a1, _, _ = _noalloc(L, torch, s1, a3_dev)
    assert rc == 0
    _assert_close(a1, _regular(s1))
    _assert_oracle(a1, s1)

    # second call: smaller plume, other statuses, same static array
    rc, a2, free_before, free_after = _noalloc(L, torch, s2, a3_dev)
    assert rc == 0
    _assert_close(a2, _regular(s2))
    _assert_oracle(a2, s2)
    assert np.all(a2[300:400] == 0.0) and np.all(a2[:300] == 0.0)
    assert free_after >= free_before

    # the stated maximum size: keys, sorted copy and the sort's temporary
    # storage all inside the static array
    nmax = 262144
    s3 = plume.make_plume(nmax, 20e-6, 503)
    big = torch.empty((nmax, 3), dtype=torch.float64, device="cuda:0")
    rc, a3, free_before, free_after = _noalloc(L, torch, s3, big)
    assert rc == 0
    _assert_close(a3, _regular(s3))
    _assert_oracle(a3, s3)
    assert free_after >= free_before

    # sizes beyond the stated maximum are refused before any work
    rc = L.sv_direct_accel_noalloc(C.c_int64(262144 + 1), C.c_void_p(a3_dev.data_ptr()),
                                   C.c_void_p(a3_dev.data_ptr()), C.c_void_p(a3_dev.data_ptr()),
                                   C.c_void_p(a3_dev.data_ptr()), C.c_double(EPS20), C.c_double(1.0),
                                   C.c_void_p(a3_dev.data_ptr()), None)
    assert rc == 5
