"""Snapshot records (sv_snapshot) against the snapshot files written by the
reference's own integrators (Integrator::saveData, newOriginal layout) in
tests/golden/substeps.npz: the records at the start are the uploaded state
bit for bit; at the end, positions and velocities agree to the reference's
FP32 accuracy and the particle-particle field E1 to its force accuracy."""
import numpy as np
import pytest

import solveit_gpu as sv
from test_oracle_substeps import SUBSTEP_CASES, fixture

pytestmark = pytest.mark.gpu

REC = np.dtype([("index", "<i4"), ("species", "<u4"), ("f", "<f4", (12,))])


def split_file(raw, n_first):
    """The two saveData calls of a run: at the start (n_first records) and at the end."""
    first = raw[:12 + 56 * n_first]
    return first, raw[len(first):]


def records(buf):
    head = buf[:12]
    return head[:4].view("<u4")[0], head[4:8].view("<i4")[0], head[8:12].view("<f4")[0], buf[12:].view(REC)


@pytest.mark.parametrize("name", ["single"] + sorted(SUBSTEP_CASES))
def test_snapshots_match_reference_files(name):
    g = fixture()
    n = g["pos4"].shape[0]
    steps, dt = int(g["steps"]), np.float32(g["dt"])
    ref0, ref1 = split_file(g[name + "_snapshot"], n)
    with sv.ForceMethod(softening2=float(g["eps"]), precision=sv.FP64) as fm:
        fm.upload_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
        if name != "single":
            fm.set_substeps(float(dt), SUBSTEP_CASES[name])
        s0 = fm.snapshot(sv.SNAPSHOT_NEW_ORIGINAL, 0, n, 0.0)
        fm.leapfrog(steps, float(dt))
        t_end = np.float32(dt * np.float32(steps))
        last = int(np.searchsorted(g["tinj"], np.float32(dt * np.float32(steps)), side="right"))
        s1 = fm.snapshot(sv.SNAPSHOT_NEW_ORIGINAL, 0, last, float(t_end))
        s1o = fm.snapshot(sv.SNAPSHOT_ORIGINAL, 0, last, float(t_end))
    # the start of the run: the uploaded FP32 state, no field yet
    assert s0.tobytes() == ref0.tobytes()
    tag, lp, tm, rec = records(s1)
    rtag, rlp, rtm, rrec = records(ref1)
    assert (tag, lp, tm) == (rtag, rlp, rtm)
    assert np.array_equal(rec["index"], rrec["index"]) and np.array_equal(rec["species"], rrec["species"])
    f, rf = rec["f"].astype(np.float64), rrec["f"].astype(np.float64)
    assert np.max(np.abs(f[:, :3] - rf[:, :3])) < 5e-12
    vr = np.linalg.norm(rf[:, 3:6], axis=1)
    assert np.max(np.abs(f[:, 3:6] - rf[:, 3:6]).max(1) / vr) < 1e-5
    e1 = np.linalg.norm(rf[:, 6:9], axis=1)
    live = e1 > 0
    assert live.sum() > n // 4
    # E1 is the sum over close pairs: the reference's FP32 positions (rounded
    # at every one of up to 27 drifts per step) move it by up to ~1e-3 for a
    # particle with a near neighbour; typical particles agree far better
    rel = np.abs(f[live, 6:9] - rf[live, 6:9]).max(1) / e1[live]
    assert np.median(rel) < 1e-4 and rel.max() < 5e-3
    assert np.all(f[~live, 6:9] == 0) and np.all(f[:, 9:12] == 0) and np.all(rf[:, 9:12] == 0)
    # the original layout carries the same fields
    orig = s1o.view(np.dtype([("f", "<f4", (12,)), ("species", "<u4"), ("index", "<i4"), ("last", "<i4")]))
    assert np.array_equal(orig["f"], rec["f"]) and np.array_equal(orig["index"], rec["index"])
    assert np.all(orig["last"] == last)


def test_snapshot_field_of_the_kick():
    """E2 is the background field at each inbound particle's last kick."""
    import plume

    st = plume.make_plume(3000, 1e-6, 95)
    st["status"][:50] = 2
    with sv.ForceMethod(softening2=1e-20, efield=(1e6, 0.0, 3e8)) as fm:
        fm.upload(st)
        fm.leapfrog(2, 1e-13)
        rec = fm.snapshot(sv.SNAPSHOT_NEW_ORIGINAL)[12:].view(REC)
    e2 = rec["f"][:, 9:12]
    kicked = rec["index"] >= 50
    assert np.all(e2[kicked] == np.float32([1e6, 0.0, 3e8])) and np.all(e2[~kicked] == 0)
