"""The energy bookkeeping on the GPU (sv_set_energy, sv_get_energy_records)
against the energy files of the reference's own LeapfrogDKD::runSimulation
(tests/golden/energy.npz) and against the oracle's FP32 restatement of it;
the full-state snapshot (saveFullCurrentConditions).

Tolerance: the reference integrates with FP32 positions and sums its energies
in FP32 in index order; the GPU integrates in FP64 and sums in FP64 (pair
terms of the potential in FP32 on hi + lo offsets).  Every record component
agrees to a relative 2e-5 of the reference's value; components that are zero
in the reference (no emitter field) are zero.
"""
import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv
from test_oracle_emitter_field import field_of
from test_oracle_energy import CASES, fixture

pytestmark = pytest.mark.gpu

RTOL = 2e-5


def set_field(fm, g):
    fm.set_emitter_field(g["node_rz"], g["e_r"], g["e_z"], g["triangles"], g["neighbors"], float(g["r0"]),
                         float(g["e0"]))


def as_array(rec):
    return np.stack([rec[k] for k in sv.ENERGY_DTYPE.names], axis=1).astype(np.float64)


def assert_records_close(got, ref, rtol=RTOL):
    ref = np.asarray(ref, np.float64)
    assert got.shape == ref.shape
    zero = ref == 0
    assert np.all(got[zero] == 0)
    rel = np.abs(got[~zero] - ref[~zero]) / np.abs(ref[~zero])
    assert rel.max() < rtol, rel.max()


def run_gpu(g, name, prec=sv.FP64):
    init, each, interval, fld = (int(v) for v in g[f"{name}_setup"])
    with sv.ForceMethod(softening2=float(g["eps"]), precision=prec) as fm:
        fm.upload_ref32(g[f"{name}_pos4"], g[f"{name}_vel4"], g[f"{name}_acc4"], g[f"{name}_tinj"])
        if fld:
            set_field(fm, g)
        fm.set_energy(init, each, interval)
        fm.leapfrog(int(g["steps"]), float(g["dt"]))
        return as_array(fm.energy_records())


@pytest.mark.parametrize("prec", [sv.FP64, sv.MIXED])
@pytest.mark.parametrize("name", CASES)
def test_energy_records_match_reference(name, prec):
    g = fixture()
    assert_records_close(run_gpu(g, name, prec), g[f"{name}_records"])


def test_energy_matches_oracle_on_a_larger_plume():
    """2000 ions in four injection groups, the emitter field, a record every
    step, calls split mid-run: the GPU against the oracle's restatement."""
    g = fixture()
    st = plume.make_plume(2000, 1.2e-6, 9060)
    st["t_inj"][:] = np.floor(np.arange(2000) / 500) * 1.01e-12
    st["status"][[3, 999]] = 2
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    eps, dt, steps = 1e-20, 1e-12, 5
    _, _, _, ref = O.leapfrog_ref32_energy(pos4, vel4, acc4, tinj, steps, dt, eps, 30, 10, 1, fld=field_of(g),
                                           threads=8)
    with sv.ForceMethod(softening2=eps, precision=sv.FP64) as fm:
        fm.upload_ref32(pos4, vel4, acc4, tinj)
        set_field(fm, g)
        fm.set_energy(30, 10, 1)
        fm.leapfrog(2, dt)
        first = as_array(fm.energy_records())
        fm.leapfrog(3, dt, 2 * dt)
        rest = as_array(fm.energy_records())
    assert first.shape[0] == 2 and rest.shape[0] == 3
    assert_records_close(np.concatenate([first, rest]), ref)


def test_energy_rearm_and_errors():
    g = fixture()
    name = "field"
    args = (g[f"{name}_pos4"], g[f"{name}_vel4"], g[f"{name}_acc4"], g[f"{name}_tinj"])
    dt = float(g["dt"])
    with sv.ForceMethod(softening2=float(g["eps"]), precision=sv.FP64) as fm:
        with pytest.raises(sv.SolveitError):
            fm.set_energy(10, 10, 0)
        fm.upload_ref32(*args)
        set_field(fm, g)
        fm.set_energy(40, 20, 2)
        fm.leapfrog(4, dt)
        a = as_array(fm.energy_records())
        assert a.shape[0] == 2 and fm.energy_records().shape[0] == 0  # drained
        # a new upload sets up again and clears what was not drained
        fm.leapfrog(2, dt, 4 * dt)
        fm.upload_ref32(*args)
        assert fm.energy_records().shape[0] == 0
        fm.leapfrog(4, dt)
        np.testing.assert_allclose(as_array(fm.energy_records()), a, rtol=1e-6)
        with pytest.raises(sv.SolveitError):
            fm.adjoint_forward(2, dt, 0.0, 1)
        fm.set_substeps(dt, [(3.4e-13, 1, (0.0, 0.0, 0.0, 1.4e-8), 0.0)])
        with pytest.raises(sv.SolveitError):
            fm.leapfrog(1, dt)
        fm.set_substeps(dt, [])
        fm.set_energy(0, 0, 1, enable=False)
        fm.leapfrog(2, dt, 4 * dt)
        assert fm.energy_records().shape[0] == 0
    states = [plume.make_plume(n, 1e-6, 9070 + n) for n in (500, 700)]
    with sv.ForceMethod(softening2=1e-20) as fm:
        fm.upload_batch(states, [sv.DIRECT, sv.DIRECT], [sv.SYM_NONE, sv.SYM_NONE])
        with pytest.raises(sv.SolveitError):
            fm.set_energy(10, 10, 1)


REC = np.dtype([("index", "<i4"), ("species", "<u4"), ("f", "<f4", (12,))])
REC_ORIG = np.dtype([("f", "<f4", (12,)), ("species", "<u4"), ("index", "<i4"), ("last", "<i4")])


def test_full_snapshot_holds_every_particle():
    """saveFullCurrentConditions: every particle in index order whatever its
    status or injection time; the records of the particles saveData keeps
    are the same bytes in both."""
    n = 600
    st = plume.make_plume(n, 1e-6, 9080)
    st["t_inj"][:] = np.floor(np.arange(n) / 200) * 2.03e-12
    st["status"][[5, 6]] = 0
    st["status"][[7]] = -1
    st["status"][[8]] = 2
    dt = 1e-12
    with sv.ForceMethod(softening2=1e-20, precision=sv.FP64) as fm:
        fm.upload(st)
        fm.leapfrog(3, dt)
        x, v, status = fm.download()
        last = 400
        part = fm.snapshot(sv.SNAPSHOT_NEW_ORIGINAL, 0, last, 3e-12)
        full = fm.snapshot(sv.SNAPSHOT_NEW_ORIGINAL | sv.SNAPSHOT_FULL, 0, last, 3e-12)
        full_o = fm.snapshot(sv.SNAPSHOT_ORIGINAL | sv.SNAPSHOT_FULL, 123, last, 3e-12)
    assert full.size == 12 + 56 * n and full_o.size == 60 * n
    assert full[:12].tobytes() == part[:12].tobytes()
    rec = full[12:].view(REC)
    assert np.array_equal(rec["index"], np.arange(n))
    assert np.array_equal(rec["f"][:, :3], x.astype(np.float32))
    assert np.array_equal(rec["f"][:, 3:6], v.astype(np.float32))
    sub = part[12:].view(REC)
    keep = (np.arange(n) < last) & ((status == 1) | (status == 2))
    assert np.array_equal(sub["index"], np.nonzero(keep)[0])
    assert full[12:].reshape(n, 56)[keep].tobytes() == part[12:].tobytes()
    ro = full_o.view(REC_ORIG)
    assert np.array_equal(ro["index"], np.arange(n)) and np.all(ro["last"] == last)
    assert np.array_equal(ro["f"], rec["f"]) and np.array_equal(ro["species"], rec["species"])


def test_energy_records_of_an_empty_state():
    st = {k: v[:0] for k, v in plume.make_plume(1, 1e-6, 9090).items()}
    with sv.ForceMethod(softening2=1e-20, precision=sv.FP64) as fm:
        fm.upload(st)
        fm.set_energy(10, 10, 1)
        fm.leapfrog(2, 1e-12)
        rec = as_array(fm.energy_records())
    # the reference writes a record per interval whatever the window holds
    assert rec.shape == (2, 6) and np.all(rec == 0)
