"""The single-emitter background field on the GPU (sv_set_emitter_field,
sv_emitter_field_at, the kick of sv_leapfrog) against the FP64 oracle and the
reference's own outputs (tests/golden/emitter_field.npz)."""
import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv
from test_oracle_emitter_field import field_of, fixture, inside_map

pytestmark = pytest.mark.gpu

EPS20 = 1e-20


def set_field(fm, g):
    fm.set_emitter_field(g["node_rz"], g["e_r"], g["e_z"], g["triangles"], g["neighbors"], float(g["r0"]),
                         float(g["e0"]))


def test_field_at_points():
    g = fixture()
    st = plume.from_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
    with sv.ForceMethod(softening2=EPS20) as fm:
        set_field(fm, g)
        e = fm.emitter_field_at(st["x"])
    ins = inside_map(g, st["x"])
    e64 = O.emitter_field_f64(field_of(g), st["x"])
    # same walk, same barycentric arithmetic (no fused multiply-adds): FP64 round-off
    np.testing.assert_allclose(e[ins], e64[ins], rtol=1e-13, atol=1e-30)
    ref = g["e_out"].astype(np.float64)
    rel = np.abs(e[ins] - ref[ins]).max(1) / np.linalg.norm(ref[ins], axis=1)
    assert rel.max() < 5e-7
    z = st["x"][:, 2] / float(g["r0"])
    assert np.all(e[(z < 0) | (z > 140)] == 0)
    # outside the map the field is extrapolated from a hull triangle
    assert np.all(np.isfinite(e))


@pytest.mark.parametrize("prec", [sv.FP64, sv.MIXED])
def test_leapfrog_with_field_matches_reference(prec):
    g = fixture()
    with sv.ForceMethod(softening2=float(g["eps"]), precision=prec) as fm:
        fm.upload_ref32(g["dkd_pos4"], g["dkd_vel4"], g["dkd_acc4"], g["dkd_tinj"])
        set_field(fm, g)
        fm.leapfrog(int(g["steps"]), float(g["dt"]))
        x, v, _ = fm.download()
    vr = g["dkd_vel4_out"][:, :3]
    assert np.max(np.abs(x - g["dkd_pos4_out"][:, :3])) < 2e-12
    assert np.max(np.abs(v - vr).max(1) / np.linalg.norm(vr, axis=1)) < 2e-6


def test_leapfrog_with_field_matches_oracle():
    g = fixture()
    st = plume.from_ref32(g["dkd_pos4"], g["dkd_vel4"], g["dkd_acc4"], g["dkd_tinj"])
    ez = (0.0, 0.0, 3e7)  # the uniform field adds to the map's
    xr, vr, _, _ = O.leapfrog_f64_bc(st, 10, 1e-12, EPS20, ez, fld=field_of(g))
    with sv.ForceMethod(softening2=EPS20, precision=sv.FP64, efield=ez) as fm:
        fm.upload(st)
        set_field(fm, g)
        fm.leapfrog(6, 1e-12)
        fm.leapfrog(4, 1e-12, 6e-12)
        x, v, _ = fm.download()
    assert np.max(np.abs(x - xr)) < 1e-15 + 1e-12 * np.max(np.abs(xr))
    assert np.max(np.abs(v - vr).max(1) / np.linalg.norm(vr, axis=1)) < 1e-10


def test_batch_with_field():
    g = fixture()
    states = [plume.make_plume(n, 1.2e-6, 9100 + i) for i, n in enumerate((3000, 9000))]
    methods, syms = [sv.DIRECT, sv.FMM], [sv.SYM_NONE, sv.SYM_NONE]
    with sv.ForceMethod(softening2=EPS20, fmm_order=8, fmm_ws=2) as fm:
        fm.upload_batch(states, methods, syms)
        set_field(fm, g)
        fm.leapfrog(5, 1e-12)
        _, v, _ = fm.download()
    o = 0
    for s, meth in zip(states, methods):
        n = s["x"].shape[0]
        _, vr, _, _ = O.leapfrog_f64_bc(s, 5, 1e-12, EPS20, fld=field_of(g))
        dv = np.linalg.norm(vr - s["v"])
        tol = 1e-5 if meth == sv.DIRECT else 1e-4
        assert np.linalg.norm(v[o:o + n] - vr) <= tol * dv, (meth, np.linalg.norm(v[o:o + n] - vr) / dv)
        o += n


def test_field_errors_and_removal():
    g = fixture()
    st = plume.make_plume(500, 1.2e-6, 9200)
    with sv.ForceMethod(softening2=EPS20) as fm:
        bad = g["triangles"].copy()
        bad[3, 1] = len(g["e_r"])
        with pytest.raises(sv.SolveitError):
            fm.set_emitter_field(g["node_rz"], g["e_r"], g["e_z"], bad, g["neighbors"], 1e-8, 1e9)
        with pytest.raises(sv.SolveitError):
            fm.emitter_field_at(st["x"])  # no map set
        fm.upload(st)
        set_field(fm, g)
        with pytest.raises(sv.SolveitError):
            fm.adjoint_forward(2, 1e-13, 0.0, 1)  # the adjoint covers the uniform field only
        fm.set_emitter_field(None, None, None, None, None, 1.0, 0.0)
        fm.leapfrog(2, 1e-13)
        _, v, _ = fm.download()
    xr, vr, _, _ = O.leapfrog_f64_bc(st, 2, 1e-13, EPS20)
    assert np.linalg.norm(v - vr) <= 1e-5 * np.linalg.norm(vr - st["v"])
