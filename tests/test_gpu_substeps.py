"""The multi-rate leapfrog on the GPU (sv_set_substeps + sv_leapfrog)
against the reference's own LeapfrogDKDSubsteps::runSimulation
(tests/golden/substeps.npz) and the oracle's bit-exact restatement of it;
the single-rate sv_leapfrog against the reference's LeapfrogDKD::runSimulation.

The reference integrates in FP32: statuses and substep levels must be
identical, positions and velocities agree to its accuracy."""
import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv
from test_oracle_substeps import SUBSTEP_CASES, args_of, fixture

pytestmark = pytest.mark.gpu


def run_gpu(g, subs, prec=sv.FP64, steps=None):
    with sv.ForceMethod(softening2=float(g["eps"]), precision=prec) as fm:
        fm.upload_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
        if subs:
            fm.set_substeps(float(g["dt"]), subs)
        n = int(g["steps"]) if steps is None else steps
        fm.leapfrog(n, float(g["dt"]))
        x, v, status = fm.download()
        lev = fm.substep_levels() if subs else None
    return x, v, status, lev


def close_to(x, v, pr, vr):
    assert np.max(np.abs(x - pr[:, :3])) < 5e-12
    assert np.max(np.abs(v - vr[:, :3]).max(1) / np.linalg.norm(vr[:, :3], axis=1)) < 1e-5


def test_single_rate_matches_reference_integrator():
    g = fixture()
    x, v, status, _ = run_gpu(g, None)
    assert np.array_equal(status, g["single_acc4_out"][:, 3].astype(np.int32))
    close_to(x, v, g["single_pos4_out"], g["single_vel4_out"])


@pytest.mark.parametrize("name", sorted(SUBSTEP_CASES))
@pytest.mark.parametrize("prec", [sv.FP64, sv.MIXED])
def test_substeps_match_reference(name, prec):
    g = fixture()
    x, v, status, lev = run_gpu(g, SUBSTEP_CASES[name], prec)
    _, _, _, lev_ref = O.leapfrog_substeps_ref32(*args_of(g), SUBSTEP_CASES[name])
    assert np.array_equal(lev, lev_ref)
    assert np.array_equal(status, g[name + "_acc4_out"][:, 3].astype(np.int32))
    close_to(x, v, g[name + "_pos4_out"], g[name + "_vel4_out"])


def test_substeps_other_plume_against_oracle():
    """A second seed and more particles: the GPU against the oracle's
    restatement (the reference's arithmetic) of the same run."""
    st = plume.make_plume(1500, 1e-6, 9050)
    st["t_inj"][:] = np.floor(np.arange(1500) / 300) * 1.53e-12
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    subs = SUBSTEP_CASES["nested"]
    p, vr, a, lev_ref = O.leapfrog_substeps_ref32(pos4, vel4, acc4, tinj, 5, 1e-12, 1e-20, subs)
    with sv.ForceMethod(softening2=1e-20, precision=sv.FP64) as fm:
        fm.upload_ref32(pos4, vel4, acc4, tinj)
        fm.set_substeps(1e-12, subs)
        fm.leapfrog(2, 1e-12)
        fm.leapfrog(3, 1e-12, 2e-12)
        x, v, status = fm.download()
        lev = fm.substep_levels()
    assert np.mean(lev == lev_ref) > 0.998 and np.mean(status == a[:, 3]) > 0.998
    same = (lev == lev_ref) & (status == a[:, 3])
    assert np.max(np.abs(x[same] - p[same, :3])) < 5e-12
    assert np.max(np.abs(v[same] - vr[same, :3]).max(1) / np.linalg.norm(vr[same, :3], axis=1)) < 1e-5


def test_substeps_switch_off_and_errors():
    g = fixture()
    with sv.ForceMethod(softening2=float(g["eps"]), precision=sv.FP64) as fm:
        fm.upload_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
        fm.set_substeps(float(g["dt"]), SUBSTEP_CASES["core"])
        with pytest.raises(sv.SolveitError):
            fm.leapfrog(1, 2e-12)  # not the table's step
        with pytest.raises(sv.SolveitError):
            fm.adjoint_forward(1, float(g["dt"]), 0.0, 1)
        fm.set_substeps(float(g["dt"]), [])
        fm.leapfrog(int(g["steps"]), float(g["dt"]))
        x, v, status = fm.download()
    assert np.array_equal(status, g["single_acc4_out"][:, 3].astype(np.int32))
    close_to(x, v, g["single_pos4_out"], g["single_vel4_out"])
