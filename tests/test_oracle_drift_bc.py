"""The drift's injection window, crash test, folding and boundary conditions:
the oracle pinned against the reference's own code (tests/golden/drift_bc.npz,
made by tests/golden/make_golden.py from ParticleSystem::propagatePositionNew,
findMostRecentInjected and the events file)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
sys.path.insert(0, os.path.join(HERE, "..", "solveit-code_gb300"))
import oracle_py as O  # noqa: E402
import plume  # noqa: E402

# the three fixture cases: symmetry and the reference's crash / boundary keys
CASES = {
    "plain": (0, dict(crash=1, cz=5e-7, cw=1e-7, cr=1e-8, bc=3, bz=9e-7, br=2.5e-8, bt=5.25e-12)),
    "rot": (1, dict(crash=1, cz=5e-7, cw=1e-7, cr=1e-8, bc=1, bz=9e-7, br=2.5e-8)),
    "trans": (2, dict()),
}
DOMAIN = (2e-6, 2e-6, 0.0)
AXES = (1, 1, 0)


def fixture():
    return np.load(os.path.join(HERE, "golden", "drift_bc.npz"))


def boundary_of(sym, keys, fold):
    return O.boundary(crash=keys.get("crash", 0), crash_z=keys.get("cz", 0.0), crash_width=keys.get("cw", 0.0),
                      crash_r=keys.get("cr", 0.0), bc=keys.get("bc", 0),
                      bc_space=(keys.get("bx", 0.0), keys.get("by", 0.0), keys.get("bz", 0.0), keys.get("br", 0.0)),
                      bc_time=keys.get("bt", 0.0), fold=sym if fold else 0, axes=AXES, domain=DOMAIN)


def ref_events(g, name):
    return np.frombuffer(g[name + "_events"].tobytes(), O.EVENT_DTYPE)


def test_fixture_exercises_every_path():
    g = fixture()
    st_plain = g["plain_acc4_out"][:, 3]
    assert (st_plain == -1).sum() > 10 and (st_plain == 0).sum() > 10
    ev = ref_events(g, "plain")
    assert set(np.unique(ev["status"])) == {-1, 0}
    assert len(np.unique(g["plain_tinj"])) == 8  # staggered injection groups
    # the translational plume straddles x = L/2 and is folded back
    assert (g["trans_pos4"][:, 0] > 1e-6).any() and (g["trans_pos4_out"][:, 0] < 0).any()


@pytest.mark.parametrize("name", sorted(CASES))
def test_ref32_bit_exact(name):
    g = fixture()
    sym, keys = CASES[name]
    imgs = O.trans_images(2, AXES, lattice=g["lattice"]) if sym == 2 else None
    p, v, a, ev = O.leapfrog_ref32_bc(g[name + "_pos4"], g[name + "_vel4"], g[name + "_acc4"], g[name + "_tinj"],
                                      int(g["steps"]), float(g["dt"]), float(g["eps"]), (0.0, 0.0, float(g["ez"])),
                                      sym=sym, bd=boundary_of(sym, keys, False), images=imgs, domain_size=DOMAIN)
    assert np.array_equal(p, g[name + "_pos4_out"])
    assert np.array_equal(v, g[name + "_vel4_out"])
    assert np.array_equal(a, g[name + "_acc4_out"])
    assert ev.tobytes() == g[name + "_events"].tobytes()


@pytest.mark.parametrize("name", sorted(CASES))
def test_f64_matches_reference(name):
    """The FP64 restatement (the GPU's semantics: a per-particle injection
    test) takes the same decisions as the reference's FP32 loop."""
    g = fixture()
    sym, keys = CASES[name]
    st = plume.from_ref32(g[name + "_pos4"], g[name + "_vel4"], g[name + "_acc4"], g[name + "_tinj"])
    off = O.trans_images(2, AXES, lattice=g["lattice"]) * np.array(DOMAIN) if sym == 2 else None
    x, v, status, ev = O.leapfrog_f64_bc(st, int(g["steps"]), float(g["dt"]), float(g["eps"]),
                                         (0.0, 0.0, float(g["ez"])), sym=sym, img_off=off,
                                         bd=boundary_of(sym, keys, True))
    pr, vr, ar = g[name + "_pos4_out"], g[name + "_vel4_out"], g[name + "_acc4_out"]
    assert np.array_equal(status, ar[:, 3].astype(np.int32))
    evr = ref_events(g, name)
    assert len(ev) == len(evr)
    for f in ("index", "species", "status"):
        assert np.array_equal(ev[f], evr[f]), f
    # the reference keeps time and positions in FP32
    assert np.max(np.abs(ev["time"] - evr["time"])) < 1e-16 if len(ev) else True
    assert np.max(np.abs(x - pr[:, :3])) < 5e-12
    assert np.max(np.abs(v - vr[:, :3]).max(1) / np.linalg.norm(vr[:, :3], axis=1)) < 1e-5


def test_window_excludes_particles_not_yet_injected():
    """A particle injected after the step's mid time neither exerts nor feels
    force in that step (lastParticle, integration_schemes.cpp:711-713)."""
    st = plume.make_plume(64, 1e-7, 31)
    st["t_inj"][:] = 0.0
    late = dict((k, v.copy()) for k, v in st.items())
    late["t_inj"][40:] = 0.8e-13  # after the mid time 0.5e-13 of the first step
    ref = dict((k, v[:40].copy()) for k, v in st.items())
    x1, v1, _, _ = O.leapfrog_f64_bc(late, 1, 1e-13, 1e-20, (0.0, 0.0, 1e8))
    x0, v0, _, _ = O.leapfrog_f64_bc(ref, 1, 1e-13, 1e-20, (0.0, 0.0, 1e8))
    assert np.array_equal(v1[:40], v0)
    assert np.array_equal(x1[:40], x0)
    # the late particles drift for the part of the second half step after injection, unkicked
    s = 1e-13 - 0.8e-13
    assert np.allclose(x1[40:], st["x"][40:] + st["v"][40:] * s, rtol=0, atol=1e-20)
    assert np.array_equal(v1[40:], st["v"][40:])


def test_ref32_window_matches_f64_window():
    """findMostRecentInjected's binary search (sorted injection times) and the
    per-particle test select the same particles."""
    st = plume.make_plume(300, 1e-6, 32)
    st["t_inj"][:] = np.sort(np.random.default_rng(3).uniform(0, 6e-13, 300))
    st["t_inj"][0] = 0.0
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    st32 = plume.from_ref32(pos4, vel4, acc4, tinj)
    p, v, a, _ = O.leapfrog_ref32_bc(pos4, vel4, acc4, tinj, 6, 1e-13, 1e-20, (0.0, 0.0, 1e8))
    x, vv, _, _ = O.leapfrog_f64_bc(st32, 6, 1e-13, 1e-20, (0.0, 0.0, 1e8))
    moved32 = np.any(v[:, :3] != vel4[:, :3], axis=1)
    moved64 = np.any(vv != st32["v"], axis=1)
    assert np.array_equal(moved32, moved64)
    assert np.max(np.abs(vv - v[:, :3]).max(1) / np.linalg.norm(v[:, :3], axis=1)) < 1e-5
