"""sv_leapfrog's injection window, crash test, folding, boundary conditions
and event records on the GPU, against the reference's own outputs
(tests/golden/drift_bc.npz) and the FP64 oracle.

The reference integrates in FP32, so positions and velocities are compared
to its accuracy; statuses and event records (index, species, status) must be
identical, and event times and positions agree to FP32 rounding.
"""
import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv
from test_oracle_drift_bc import AXES, CASES, DOMAIN, boundary_of, fixture, ref_events

pytestmark = pytest.mark.gpu

EPS20 = 1e-20


def ctx_kwargs(g, sym, prec, method=sv.DIRECT):
    kw = dict(softening2=float(g["eps"]), precision=prec, method=method, efield=(0.0, 0.0, float(g["ez"])),
              symmetry=sym)
    if sym == sv.SYM_TRANSLATIONAL:
        kw.update(sym_axes=AXES, sym_levels=2, domain_size=DOMAIN)
    return kw


def set_boundary(fm, sym, keys):
    fm.set_boundary(crash=keys.get("crash", 0), crash_z=keys.get("cz", 0.0), crash_width=keys.get("cw", 0.0),
                    crash_r=keys.get("cr", 0.0), bc=keys.get("bc", 0),
                    bc_space=(keys.get("bx", 0.0), keys.get("by", 0.0), keys.get("bz", 0.0), keys.get("br", 0.0)),
                    bc_time=keys.get("bt", 0.0), fold=1 if sym else 0)


@pytest.mark.parametrize("name", sorted(CASES))
@pytest.mark.parametrize("prec", [sv.FP64, sv.MIXED])
def test_matches_reference_fixture(name, prec):
    g = fixture()
    sym, keys = CASES[name]
    with sv.ForceMethod(**ctx_kwargs(g, sym, prec)) as fm:
        fm.upload_ref32(g[name + "_pos4"], g[name + "_vel4"], g[name + "_acc4"], g[name + "_tinj"])
        set_boundary(fm, sym, keys)
        fm.leapfrog(int(g["steps"]), float(g["dt"]))
        x, v, status = fm.download()
        ev = fm.events()
        assert len(fm.events()) == 0  # the log was drained
    pr, vr, ar = g[name + "_pos4_out"], g[name + "_vel4_out"], g[name + "_acc4_out"]
    assert np.array_equal(status, ar[:, 3].astype(np.int32))
    evr = ref_events(g, name)
    assert len(ev) == len(evr)
    for f in ("index", "species", "status"):
        assert np.array_equal(ev[f], evr[f]), f
    if len(ev):
        assert np.max(np.abs(ev["time"] - evr["time"])) < 1e-16
        for f in ("x", "y", "z"):
            assert np.max(np.abs(ev[f] - evr[f])) < 1e-12, f
    assert np.max(np.abs(x - pr[:, :3])) < 5e-12
    assert np.max(np.abs(v - vr[:, :3]).max(1) / np.linalg.norm(vr[:, :3], axis=1)) < 1e-5


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_matches_oracle(name):
    """FP64 GPU against the FP64 oracle with the same semantics: to round-off."""
    g = fixture()
    sym, keys = CASES[name]
    st = plume.from_ref32(g[name + "_pos4"], g[name + "_vel4"], g[name + "_acc4"], g[name + "_tinj"])
    off = O.trans_images(2, AXES, lattice=g["lattice"]) * np.array(DOMAIN) if sym == 2 else None
    xr, vr, sr, evr = O.leapfrog_f64_bc(st, int(g["steps"]), float(g["dt"]), float(g["eps"]),
                                        (0.0, 0.0, float(g["ez"])), sym=sym, img_off=off,
                                        bd=boundary_of(sym, keys, True))
    with sv.ForceMethod(**ctx_kwargs(g, sym, sv.FP64)) as fm:
        fm.upload(st)
        set_boundary(fm, sym, keys)
        fm.leapfrog(5, float(g["dt"]))
        fm.leapfrog(int(g["steps"]) - 5, float(g["dt"]), 5 * float(g["dt"]))  # a second call continues the log
        x, v, status = fm.download()
        ev = fm.events()
    assert np.array_equal(status, sr)
    assert ev.tobytes() == evr.tobytes() or (
        np.array_equal(ev["index"], evr["index"]) and np.array_equal(ev["status"], evr["status"])
        and np.max(np.abs(ev["time"] - evr["time"])) < 1e-20)
    assert np.max(np.abs(x - xr)) < 1e-15 + 1e-12 * np.max(np.abs(xr))
    assert np.max(np.abs(v - vr).max(1) / np.linalg.norm(vr, axis=1)) < 1e-10


def test_window_with_fmm_and_bh():
    """Particles not yet injected are outside the force's window for the tree
    methods too."""
    st = plume.make_plume(6000, 1e-6, 77)
    st["t_inj"][:] = np.floor(np.arange(6000) / 1000) * 1.3e-13  # the last group arrives after the run
    nsteps, dt, ez = 6, 1e-13, (0.0, 0.0, 1e8)
    xr, vr, _, _ = O.leapfrog_f64_bc(st, nsteps, dt, EPS20, ez)
    for method, tol in ((sv.FMM, 1e-3), (sv.BARNES_HUT, 1e-2)):
        kw = dict(fmm_order=8, fmm_ws=2) if method == sv.FMM else dict(theta=0.3)
        with sv.ForceMethod(softening2=EPS20, method=method, efield=ez, **kw) as fm:
            fm.upload(st)
            fm.leapfrog(nsteps, dt)
            x, v, _ = fm.download()
        dv = np.linalg.norm(vr - st["v"])
        assert np.linalg.norm(v - vr) <= tol * dv, (method, np.linalg.norm(v - vr) / dv)
        late = st["t_inj"] > (nsteps - 0.5) * dt
        assert late.sum() == 1000 and np.array_equal(v[late], st["v"][late])


def test_batch_boundary_and_folding():
    """Batched plumes: per-plume folding (rotational plumes only), the crash
    test and boundary conditions inside the captured step graph, events of
    every plume in one log."""
    sizes = [1200, 9000, 2500]
    methods = [sv.DIRECT, sv.FMM, sv.DIRECT]
    syms = [sv.SYM_ROTATIONAL, sv.SYM_NONE, sv.SYM_NONE]
    states = []
    for i, n in enumerate(sizes):
        s = plume.make_plume(n, 1e-6, 5100 + i)
        s["t_inj"][:] = np.floor(np.arange(n) / (n // 4)) * 1e-12
        states.append(s)
    keys = dict(crash=1, cz=5e-7, cw=1e-7, cr=1e-8, bc=3, bz=9e-7, br=2.5e-8, bt=5.25e-12)
    dt, nsteps, ez = 1e-12, 8, (0.0, 0.0, 1e8)
    with sv.ForceMethod(softening2=EPS20, efield=ez, fmm_order=6, fmm_ws=2) as fm:
        fm.upload_batch(states, methods, syms)
        set_boundary(fm, 1, keys)
        fm.leapfrog(4, dt)
        fm.leapfrog(nsteps - 4, dt, 4 * dt)
        x, v, status = fm.download()
        ev = fm.events()
    off = np.cumsum([0] + sizes)
    for p, (s, meth, sym) in enumerate(zip(states, methods, syms)):
        bd = boundary_of(sym, keys, True)
        xr, vr, sr, evr = O.leapfrog_f64_bc(s, nsteps, dt, EPS20, ez, sym=sym, bd=bd)
        mine = (ev["index"] >= off[p]) & (ev["index"] < off[p + 1])
        evp = ev[mine]
        assert len(evr) > 0
        sl = slice(off[p], off[p + 1])
        if meth == sv.DIRECT:
            # mixed-precision pairs: ~1e-6 of the Coulomb kick, far from every threshold
            assert np.array_equal(status[sl], sr)
            assert np.max(np.abs(x[sl] - xr)) < 1e-12
            # within a plume the merged log keeps the plume's own file order
            assert np.array_equal(evp["index"] - off[p], evr["index"])
            assert np.array_equal(evp["status"], evr["status"])
        else:
            # the FMM's p = 6 force error can move a particle across a threshold
            assert np.mean(status[sl] == sr) > 0.995
            assert abs(len(evp) - len(evr)) <= 0.01 * len(evr) + 2
        if sym == sv.SYM_ROTATIONAL:
            assert np.all(x[sl][:, 0] >= 0) and np.all(x[sl][:, 1] >= 0)
        else:
            assert np.any(x[sl][:, 0] < 0)


def test_events_order_and_drain():
    st = plume.make_plume(2000, 1e-6, 88)
    with sv.ForceMethod(softening2=EPS20) as fm:
        fm.upload(st)
        fm.set_boundary(bc=sv.BC_TIME, bc_time=0.0)  # every inbound particle leaves at the first drift
        fm.leapfrog(1, 1e-13)
        ev = fm.events()
        _, _, status = fm.download()
    assert len(ev) == 2000 and np.all(status == 0)
    assert np.array_equal(ev["index"], np.arange(2000))
    assert np.all(ev["time"] == np.float32(0.5e-13))


def test_adjoint_with_staggered_injection():
    """The adjoint follows the forward window: its dL/dE_z matches central
    differences of the FP64 oracle rollout with staggered injection."""
    st = plume.make_plume(384, 0.3e-6, 4010)
    st["t_inj"][:] = np.floor(np.arange(384) / 64) * 1.3e-13
    nsteps, dt, ez = 10, 1e-13, 1e8
    with sv.ForceMethod(softening2=EPS20, precision=sv.FP64, efield=(0.0, 0.0, ez)) as fm:
        fm.upload(st)
        fm.adjoint_forward(nsteps, dt, 0.0, 4)
        x, v, _ = fm.download()
        gv = np.zeros_like(v)
        gv[:, 2] = st["m"] / st["m"].size
        _, _, ge = fm.adjoint_backward(np.zeros_like(x), gv)
    h = 1e-6 * ez
    vals = []
    for e in (ez + h, ez - h):
        _, vv, _, _ = O.leapfrog_f64_bc(st, nsteps, dt, EPS20, (0.0, 0.0, e))
        vals.append(float(np.mean(st["m"] * vv[:, 2])))
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(ge[2] - fd) <= 1e-4 * abs(fd), (ge[2], fd)
    with sv.ForceMethod(softening2=EPS20) as fm:
        fm.upload(st)
        fm.set_boundary(fold=1)
        with pytest.raises(sv.SolveitError):
            fm.adjoint_forward(2, dt, 0.0, 1)
