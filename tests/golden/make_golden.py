"""Generate the golden fixtures in this directory by running the reference.

The reference SOLVEiT code is compiled from its own sources by
``make -C oracle ref`` (one-line header fix, see oracle/Makefile) into
oracle/_ref/{stock,eps20}/ref_harness, which fills the reference's
ChargedParticles by hand and calls its own updateAcceleration() /
propagate*New() methods.  This script feeds it seeded plumes and stores the
inputs and the reference's outputs as compressed .npz files, so the tests
can pin the oracle and the GPU path to the reference without the reference
being present.

    make -C oracle ref && python tests/golden/make_golden.py

Fixtures (all FP32 vec4 arrays in the reference layout):
  direct_n512.npz   direct sum, symmetry none / rotational / translational
                    (x,y periodic, 2 levels = 81 images), reference softening
                    6.4e-19 m^2; includes status 2 / 0 / -1 particles and the
                    Grid's lattice order.
  dkd_n256.npz      10 LeapfrogDKD steps (dt 1e-13 s, E_z 1e8 V/m, softening
                    1e-20 m^2, direct force).
  bh_n4096.npz      Barnes-Hut theta 0.5 (reference tree: 1 particle/leaf).
  fmm_n4096.npz     FMM p = 8 (reference uniform-depth rotation FMM).
  drift_bc.npz      10 LeapfrogDKD steps with staggered injection (the
                    driftNew window), the extractor-grid crash test, spatial
                    and temporal boundary conditions, rotational and
                    translational folding, and the events file
                    (``python tests/golden/make_golden.py drift_bc``).
  emitter_field.npz a seeded single-emitter field map (Delaunay triangulation
                    of jittered nodes, scipy) in the reference's Fields /
                    Triangles CSV format, InterpolationScheme::Efield at plume
                    particles (inside and outside the map) and 10 DKD steps
                    with computeBackgroundAcceleration
                    (``python tests/golden/make_golden.py emitter_field``).
  substeps.npz      the reference's own LeapfrogDKD::runSimulation and
                    LeapfrogDKDSubsteps::runSimulation (two substep tables)
                    over 6 steps with staggered injection, with the snapshot
                    files they write (``... make_golden.py substeps``).
  energy.npz        the reference's LeapfrogDKD::runSimulation with
                    toggleEnergy over 6 steps: the energy file's records,
                    without and with the emitter field and with inactive
                    particles at the front (``... make_golden.py energy``).
  bh_n65536_sampled.npz, fmm_n65536_z50_sampled.npz
                    the reference's Barnes-Hut (theta 0.5) at the treecode
                    workload's size and its FMM (p = 8) on the long 50 um
                    plume at N = 65,536 (the largest size it runs cleanly),
                    softening 1e-20 m^2: accelerations of every 64th particle
                    and those particles' positions
                    (``... make_golden.py sampled``).
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "solveit-code_gb300"))
import plume  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "{}", "ref_harness")
# scratch files of the harness runs stay inside the repository (oracle/_ref is git-ignored)
SCRATCH = os.path.join(ROOT, "oracle", "_ref", "scratch")


def scratch_dir():
    os.makedirs(SCRATCH, exist_ok=True)
    return tempfile.TemporaryDirectory(dir=SCRATCH)


def run_ref(variant, mode, pos4, vel4, acc4, tinj, **kw):
    n = pos4.shape[0]
    with scratch_dir() as td:
        fin = os.path.join(td, "in.bin")
        fout = os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([n], np.int32).tofile(f)
            for a in (pos4, vel4, acc4, tinj):
                np.ascontiguousarray(a).tofile(f)
        if "energy" in kw:
            kw = dict(kw, edir=os.path.join(td, "energy") + "/")
            os.mkdir(kw["edir"])
        args = [HARNESS.format(variant), mode, fin, fout] + [f"{k}={v}" for k, v in kw.items()]
        subprocess.check_call(args, stdout=subprocess.DEVNULL)
        if mode == "run":
            raw = np.fromfile(fout, np.uint8)
            out = raw[:48 * n].view(np.float32).reshape(3, n, 4)
            nb = int(raw[48 * n:48 * n + 4].view(np.int32)[0])
            snap = raw[48 * n + 4:48 * n + 4 + nb].copy()
            if "energy" in kw:
                o = 48 * n + 4 + nb
                cnt = int(raw[o:o + 4].view(np.int32)[0])
                rec = raw[o + 4:o + 4 + 24 * cnt].view(np.float32).reshape(cnt, 6).copy()
                return out[0].copy(), out[1].copy(), out[2].copy(), snap, rec
            return out[0].copy(), out[1].copy(), out[2].copy(), snap
        if mode == "efield":
            return np.fromfile(fout, np.float32).reshape(n, 3)
        if mode == "grid":
            raw = np.fromfile(fout, np.int32)
            return raw[1:].reshape(raw[0], 3)
        if mode == "outliers":
            raw = np.fromfile(fout, np.int32)
            return raw[1:].copy(), int(raw[0])
        raw = np.fromfile(fout, np.uint8)
        out = raw[:48 * n].view(np.float32).reshape(3, n, 4)
        if kw.get("events"):
            cnt = int(raw[48 * n:48 * n + 4].view(np.int32)[0])
            ev = raw[48 * n + 4:48 * n + 4 + 40 * cnt].copy()
            return out[0].copy(), out[1].copy(), out[2].copy(), ev
    return out[0].copy(), out[1].copy(), out[2].copy()


def main():
    # direct, three symmetry variants
    st = plume.make_plume(512, 1e-6, 9001)
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    acc4[5, 3] = 2.0   # affectsAcceleration: source only
    acc4[7, 3] = 0.0   # outOfBounds: ignored
    acc4[9, 3] = -1.0  # crashed: ignored
    lattice = run_ref("stock", "grid", pos4, vel4, acc4, tinj, levels=2, axes="110")
    outs = {}
    for sym in (0, 1, 2):
        _, _, a = run_ref("stock", "direct", pos4, vel4, acc4, tinj, threads=4, sym=sym,
                          levels=2, axes="110", dom="2e-6,2e-6,0")
        outs[f"acc_sym{sym}"] = a
    np.savez_compressed(os.path.join(HERE, "direct_n512.npz"), pos4=pos4, vel4=vel4, acc4=acc4,
                        tinj=tinj, lattice=lattice.astype(np.int32), eps=np.float64(6.4e-19),
                        domain=np.array([2e-6, 2e-6, 0.0], np.float32), **outs)

    # leapfrog DKD
    st = plume.make_plume(256, 1e-6, 9002)
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    p, v, a = run_ref("eps20", "dkd", pos4, vel4, acc4, tinj, threads=4, steps=10, dt=1e-13, ez=1e8)
    np.savez_compressed(os.path.join(HERE, "dkd_n256.npz"), pos4=pos4, vel4=vel4, acc4=acc4,
                        tinj=tinj, pos4_out=p, vel4_out=v, acc4_out=a, steps=np.int32(10),
                        dt=np.float32(1e-13), ez=np.float32(1e8), eps=np.float64(1e-20))

    # Barnes-Hut and FMM, reference softening
    st = plume.make_plume(4096, 1e-6, 9003)
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    _, _, ab = run_ref("stock", "bh", pos4, vel4, acc4, tinj, threads=4, theta=0.5)
    np.savez_compressed(os.path.join(HERE, "bh_n4096.npz"), pos4=pos4, vel4=vel4, acc4=acc4,
                        tinj=tinj, acc_bh=ab, theta=np.float32(0.5), eps=np.float64(6.4e-19))
    _, _, af = run_ref("stock", "fmm", pos4, vel4, acc4, tinj, threads=4, p=8)
    np.savez_compressed(os.path.join(HERE, "fmm_n4096.npz"), pos4=pos4, vel4=vel4, acc4=acc4,
                        tinj=tinj, acc_fmm=af, p=np.int32(8), eps=np.float64(6.4e-19))
    outliers()
    sampled_configs()
    print("fixtures written to", HERE)


def sampled_configs(ntarget=1024):
    """The reference's Barnes-Hut at the treecode workload's size (N = 65,536,
    z in [0, 10] um, theta 0.5, seed 1000) and its FMM at the largest size it
    runs cleanly with the long plume (N = 65,536, z in [0, 50] um, p 8, seed
    2000), softening 1e-10 m: accelerations of every 64th particle, with those
    particles' FP32 positions to check that the plume generator reproduces the
    same plume where the test runs."""
    for name, mode, length, seed, kw in (("bh_n65536_sampled.npz", "bh", 10e-6, 1000, dict(theta=0.5)),
                                         ("fmm_n65536_z50_sampled.npz", "fmm", 50e-6, 2000, dict(p=8))):
        n = 65536
        st = plume.make_plume(n, length, seed)
        pos4, vel4, acc4, tinj = plume.to_ref32(st)
        _, _, a = run_ref("eps20", mode, pos4, vel4, acc4, tinj, threads=os.cpu_count() or 4, **kw)
        tg = np.arange(0, n, n // ntarget, dtype=np.int32)
        np.savez_compressed(os.path.join(HERE, name), n=np.int32(n), length=np.float64(length),
                            seed=np.int64(seed), eps=np.float64(1e-20), targets=tg, pos4_targets=pos4[tg],
                            acc_ref=a[tg, :3].copy(), **{k: np.float64(v) for k, v in kw.items()})


def outliers():
    """isOutlier on plumes with ions far off the plume (odd and even counts)."""
    cases = {}
    for n, seed in ((2001, 9005), (2000, 9006)):
        st = plume.make_plume(n, 1e-6, seed)
        rng = np.random.default_rng(seed)
        st["x"][:6] += rng.normal(size=(6, 3)) * 5e-6
        pos4, vel4, acc4, tinj = plume.to_ref32(st)
        flags, count = run_ref("stock", "outliers", pos4, vel4, acc4, tinj)
        cases[f"n{n}"] = (pos4, vel4, acc4, tinj, flags, count)
    np.savez_compressed(os.path.join(HERE, "outliers.npz"),
                        **{f"{k}_{name}": v for k, c in cases.items()
                           for name, v in zip(("pos4", "vel4", "acc4", "tinj", "flags", "count"), c)})


# staggered injection: groups of 32 injected 1 ps apart (sorted, the first at 0)
DRIFT_BC_CASES = {
    # name: (sym, plume x offset, reference keys)
    "plain": (0, 0.0, dict(crash=1, cz=5e-7, cw=1e-7, cr=1e-8, bc=3, bz=9e-7, br=2.5e-8, bt=5.25e-12)),
    "rot": (1, 0.0, dict(crash=1, cz=5e-7, cw=1e-7, cr=1e-8, bc=1, bz=9e-7, br=2.5e-8)),
    "trans": (2, 9.95e-7, dict()),
}


def drift_bc_state(sym, xoff, seed=9010, n=256):
    st = plume.make_plume(n, 1e-6, seed)
    st["x"][:, 0] += xoff
    st["t_inj"][:] = np.floor(np.arange(n) / 32) * 1e-12
    st["status"][[17, 90, 201]] = 2  # source-only particles
    return st


def drift_bc():
    """The reference's own drift, crash, folding and boundary code on a plume
    that crosses the grid, leaves the bounds and is injected in groups."""
    out = {}
    for name, (sym, xoff, keys) in DRIFT_BC_CASES.items():
        st = drift_bc_state(sym, xoff)
        pos4, vel4, acc4, tinj = plume.to_ref32(st)
        extra = dict(levels=2, axes="110", dom="2e-6,2e-6,0") if sym == 2 else {}
        p, v, a, ev = run_ref("eps20", "dkd", pos4, vel4, acc4, tinj, threads=4, steps=10, dt=1e-12, ez=1e8,
                              sym=sym, events=1, **keys, **extra)
        out.update({f"{name}_pos4": pos4, f"{name}_vel4": vel4, f"{name}_acc4": acc4, f"{name}_tinj": tinj,
                    f"{name}_pos4_out": p, f"{name}_vel4_out": v, f"{name}_acc4_out": a, f"{name}_events": ev})
        print(name, "events", len(ev) // 40, "crashed", int((a[:, 3] == -1).sum()), "out",
              int((a[:, 3] == 0).sum()))
    st = drift_bc_state(0, 0.0)
    lattice = run_ref("eps20", "grid", *plume.to_ref32(st), levels=2, axes="110")
    np.savez_compressed(os.path.join(HERE, "drift_bc.npz"), steps=np.int32(10), dt=np.float32(1e-12),
                        ez=np.float32(1e8), eps=np.float64(1e-20), lattice=lattice.astype(np.int32),
                        domain=np.array([2e-6, 2e-6, 0.0], np.float32), **out)


def emitter_mesh(seed=9020, r_max=8.0, z_max=140.0):
    """Jittered (r, z) nodes in units of r0, their Delaunay triangulation
    (neighbour k across the edge opposite vertex k, -1 on the hull) and a
    smooth synthetic field in units of E0."""
    from scipy.spatial import Delaunay

    rng = np.random.default_rng(seed)
    r = np.linspace(0.0, r_max, 17)
    z = np.linspace(0.0, z_max, 141)
    rr, zz = np.meshgrid(r, z, indexing="ij")
    pts = np.stack([rr.ravel(), zz.ravel()], axis=1)
    inner = (pts[:, 0] > 0) & (pts[:, 0] < r_max) & (pts[:, 1] > 0) & (pts[:, 1] < z_max)
    pts[inner] += rng.uniform(-0.2, 0.2, (inner.sum(), 2)) * [r[1], z[1]]
    d = Delaunay(pts)
    er = 0.3 * pts[:, 0] * np.exp(-pts[:, 1] / 60.0) / (1.0 + 0.05 * pts[:, 0] ** 2)
    ez = np.exp(-pts[:, 1] / 40.0) * (1.0 - 0.02 * pts[:, 0]) + 0.1
    return pts, er, ez, d.simplices.astype(np.int32), d.neighbors.astype(np.int32)


def emitter_field():
    """The reference's InterpolationScheme reading a seeded field map through
    its own CSV readers; Efield at plume particles and a leapfrog with it."""
    nodes, er, ez, tri, nbr = emitter_mesh()
    r0, e0 = 1e-8, 1e9
    st = plume.make_plume(256, 1.2e-6, 9021)
    st["x"][:8, 2] = [-5e-8, -1e-9, 1.39e-6, 1.41e-6, 1.5e-6, 0.3e-6, 0.7e-6, 1.0e-6]  # z outside [0, 140 r0]
    st["x"][5:8, 0] = [9e-8, 1.2e-7, -1.0e-7]  # r outside the map: extrapolated
    st["x"][8, :2] = 0.0      # on the axis
    st["x"][9, 0] = 0.0       # on the y axis (phi = pi/2 whatever the sign of y)
    st["x"][9, 1] = -1e-8
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    with scratch_dir() as td:
        with open(os.path.join(td, "fields.csv"), "w") as f:
            for k in range(len(er)):
                f.write(f"{nodes[k, 0]:.17g},{nodes[k, 1]:.17g},{er[k]:.17g},{ez[k]:.17g}\n")
        with open(os.path.join(td, "triangles.csv"), "w") as f:
            for t, nb in zip(tri, nbr):
                f.write(",".join(str(int(v)) for v in (*t, *nb)) + "\n")
        keys = dict(fdir=td + "/", fnodes="fields.csv", ftris="triangles.csv", r0=r0, e0=e0)
        e_at = run_ref("eps20", "efield", pos4, vel4, acc4, tinj, **keys)
        # leapfrog inside the map only (the walk outside the hull depends on the search order)
        st2 = plume.make_plume(256, 1.2e-6, 9022)
        st2["t_inj"][:] = np.floor(np.arange(256) / 64) * 1e-12
        p4, v4, a4, t4 = plume.to_ref32(st2)
        p, v, a = run_ref("eps20", "dkd", p4, v4, a4, t4, threads=4, steps=10, dt=1e-12, **keys)
    np.savez_compressed(os.path.join(HERE, "emitter_field.npz"), node_rz=nodes, e_r=er, e_z=ez, triangles=tri,
                        neighbors=nbr, r0=np.float64(r0), e0=np.float64(e0), pos4=pos4, vel4=vel4, acc4=acc4,
                        tinj=tinj, e_out=e_at, dkd_pos4=p4, dkd_vel4=v4, dkd_acc4=a4, dkd_tinj=t4, dkd_pos4_out=p,
                        dkd_vel4_out=v, dkd_acc4_out=a, steps=np.int32(10), dt=np.float32(1e-12),
                        eps=np.float64(1e-20))
    print("emitter field:", len(er), "nodes", len(tri), "triangles;", int((e_at == 0).all(1).sum()),
          "points without field")


# substep requests: (dt, BoundaryConditionOptions, (|x|, |y|, |z|, r) limits, time limit)
SUBSTEP_CASES = {
    # the plume core (r < 10 nm) at dt/27, the rest at dt
    "core": [(1e-13, 1, (0.0, 0.0, 0.0, 1e-8), 0.0)],
    # two nested regions: r < 14 nm at dt/3, r < 8 nm and the first 2.9 ps after injection at dt/9
    # (the time limit off the grid of half-step times, where FP32 and FP64 clocks could order a tie apart)
    "nested": [(3.4e-13, 1, (0.0, 0.0, 0.0, 1.4e-8), 0.0), (1.2e-13, 3, (0.0, 0.0, 0.0, 8e-9), 2.9e-12)],
}


def substeps_arg(subs):
    return ";".join(f"{dt:.9g},{bc},{s[0]:.9g},{s[1]:.9g},{s[2]:.9g},{s[3]:.9g},{bt:.9g}" for dt, bc, s, bt in subs)


def substeps():
    """The reference's own LeapfrogDKDSubsteps::runSimulation (and
    LeapfrogDKD::runSimulation) on plumes injected in groups, with its
    snapshot file."""
    out = {}
    st = plume.make_plume(256, 1e-6, 9040)
    # injection times off the grid of half-step times (a tie there is broken
    # differently by FP32 and FP64 clocks)
    st["t_inj"][:] = np.floor(np.arange(256) / 64) * 2.03e-12
    st["status"][[11, 77]] = 2
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    out.update(pos4=pos4, vel4=vel4, acc4=acc4, tinj=tinj)
    p, v, a, snap = run_ref("eps20", "run", pos4, vel4, acc4, tinj, threads=4, steps=6, dt=1e-12)
    out.update(single_pos4_out=p, single_vel4_out=v, single_acc4_out=a, single_snapshot=snap)
    for name, subs in SUBSTEP_CASES.items():
        p, v, a, snap = run_ref("eps20", "run", pos4, vel4, acc4, tinj, threads=4, steps=6, dt=1e-12,
                                subs=substeps_arg(subs))
        out.update({f"{name}_pos4_out": p, f"{name}_vel4_out": v, f"{name}_acc4_out": a, f"{name}_snapshot": snap})
        print(name, "statuses", dict(zip(*np.unique(a[:, 3], return_counts=True))))
    np.savez_compressed(os.path.join(HERE, "substeps.npz"), steps=np.int32(6), dt=np.float32(1e-12),
                        eps=np.float64(1e-20), **out)


# energy bookkeeping runs: (init steps, steps per interval, interval, with the emitter field, leading inactive)
ENERGY_CASES = {
    "plain": (10, 10, 2, False, False),
    "field": (40, 20, 2, True, False),
    "window": (40, 20, 3, True, True),
}


def energy():
    """The reference's own LeapfrogDKD::runSimulation with toggleEnergy: the
    energy file's records (KE_inj, PE_inj, FE_inj, KE, PE, FE per interval)
    on a plume injected in groups, without and with the emitter field, and
    with inactive particles at the front of the array (the window's first
    particle moves past them; inactive ones behind it still count)."""
    nodes, er, ez, tri, nbr = emitter_mesh()
    r0, e0 = 1e-8, 1e9
    out = dict(node_rz=nodes, e_r=er, e_z=ez, triangles=tri, neighbors=nbr, r0=np.float64(r0), e0=np.float64(e0))
    st = plume.make_plume(256, 1.2e-6, 9050)
    st["t_inj"][:] = np.floor(np.arange(256) / 64) * 2.03e-12
    st["status"][[11, 77]] = 2
    with scratch_dir() as td:
        with open(os.path.join(td, "fields.csv"), "w") as f:
            for k in range(len(er)):
                f.write(f"{nodes[k, 0]:.17g},{nodes[k, 1]:.17g},{er[k]:.17g},{ez[k]:.17g}\n")
        with open(os.path.join(td, "triangles.csv"), "w") as f:
            for t, nb in zip(tri, nbr):
                f.write(",".join(str(int(v)) for v in (*t, *nb)) + "\n")
        keys = dict(fdir=td + "/", fnodes="fields.csv", ftris="triangles.csv", r0=r0, e0=e0)
        for name, (init, each, interval, fld, lead) in ENERGY_CASES.items():
            s = {k: v.copy() for k, v in st.items()}
            if lead:
                s["status"][:5] = 0
                s["status"][100] = -1
            pos4, vel4, acc4, tinj = plume.to_ref32(s)
            p, v, a, _, rec = run_ref("eps20", "run", pos4, vel4, acc4, tinj, threads=4, steps=6, dt=1e-12,
                                      interval=interval, energy=f"{init},{each}", **(keys if fld else {}))
            out.update({f"{name}_pos4": pos4, f"{name}_vel4": vel4, f"{name}_acc4": acc4, f"{name}_tinj": tinj,
                        f"{name}_pos4_out": p, f"{name}_vel4_out": v, f"{name}_acc4_out": a,
                        f"{name}_records": rec, f"{name}_setup": np.array([init, each, interval, fld], np.int32)})
            print(name, "records", rec.shape[0])
    np.savez_compressed(os.path.join(HERE, "energy.npz"), steps=np.int32(6), dt=np.float32(1e-12),
                        eps=np.float64(1e-20), **out)


if __name__ == "__main__":
    if sys.argv[1:] == ["outliers"]:
        outliers()
    elif sys.argv[1:] == ["drift_bc"]:
        drift_bc()
    elif sys.argv[1:] == ["emitter_field"]:
        emitter_field()
    elif sys.argv[1:] == ["substeps"]:
        substeps()
    elif sys.argv[1:] == ["energy"]:
        energy()
    elif sys.argv[1:] == ["sampled"]:
        sampled_configs()
    else:
        main()
