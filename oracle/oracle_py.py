"""ctypes binding of the C oracle (oracle/sv_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker and by bench.py's CPU-baseline leg.  Never by the product path.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsv_oracle.so")

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")

_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "lib"])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        for name in ("orc_k_const", "orc_e_over_amu", "orc_coulomb_ke", "orc_elem_charge", "orc_amu"):
            getattr(L, name).restype = C.c_double
            getattr(L, name).argtypes = []
        L.orc_species_mass.restype = C.c_double
        L.orc_species_mass.argtypes = [C.c_int]
        L.orc_direct_ref32.argtypes = [_f32p, _f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_double, C.c_int]
        L.orc_direct_rot4_ref32.argtypes = L.orc_direct_ref32.argtypes
        L.orc_direct_trans_ref32.argtypes = [_f32p, _f32p, _f32p, C.c_int, C.c_int, C.c_int, C.c_int,
                                             C.c_double, C.c_int, _i32p, _f32p, C.c_int]
        L.orc_trans_images.restype = C.c_int
        L.orc_trans_images.argtypes = [C.c_int, _i32p, C.c_void_p, C.c_int, _i32p, C.c_int]
        L.orc_direct_f64.argtypes = [C.c_int64, _f64p, _f64p, _f64p, _i32p, C.c_void_p, C.c_int64,
                                     C.c_double, C.c_double, C.c_int, C.c_int, C.c_void_p, _f64p, C.c_int]
        L.orc_potential_f64.argtypes = [C.c_int64, _f64p, _f64p, _i32p, C.c_void_p, C.c_int64,
                                        C.c_double, _f64p, C.c_int]
        L.orc_leapfrog_ref32.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_float,
                                         C.c_double, _f32p, C.c_int, C.c_int, C.c_void_p, _f32p, C.c_int]
        L.orc_leapfrog_f64.argtypes = [C.c_int64, _f64p, _f64p, _f64p, _f64p, _i32p, _f64p, C.c_int,
                                       C.c_double, C.c_double, C.c_double, C.c_double, _f64p, C.c_int,
                                       C.c_int, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_leapfrog_ref32_bc.argtypes = L.orc_leapfrog_ref32.argtypes[:-1] + [
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_int]
        L.orc_leapfrog_f64_bc.argtypes = L.orc_leapfrog_f64.argtypes[:-2] + [
            C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int), C.c_int]
        L.orc_leapfrog_substeps_ref32.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_float,
                                                  C.c_double, _f32p, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                                  C.c_void_p, C.c_int]
        L.orc_leapfrog_ref32_energy.argtypes = [C.c_int, _f32p, _f32p, _f32p, _f32p, C.c_int, C.c_float,
                                                C.c_double, _f32p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.orc_emitter_field_ref32.argtypes = [C.c_void_p, C.c_int, _f32p, _f32p, C.POINTER(C.c_int)]
        L.orc_emitter_field_f64.argtypes = [C.c_void_p, C.c_int64, _f64p, _f64p]
        L.orc_energy_f64.argtypes = [C.c_int64, _f64p, _f64p, _f64p, _f64p, C.c_double,
                                     C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_int]
        L.orc_rel_l2.argtypes = [C.c_int64, _f64p, _f64p, C.c_void_p, C.POINTER(C.c_double),
                                 C.POINTER(C.c_double), C.POINTER(C.c_int64), C.POINTER(C.c_double)]
        L.orc_outliers.restype = C.c_int64
        L.orc_outliers.argtypes = [C.c_int64, _f64p, _i32p, _i32p]
        _lib = L
    return _lib


def k_const():
    return lib().orc_k_const()


def e_over_amu():
    return lib().orc_e_over_amu()


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def direct_ref32(pos4, vel4, acc4, eps, sym=0, images=None, domain_size=(2e-6, 2e-6, 0.0),
                 threads=0, i_range=None, j_range=None):
    """Reference-arithmetic direct sum on FP32 vec4 state; returns a new acc4."""
    n = pos4.shape[0]
    acc = np.ascontiguousarray(acc4, np.float32).copy()
    i0, i1 = i_range or (0, n)
    j0, j1 = j_range or (0, n)
    p = np.ascontiguousarray(pos4, np.float32)
    v = np.ascontiguousarray(vel4, np.float32)
    if sym == 0:
        lib().orc_direct_ref32(p, v, acc, i0, i1, j0, j1, eps, threads)
    elif sym == 1:
        lib().orc_direct_rot4_ref32(p, v, acc, i0, i1, j0, j1, eps, threads)
    else:
        img = np.ascontiguousarray(images, np.int32).reshape(-1)
        dom = np.asarray(domain_size, np.float32)
        lib().orc_direct_trans_ref32(p, v, acc, i0, i1, j0, j1, eps, img.size // 3, img, dom, threads)
    return acc


def trans_images(levels=2, axes=(1, 1, 0), lattice=None):
    """Expanded image list (k, 3) of the reference's periodic Grid."""
    box = 3 ** levels
    ax = np.asarray(axes, np.int32)
    cap = box ** 3 * 8 + 8
    out = np.zeros(3 * cap, np.int32)
    if lattice is not None:
        lat = np.ascontiguousarray(lattice, np.int32).reshape(-1)
        cnt = lib().orc_trans_images(box, ax, lat.ctypes.data_as(C.c_void_p), lat.size // 3, out, cap)
    else:
        cnt = lib().orc_trans_images(box, ax, None, 0, out, cap)
    return out[: 3 * cnt].reshape(cnt, 3).copy()


def direct_f64(state, eps2, sym=0, img_off=None, targets=None, threads=0, kconst=None):
    """FP64 direct-sum acceleration (ntargets, 3) in m/s^2."""
    x = np.ascontiguousarray(state["x"], np.float64).reshape(-1)
    n = x.size // 3
    q = np.ascontiguousarray(state["q"], np.float64)
    m = np.ascontiguousarray(state["m"], np.float64)
    st = np.ascontiguousarray(state["status"], np.int32)
    t = None if targets is None else np.ascontiguousarray(targets, np.int64)
    nt = n if t is None else t.size
    out = np.zeros(3 * nt, np.float64)
    io = None if img_off is None else np.ascontiguousarray(img_off, np.float64).reshape(-1)
    nimg = 0 if io is None else io.size // 3
    lib().orc_direct_f64(n, x, q, m, st, _ptr(t), nt, eps2, k_const() if kconst is None else kconst,
                         sym, nimg, _ptr(io), out, threads)
    return out.reshape(nt, 3)


def leapfrog_ref32(pos4, vel4, acc4, t_inj, nsteps, dt, eps, efield=(0.0, 0.0, 0.0), sym=0,
                   images=None, domain_size=(2e-6, 2e-6, 0.0), threads=0):
    p = np.ascontiguousarray(pos4, np.float32).copy()
    v = np.ascontiguousarray(vel4, np.float32).copy()
    a = np.ascontiguousarray(acc4, np.float32).copy()
    t = np.ascontiguousarray(t_inj, np.float32)
    e = np.asarray(efield, np.float32)
    img = None if images is None else np.ascontiguousarray(images, np.int32).reshape(-1)
    nimg = 0 if img is None else img.size // 3
    lib().orc_leapfrog_ref32(p.shape[0], p, v, a, t, nsteps, dt, eps, e, sym, nimg, _ptr(img),
                             np.asarray(domain_size, np.float32), threads)
    return p, v, a


def leapfrog_f64(state, nsteps, dt, eps2, efield=(0.0, 0.0, 0.0), t0=0.0, sym=0, img_off=None,
                 threads=0):
    """FP64 DKD; returns (x, v, a_last) as (n, 3) arrays."""
    x = np.ascontiguousarray(state["x"], np.float64).reshape(-1).copy()
    v = np.ascontiguousarray(state["v"], np.float64).reshape(-1).copy()
    n = x.size // 3
    st = np.ascontiguousarray(state["status"], np.int32).copy()
    a = np.zeros(3 * n, np.float64)
    io = None if img_off is None else np.ascontiguousarray(img_off, np.float64).reshape(-1)
    nimg = 0 if io is None else io.size // 3
    lib().orc_leapfrog_f64(n, x, v, np.ascontiguousarray(state["q"], np.float64),
                           np.ascontiguousarray(state["m"], np.float64), st,
                           np.ascontiguousarray(state["t_inj"], np.float64), nsteps, dt, t0, eps2,
                           k_const(), np.asarray(efield, np.float64), sym, nimg, _ptr(io), _ptr(a),
                           threads)
    return x.reshape(n, 3), v.reshape(n, 3), a.reshape(n, 3)


class Boundary(C.Structure):
    """orc_boundary: crash test, folding and boundary conditions of the drift."""
    _fields_ = [("crash", C.c_int), ("bc", C.c_int), ("fold", C.c_int), ("axes", C.c_int * 3),
                ("crash_z", C.c_double), ("crash_width", C.c_double), ("crash_r", C.c_double),
                ("bc_space", C.c_double * 4), ("bc_time", C.c_double), ("domain", C.c_double * 3)]


# the events-file record (ChargedParticles::writeToEventsFile, particles.cpp:666-684)
EVENT_DTYPE = np.dtype([("time", "<f4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("vx", "<f4"), ("vy", "<f4"),
                        ("vz", "<f4"), ("index", "<i4"), ("species", "<u4"), ("status", "<i4")])


def boundary(crash=0, crash_z=0.0, crash_width=0.0, crash_r=0.0, bc=0, bc_space=(0, 0, 0, 0), bc_time=0.0,
             fold=0, axes=(0, 0, 0), domain=(0.0, 0.0, 0.0)):
    b = Boundary()
    b.crash, b.bc, b.fold = crash, bc, fold
    b.crash_z, b.crash_width, b.crash_r, b.bc_time = crash_z, crash_width, crash_r, bc_time
    for k in range(3):
        b.axes[k] = axes[k]
        b.domain[k] = domain[k]
    for k in range(4):
        b.bc_space[k] = bc_space[k]
    return b


class Field(C.Structure):
    """orc_field: a single emitter's field map (keeps its arrays alive)."""
    _fields_ = [("n_nodes", C.c_int), ("n_tri", C.c_int), ("node_rz", C.c_void_p), ("er", C.c_void_p),
                ("ez", C.c_void_p), ("tri", C.c_void_p), ("nbr", C.c_void_p), ("r0", C.c_double),
                ("e0", C.c_double), ("zmax", C.c_double)]


def field(node_rz, e_r, e_z, triangles, neighbors, r0, e0, zmax=140.0):
    f = Field()
    f._keep = [np.ascontiguousarray(node_rz, np.float64), np.ascontiguousarray(e_r, np.float64),
               np.ascontiguousarray(e_z, np.float64), np.ascontiguousarray(triangles, np.int32),
               np.ascontiguousarray(neighbors, np.int32)]
    f.n_nodes, f.n_tri = f._keep[1].size, f._keep[3].size // 3
    f.node_rz, f.er, f.ez, f.tri, f.nbr = (a.ctypes.data for a in f._keep)
    f.r0, f.e0, f.zmax = r0, e0, zmax
    return f


def emitter_field_ref32(fld, pos4):
    """InterpolationScheme::Efield at each particle in index order (FP32)."""
    p = np.ascontiguousarray(pos4, np.float32)
    out = np.zeros(3 * p.shape[0], np.float32)
    save = C.c_int(-1)
    lib().orc_emitter_field_ref32(C.byref(fld), p.shape[0], p.reshape(-1), out, C.byref(save))
    return out.reshape(-1, 3)


def emitter_field_f64(fld, x3):
    x = np.ascontiguousarray(x3, np.float64)
    out = np.zeros(x.size, np.float64)
    lib().orc_emitter_field_f64(C.byref(fld), x.shape[0], x.reshape(-1), out)
    return out.reshape(-1, 3)


def leapfrog_ref32_bc(pos4, vel4, acc4, t_inj, nsteps, dt, eps, efield=(0.0, 0.0, 0.0), sym=0, bd=None,
                      images=None, domain_size=(2e-6, 2e-6, 0.0), threads=0, ev_cap=1 << 16, fld=None):
    """The reference's loop with its injection window, crash test, folding and
    boundary conditions: (pos4, vel4, acc4, events)."""
    p = np.ascontiguousarray(pos4, np.float32).copy()
    v = np.ascontiguousarray(vel4, np.float32).copy()
    a = np.ascontiguousarray(acc4, np.float32).copy()
    t = np.ascontiguousarray(t_inj, np.float32)
    e = np.asarray(efield, np.float32)
    img = None if images is None else np.ascontiguousarray(images, np.int32).reshape(-1)
    nimg = 0 if img is None else img.size // 3
    ev = np.zeros(ev_cap, EVENT_DTYPE)
    cnt = C.c_int()
    lib().orc_leapfrog_ref32_bc(p.shape[0], p, v, a, t, nsteps, dt, eps, e, sym, nimg, _ptr(img),
                                np.asarray(domain_size, np.float32), None if bd is None else C.byref(bd),
                                None if fld is None else C.byref(fld), ev.ctypes.data, ev_cap, C.byref(cnt),
                                threads)
    return p, v, a, ev[:min(cnt.value, ev_cap)].copy()


def leapfrog_f64_bc(state, nsteps, dt, eps2, efield=(0.0, 0.0, 0.0), t0=0.0, sym=0, img_off=None, bd=None,
                    threads=0, ev_cap=1 << 16, fld=None):
    """FP64 DKD with the window, crash, folding and boundary conditions:
    (x, v, status, events)."""
    x = np.ascontiguousarray(state["x"], np.float64).reshape(-1).copy()
    v = np.ascontiguousarray(state["v"], np.float64).reshape(-1).copy()
    n = x.size // 3
    st = np.ascontiguousarray(state["status"], np.int32).copy()
    io = None if img_off is None else np.ascontiguousarray(img_off, np.float64).reshape(-1)
    nimg = 0 if io is None else io.size // 3
    ev = np.zeros(ev_cap, EVENT_DTYPE)
    cnt = C.c_int()
    lib().orc_leapfrog_f64_bc(n, x, v, np.ascontiguousarray(state["q"], np.float64),
                              np.ascontiguousarray(state["m"], np.float64), st,
                              np.ascontiguousarray(state["t_inj"], np.float64), nsteps, dt, t0, eps2,
                              k_const(), np.asarray(efield, np.float64), sym, nimg, _ptr(io),
                              None if bd is None else C.byref(bd), None if fld is None else C.byref(fld),
                              ev.ctypes.data, ev_cap, C.byref(cnt), threads)
    return x.reshape(n, 3), v.reshape(n, 3), st, ev[:min(cnt.value, ev_cap)].copy()


class Energy(C.Structure):
    """orc_energy: the energy bookkeeping's settings and its records."""
    _fields_ = [("init_steps", C.c_int), ("steps", C.c_int), ("interval", C.c_int), ("rec", C.c_void_p),
                ("rec_cap", C.c_int), ("rec_count", C.c_int)]


def leapfrog_ref32_energy(pos4, vel4, acc4, t_inj, nsteps, dt, eps, init_steps, steps, interval,
                          efield=(0.0, 0.0, 0.0), bd=None, fld=None, threads=0):
    """The reference's loop with toggleEnergy(1, init_steps, steps): (pos4,
    vel4, acc4, records), records (k, 6) float32 = KE_inj, PE_inj, FE_inj, KE,
    PE, FE per interval, as the energy file holds them."""
    p = np.ascontiguousarray(pos4, np.float32).copy()
    v = np.ascontiguousarray(vel4, np.float32).copy()
    a = np.ascontiguousarray(acc4, np.float32).copy()
    t = np.ascontiguousarray(t_inj, np.float32)
    cap = nsteps // max(interval, 1) + 1
    rec = np.zeros((cap, 6), np.float32)
    en = Energy(init_steps, steps, interval, rec.ctypes.data, cap, 0)
    lib().orc_leapfrog_ref32_energy(p.shape[0], p, v, a, t, nsteps, dt, eps, np.asarray(efield, np.float32),
                                    None if bd is None else C.byref(bd), None if fld is None else C.byref(fld),
                                    C.byref(en), threads)
    return p, v, a, rec[:min(en.rec_count, cap)].copy()


class Substep(C.Structure):
    """orc_substep: one setSubstepTimes request."""
    _fields_ = [("dt", C.c_float), ("bc", C.c_int), ("s", C.c_float * 4), ("t", C.c_float)]


def leapfrog_substeps_ref32(pos4, vel4, acc4, t_inj, nsteps, dt, eps, subs, efield=(0.0, 0.0, 0.0), sym=0,
                            bd=None, threads=0):
    """LeapfrogDKDSubsteps restated (FP32): subs = [(dt, bc, (bx, by, bz, br), bt), ...];
    returns (pos4, vel4, acc4, levels)."""
    p = np.ascontiguousarray(pos4, np.float32).copy()
    v = np.ascontiguousarray(vel4, np.float32).copy()
    a = np.ascontiguousarray(acc4, np.float32).copy()
    t = np.ascontiguousarray(t_inj, np.float32)
    arr = (Substep * len(subs))()
    for k, (sdt, bc, space, bt) in enumerate(subs):
        arr[k].dt, arr[k].bc, arr[k].t = sdt, bc, bt
        for j in range(4):
            arr[k].s[j] = space[j]
    lev = np.zeros(p.shape[0], np.int8)
    lib().orc_leapfrog_substeps_ref32(p.shape[0], p, v, a, t, nsteps, dt, eps, np.asarray(efield, np.float32), sym,
                                      len(subs), C.cast(arr, C.c_void_p), None if bd is None else C.byref(bd),
                                      lev.ctypes.data, threads)
    return p, v, a, lev


def energy_f64(state, eps2, threads=0):
    ke = C.c_double()
    pe = C.c_double()
    lib().orc_energy_f64(state["x"].shape[0], np.ascontiguousarray(state["x"], np.float64).reshape(-1),
                         np.ascontiguousarray(state["v"], np.float64).reshape(-1),
                         np.ascontiguousarray(state["q"], np.float64),
                         np.ascontiguousarray(state["m"], np.float64), eps2, C.byref(ke), C.byref(pe),
                         threads)
    return ke.value, pe.value


def outliers(state):
    """isOutlier restated: (flags, count), flags 1 / 0 / -1 as outlierCheck."""
    x = np.ascontiguousarray(state["x"], np.float64).reshape(-1)
    st = np.ascontiguousarray(state["status"], np.int32)
    f = np.zeros(st.size, np.int32)
    cnt = lib().orc_outliers(st.size, x, st, f)
    return f, int(cnt)


def rel_l2(a, ref, status=None):
    """Reference accuracy metric: (per-particle rel-L2, max, argmax, global rel-L2)."""
    a = np.ascontiguousarray(a, np.float64).reshape(-1)
    r = np.ascontiguousarray(ref, np.float64).reshape(-1)
    st = None if status is None else np.ascontiguousarray(status, np.int32)
    l2 = C.c_double()
    mx = C.c_double()
    am = C.c_int64()
    g = C.c_double()
    lib().orc_rel_l2(a.size // 3, a, r, _ptr(st), C.byref(l2), C.byref(mx), C.byref(am), C.byref(g))
    return l2.value, mx.value, am.value, g.value
