"""Python binding of the C ABI (include/solveit_gpu.h) via ctypes.

This is the host-side mirror of the reference's ForceCalculationMethod use:
a ForceMethod object owns one GPU context (one plume), uploads the particle
state, runs updateAcceleration-equivalent evaluations and leapfrog steps, and
reads results back.  It loads the in-tree libsolveit_gpu.so and raises if the
library or a GPU is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_build", "libsolveit_gpu.so")

DIRECT, BARNES_HUT, FMM = 0, 1, 2
SYM_NONE, SYM_ROTATIONAL, SYM_TRANSLATIONAL = 0, 1, 2
MIXED, FP64 = 0, 1
FMM_FMM, FMM_OUTLIERS, TREECODE, TREECODE_OUTLIERS = 0, 1, 2, 3
CRASH_NONE, CRASH_EXTRACTOR_GRID = 0, 1
SNAPSHOT_ORIGINAL, SNAPSHOT_NEW_ORIGINAL, SNAPSHOT_FULL = 0, 1, 16
BC_NONE, BC_SPACE, BC_TIME, BC_SPACE_AND_TIME = 0, 1, 2, 3

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "allocation failed", 4: "bad state",
          5: "capacity exceeded", 6: "device wait timed out", 7: "unsupported"}

# names exported by the library, one per declaration in include/solveit_gpu.h
ABI_SYMBOLS = (
    "sv_default_params", "sv_create", "sv_destroy", "sv_set_params", "sv_get_params", "sv_upload",
    "sv_upload_ref32", "sv_download", "sv_download_ref32", "sv_compute_accel", "sv_add_accel_ref32",
    "sv_leapfrog", "sv_energy", "sv_compare_accel", "sv_get_stats", "sv_sync", "sv_stream",
    "sv_launch_count", "sv_last_error", "sv_abi_version", "sv_adjoint_forward", "sv_adjoint_backward",
    "sv_direct_accel_noalloc", "sv_upload_batch", "sv_batch_tune", "sv_batch_get_info", "sv_batch_set_tuning",
    "sv_get_outliers", "sv_set_boundary", "sv_get_boundary", "sv_get_events", "sv_set_emitter_field",
    "sv_emitter_field_at", "sv_set_substeps", "sv_get_substep_levels", "sv_snapshot", "sv_set_energy",
    "sv_get_energy_records", "sv_fmm_tune",
)

# sv_energy_record: the energy file's record (J)
ENERGY_DTYPE = np.dtype([("ke_inj", "<f4"), ("pe_inj", "<f4"), ("fe_inj", "<f4"), ("ke", "<f4"), ("pe", "<f4"),
                         ("fe", "<f4")])


class Params(C.Structure):
    _fields_ = [
        ("softening2", C.c_double), ("k_const", C.c_double), ("e_over_amu", C.c_double),
        ("efield", C.c_double * 3), ("method", C.c_int32), ("precision", C.c_int32),
        ("symmetry", C.c_int32), ("theta", C.c_float), ("leaf_size", C.c_int32),
        ("fmm_order", C.c_int32), ("fmm_ws", C.c_int32), ("fmm_leaf_target", C.c_int32),
        ("sym_axes", C.c_int32 * 3), ("sym_levels", C.c_int32), ("domain_size", C.c_double * 3),
        ("device", C.c_int32), ("profile_phases", C.c_int32), ("fmm_type", C.c_int32),
        ("fmm_root_scale", C.c_float), ("fmm_direct_pairs", C.c_int32), ("fmm_m2l_tc", C.c_int32),
        ("fmm_tune_err", C.c_float), ("fmm_near", C.c_int32),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("pair_interactions", C.c_double), ("cell_interactions", C.c_double),
        ("flops_algorithmic", C.c_double), ("ms_total", C.c_double), ("ms_phase", C.c_double * 8),
        ("levels", C.c_int32), ("boxes", C.c_int32), ("m2l_tc", C.c_int32), ("reserved", C.c_int32 * 5),
    ]


class BatchInfo(C.Structure):
    _fields_ = [
        ("nplumes", C.c_int32), ("fmm_plumes", C.c_int32), ("slots", C.c_int64), ("fmm_slots", C.c_int64),
        ("leaf_level", C.c_int32), ("m2l_weight", C.c_int32), ("direct_chunk", C.c_int32),
        ("direct_items", C.c_int32), ("graph_kernels_step", C.c_int32), ("graph_kernels_accel", C.c_int32),
        ("tuned_ms", C.c_double), ("direct_pairs", C.c_double), ("fmm_m2l", C.c_double),
        ("fmm_pairs", C.c_double), ("regrows", C.c_int32), ("overflow_mask", C.c_int32),
        ("level_boxes", C.c_int32 * 22), ("level_cap", C.c_int32 * 22), ("level_max", C.c_int32 * 22),
        ("max_leaf", C.c_int32), ("m2l_tc", C.c_int32), ("fmm_order", C.c_int32),
        ("fmm_near", C.c_int32), ("reserved", C.c_int32 * 2),
    ]


class Boundary(C.Structure):
    _fields_ = [
        ("crash", C.c_int32), ("bc", C.c_int32), ("crash_z", C.c_double), ("crash_width", C.c_double),
        ("crash_r", C.c_double), ("bc_space", C.c_double * 4), ("bc_time", C.c_double), ("fold", C.c_int32),
        ("reserved", C.c_int32 * 7),
    ]


# the 40-byte events-file record (ChargedParticles::writeToEventsFile, particles.cpp:666-684)
EVENT_DTYPE = np.dtype([("time", "<f4"), ("x", "<f4"), ("y", "<f4"), ("z", "<f4"), ("vx", "<f4"), ("vy", "<f4"),
                        ("vz", "<f4"), ("index", "<i4"), ("species", "<u4"), ("status", "<i4")])


class Substep(C.Structure):
    _fields_ = [("dt", C.c_double), ("bc", C.c_int32), ("bc_space", C.c_double * 4), ("bc_time", C.c_double)]


class SolveitError(RuntimeError):
    pass


_lib = None
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")


def load(path: str = LIB_PATH):
    """Load the native library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise SolveitError(f"{path} not built: run __graft_entry__.build() or solveit-code_gb300/build_ext.py")
    L = C.CDLL(path)
    vp = C.c_void_p
    L.sv_default_params.argtypes = [C.POINTER(Params)]
    L.sv_create.argtypes = [C.POINTER(Params), C.POINTER(vp)]
    L.sv_destroy.argtypes = [vp]
    L.sv_destroy.restype = None
    L.sv_set_params.argtypes = [vp, C.POINTER(Params)]
    L.sv_get_params.argtypes = [vp, C.POINTER(Params)]
    L.sv_upload.argtypes = [vp, C.c_int64, vp, vp, vp, vp, vp, vp]
    L.sv_upload_ref32.argtypes = [vp, C.c_int64, vp, vp, vp, vp]
    L.sv_download.argtypes = [vp, vp, vp, vp]
    L.sv_update_state.argtypes = [vp, C.c_int64, vp, vp, vp]
    L.sv_download_ref32.argtypes = [vp, vp, vp]
    L.sv_compute_accel.argtypes = [vp, C.c_int64, C.c_int64, vp]
    L.sv_add_accel_ref32.argtypes = [vp, vp]
    L.sv_leapfrog.argtypes = [vp, C.c_int32, C.c_double, C.c_double]
    L.sv_energy.argtypes = [vp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    L.sv_compare_accel.argtypes = [vp, vp, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                   C.POINTER(C.c_int64)]
    L.sv_get_stats.argtypes = [vp, C.POINTER(Stats)]
    L.sv_sync.argtypes = [vp]
    L.sv_stream.argtypes = [vp]
    L.sv_stream.restype = vp
    L.sv_launch_count.argtypes = [vp]
    L.sv_launch_count.restype = C.c_uint64
    L.sv_last_error.argtypes = [vp]
    L.sv_last_error.restype = C.c_char_p
    L.sv_abi_version.restype = C.c_int32
    L.sv_adjoint_forward.argtypes = [vp, C.c_int32, C.c_double, C.c_double, C.c_int32]
    L.sv_adjoint_backward.argtypes = [vp, vp, vp, vp, vp, vp]
    L.sv_direct_accel_noalloc.argtypes = [C.c_int64, vp, vp, vp, vp, C.c_double, C.c_double, vp, vp]
    L.sv_upload_batch.argtypes = [vp, C.c_int32, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    L.sv_batch_tune.argtypes = [vp, C.c_char_p, C.POINTER(C.c_double)]
    L.sv_batch_get_info.argtypes = [vp, C.POINTER(BatchInfo)]
    L.sv_batch_set_tuning.argtypes = [vp, C.c_int32, C.c_int32]
    L.sv_get_outliers.argtypes = [vp, vp, C.POINTER(C.c_int64)]
    L.sv_set_boundary.argtypes = [vp, C.POINTER(Boundary)]
    L.sv_get_boundary.argtypes = [vp, C.POINTER(Boundary)]
    L.sv_get_events.argtypes = [vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    L.sv_set_emitter_field.argtypes = [vp, C.c_int32, vp, vp, vp, C.c_int32, vp, vp, C.c_double, C.c_double,
                                       C.c_double]
    L.sv_emitter_field_at.argtypes = [vp, C.c_int64, vp, vp]
    L.sv_set_substeps.argtypes = [vp, C.c_double, C.c_int32, vp]
    L.sv_snapshot.argtypes = [vp, C.c_int32, C.c_int64, C.c_int64, C.c_float, vp, C.c_int64, C.POINTER(C.c_int64)]
    L.sv_get_substep_levels.argtypes = [vp, vp]
    L.sv_set_energy.argtypes = [vp, C.c_int32, C.c_int32, C.c_int32, C.c_int32]
    L.sv_fmm_tune.argtypes = [vp, C.POINTER(C.c_double)]
    L.sv_get_energy_records.argtypes = [vp, vp, C.c_int64, C.POINTER(C.c_int64)]
    for name in ABI_SYMBOLS:
        if name not in ("sv_destroy", "sv_stream", "sv_launch_count", "sv_last_error", "sv_abi_version"):
            getattr(L, name).restype = C.c_int
    _lib = L
    return L


def default_params(**kw) -> Params:
    p = Params()
    load().sv_default_params(C.byref(p))
    for k, v in kw.items():
        if k in ("efield", "sym_axes", "domain_size"):
            arr = getattr(p, k)
            for i, x in enumerate(v):
                arr[i] = x
        else:
            setattr(p, k, v)
    return p


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class ForceMethod:
    """One GPU context: the plume state plus a configured force method."""

    def __init__(self, params: Params | None = None, **kw):
        self.L = load()
        self.params = params if params is not None else default_params(**kw)
        h = C.c_void_p()
        self._check(self.L.sv_create(C.byref(self.params), C.byref(h)), ctx=None)
        self.h = h
        self.n = 0

    def _check(self, rc, ctx="self"):
        if rc != 0:
            msg = "" if ctx is None else self.L.sv_last_error(self.h).decode()
            raise SolveitError(f"{STATUS.get(rc, rc)}: {msg}")

    def close(self):
        if getattr(self, "h", None):
            self.L.sv_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_params(self, **kw):
        for k, v in kw.items():
            if k in ("efield", "sym_axes", "domain_size"):
                arr = getattr(self.params, k)
                for i, x in enumerate(v):
                    arr[i] = x
            else:
                setattr(self.params, k, v)
        self._check(self.L.sv_set_params(self.h, C.byref(self.params)))

    # -- state ---------------------------------------------------------------
    def upload(self, state):
        x = np.ascontiguousarray(state["x"], np.float64)
        v = np.ascontiguousarray(state["v"], np.float64) if state.get("v") is not None else None
        q = np.ascontiguousarray(state["q"], np.float64)
        m = np.ascontiguousarray(state["m"], np.float64)
        st = np.ascontiguousarray(state["status"], np.int32)
        t = np.ascontiguousarray(state["t_inj"], np.float64) if state.get("t_inj") is not None else None
        self.n = x.shape[0]
        self._check(self.L.sv_upload(self.h, self.n, _p(x), _p(v), _p(q), _p(m), _p(st), _p(t)))

    def upload_ref32(self, pos4, vel4, acc4, t_inj=None):
        p = np.ascontiguousarray(pos4, np.float32)
        v = np.ascontiguousarray(vel4, np.float32)
        a = np.ascontiguousarray(acc4, np.float32)
        t = None if t_inj is None else np.ascontiguousarray(t_inj, np.float32)
        self.n = p.shape[0]
        self._check(self.L.sv_upload_ref32(self.h, self.n, _p(p), _p(v), _p(a), _p(t)))

    def upload_batch(self, states, methods, symmetries):
        """Load many plumes (a list of state dicts) into this context.

        methods[i]: DIRECT or FMM; symmetries[i]: SYM_NONE or SYM_ROTATIONAL.
        """
        x = np.ascontiguousarray(np.concatenate([s["x"] for s in states]), np.float64)
        v = np.ascontiguousarray(np.concatenate([s["v"] for s in states]), np.float64)
        q = np.ascontiguousarray(np.concatenate([s["q"] for s in states]), np.float64)
        m = np.ascontiguousarray(np.concatenate([s["m"] for s in states]), np.float64)
        st = np.ascontiguousarray(np.concatenate([s["status"] for s in states]), np.int32)
        t = np.ascontiguousarray(np.concatenate([s["t_inj"] for s in states]), np.float64)
        counts = np.array([s["x"].shape[0] for s in states], np.int64)
        meth = np.ascontiguousarray(methods, np.int32)
        sym = np.ascontiguousarray(symmetries, np.int32)
        self.n = int(counts.sum())
        self.counts = counts
        self._check(self.L.sv_upload_batch(self.h, len(states), _p(counts), _p(meth), _p(sym), _p(x), _p(v),
                                           _p(q), _p(m), _p(st), _p(t)))

    def tune(self, cache_path=None):
        """Autotune the uploaded batch; returns the tuned force-evaluation time in ms."""
        ms = C.c_double()
        path = None if cache_path is None else str(cache_path).encode()
        self._check(self.L.sv_batch_tune(self.h, path, C.byref(ms)))
        self._check(self.L.sv_get_params(self.h, C.byref(self.params)))  # an order the tuner chose
        return ms.value

    def set_tuning(self, m2l_weight, direct_chunk):
        self._check(self.L.sv_batch_set_tuning(self.h, m2l_weight, direct_chunk))

    def batch_info(self) -> BatchInfo:
        b = BatchInfo()
        self._check(self.L.sv_batch_get_info(self.h, C.byref(b)))
        return b

    def update_state(self, x, v=None, status=None):
        """sv_update_state: new positions (and velocities, statuses) for the uploaded plume."""
        x = np.ascontiguousarray(x, np.float64)
        v = None if v is None else np.ascontiguousarray(v, np.float64)
        st = None if status is None else np.ascontiguousarray(status, np.int32)
        self._check(self.L.sv_update_state(self.h, x.shape[0], _p(x), _p(v), _p(st)))

    def download(self):
        x = np.zeros((self.n, 3), np.float64)
        v = np.zeros((self.n, 3), np.float64)
        st = np.zeros(self.n, np.int32)
        self._check(self.L.sv_download(self.h, _p(x), _p(v), _p(st)))
        return x, v, st

    # -- force / integration ---------------------------------------------------
    def accel(self, first=0, last=-1, out=True):
        a = np.zeros((self.n, 3), np.float64) if out else None
        self._check(self.L.sv_compute_accel(self.h, first, last, _p(a)))
        return a

    def add_accel_ref32(self, acc4):
        self._check(self.L.sv_add_accel_ref32(self.h, _p(acc4)))
        return acc4

    def leapfrog(self, nsteps, dt, t0=0.0):
        self._check(self.L.sv_leapfrog(self.h, nsteps, dt, t0))

    def set_boundary(self, crash=CRASH_NONE, crash_z=0.0, crash_width=0.0, crash_r=0.0, bc=BC_NONE,
                     bc_space=(0.0, 0.0, 0.0, 0.0), bc_time=0.0, fold=0):
        b = Boundary()
        b.crash, b.crash_z, b.crash_width, b.crash_r = crash, crash_z, crash_width, crash_r
        b.bc, b.bc_time, b.fold = bc, bc_time, fold
        for k in range(4):
            b.bc_space[k] = bc_space[k]
        self._check(self.L.sv_set_boundary(self.h, C.byref(b)))

    def set_emitter_field(self, node_rz, e_r, e_z, triangles, neighbors, r0, e0, z_max=140.0):
        """Field map of a single emitter (None removes it)."""
        if node_rz is None:
            self._check(self.L.sv_set_emitter_field(self.h, 0, None, None, None, 0, None, None, 1.0, 0.0, 0.0))
            return
        nd = np.ascontiguousarray(node_rz, np.float64)
        er = np.ascontiguousarray(e_r, np.float64)
        ez = np.ascontiguousarray(e_z, np.float64)
        tr = np.ascontiguousarray(triangles, np.int32)
        nb = np.ascontiguousarray(neighbors, np.int32)
        self._check(self.L.sv_set_emitter_field(self.h, er.size, _p(nd), _p(er), _p(ez), tr.size // 3, _p(tr),
                                                _p(nb), r0, e0, z_max))

    def emitter_field_at(self, x3):
        x = np.ascontiguousarray(x3, np.float64)
        out = np.zeros_like(x)
        self._check(self.L.sv_emitter_field_at(self.h, x.shape[0], _p(x), _p(out)))
        return out

    def set_substeps(self, time_step, substeps):
        """substeps: list of (dt, bc, (bx, by, bz, br), bt); [] returns to the single-rate leapfrog."""
        arr = (Substep * max(len(substeps), 1))()
        for k, (dt, bc, space, bt) in enumerate(substeps):
            arr[k].dt, arr[k].bc, arr[k].bc_time = dt, bc, bt
            for j in range(4):
                arr[k].bc_space[j] = space[j]
        self._check(self.L.sv_set_substeps(self.h, time_step, len(substeps), C.cast(arr, C.c_void_p)))

    def substep_levels(self):
        out = np.zeros(self.n, np.int8)
        self._check(self.L.sv_get_substep_levels(self.h, _p(out)))
        return out

    def fmm_tune(self):
        """sv_fmm_tune: returns (root scale kept, its force-evaluation ms)."""
        ms = C.c_double()
        self._check(self.L.sv_fmm_tune(self.h, C.byref(ms)))
        self._check(self.L.sv_get_params(self.h, C.byref(self.params)))  # the kept scale
        return self.params.fmm_root_scale, ms.value

    def set_energy(self, init_steps, steps, interval, enable=True):
        """Integrator::toggleEnergy: records every `interval` steps of leapfrog()."""
        self._check(self.L.sv_set_energy(self.h, 1 if enable else 0, init_steps, steps, interval))

    def energy_records(self):
        """The energy records kept since the last call (structured array of ENERGY_DTYPE)."""
        cnt = C.c_int64()
        self._check(self.L.sv_get_energy_records(self.h, None, 0, C.byref(cnt)))
        out = np.zeros(cnt.value, ENERGY_DTYPE)
        self._check(self.L.sv_get_energy_records(self.h, out.ctypes.data, cnt.value, C.byref(cnt)))
        return out[:cnt.value]

    def snapshot(self, fmt=1, first=0, last=-1, current_time=0.0):
        """The snapshot-file bytes of the current state (fmt: SNAPSHOT_ORIGINAL / SNAPSHOT_NEW_ORIGINAL,
        with SNAPSHOT_FULL or-ed in for saveFullCurrentConditions)."""
        nb = C.c_int64()
        self._check(self.L.sv_snapshot(self.h, fmt, first, last, current_time, None, 0, C.byref(nb)))
        out = np.zeros(nb.value, np.uint8)
        self._check(self.L.sv_snapshot(self.h, fmt, first, last, current_time, out.ctypes.data, nb.value,
                                       C.byref(nb)))
        return out

    def events(self):
        """Events recorded since the last call (structured array of EVENT_DTYPE, file order)."""
        cnt = C.c_int64()
        rc = self.L.sv_get_events(self.h, None, 0, C.byref(cnt))
        if rc not in (0, 5):
            self._check(rc)
        out = np.zeros(cnt.value, EVENT_DTYPE)
        self._check(self.L.sv_get_events(self.h, out.ctypes.data if len(out) else None, len(out), C.byref(cnt)))
        return out

    def adjoint_forward(self, nsteps, dt, t0=0.0, checkpoint_every=10):
        self._check(self.L.sv_adjoint_forward(self.h, nsteps, dt, t0, checkpoint_every))

    def adjoint_backward(self, dl_dx, dl_dv):
        """dL/dx, dL/dv of the final state -> (dL/dx0, dL/dv0, dL/dE)."""
        gx = np.ascontiguousarray(dl_dx, np.float64)
        gv = np.ascontiguousarray(dl_dv, np.float64)
        ox = np.zeros((self.n, 3), np.float64)
        ov = np.zeros((self.n, 3), np.float64)
        oe = np.zeros(3, np.float64)
        self._check(self.L.sv_adjoint_backward(self.h, _p(gx), _p(gv), _p(ox), _p(ov), _p(oe)))
        return ox, ov, oe

    def outliers(self):
        """(flags, count) of the last outlier-variant FMM evaluation."""
        f = np.zeros(self.n, np.int32)
        cnt = C.c_int64()
        self._check(self.L.sv_get_outliers(self.h, _p(f), C.byref(cnt)))
        return f, cnt.value

    def energy(self):
        ke = C.c_double()
        pe = C.c_double()
        self._check(self.L.sv_energy(self.h, C.byref(ke), C.byref(pe)))
        return ke.value, pe.value

    def compare(self, ref):
        r = np.ascontiguousarray(ref, np.float64)
        l2 = C.c_double()
        mx = C.c_double()
        am = C.c_int64()
        self._check(self.L.sv_compare_accel(self.h, _p(r), C.byref(l2), C.byref(mx), C.byref(am)))
        return l2.value, mx.value, am.value

    def stats(self) -> Stats:
        s = Stats()
        self._check(self.L.sv_get_stats(self.h, C.byref(s)))
        return s

    def sync(self):
        self._check(self.L.sv_sync(self.h))

    @property
    def stream(self):
        return self.L.sv_stream(self.h)

    @property
    def launches(self):
        return int(self.L.sv_launch_count(self.h))
