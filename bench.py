"""Benchmark: particle-steps/s of the GB300 force-evaluation + leapfrog path.

Default workload (fmm_n1m): one plume of N = 1,048,576 singly charged ions
(r <= 20 nm, z in [0, 50] um, softening 1e-10 m), leapfrog DKD steps of
dt = 1e-13 s with E_z = 1e8 V/m, forces by the FMM (p = 8, ws = 2) in mixed
precision (FP32 pair / expansion arithmetic, FP64 positions, velocities,
accumulation and integration).  A step = drift dt/2 + force evaluation + kick
+ drift dt/2 over the whole plume.

  value          particle-steps/s with the plume resident in HBM (CUDA events
                 on the context stream around each step; L2 flushed between
                 steps by writing 512 MB)
  e2e            same metric over the same steps from the same state, through
                 the C ABI with host buffers: per step, upload of the current
                 state from pinned host memory, one step, and download of
                 positions / velocities / status (the next step's upload)
  fp64_direct    the plain FP64 GPU direct-sum path on the same GPU (measured
                 at N = 131072, scaled by N^2 to the workload's N)
  force_err      per-particle relative L2 of the FMM acceleration against the
                 FP64 GPU direct sum on 512 sampled targets
  cpu_baseline   the C oracle's FP64 direct sum (the reference's direct sum
                 restated; the reference's own FMM crashes at this N) on a
                 bounded sample of targets, all host threads

--impl reference times that CPU path alone (the reference arm).
Under torchrun with N > 1 GPUs every rank runs an independent plume
(replicas only: the workload has no exchange step).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "solveit-code_gb300"))

import plume  # noqa: E402

METRIC = "particle-steps/s, mixed-prec vs plain FP64 path, same GB300, force err <=1e-5"
# DRAM bytes (read + write) of one near-field launch of the fmm_n1m workload,
# from one ncu capture, with the root scale and leaf level it was taken at:
# the roofline reports it only for a run at that same configuration
P2P_TRAFFIC = {"bytes": 30337280 + 143360, "root_scale": 1.375, "leaf_level": 12}
EPS2 = 1e-20
DT = 1e-13
EZ = 1e8

WORKLOADS = {
    "fmm_n1m": dict(n=1 << 20, length=50e-6, method="fmm", order=8, ws=2, leaf=32, seed=2000,
                    desc="FMM p=8 ws=2, N=1048576 ions, plume r=20nm z=50um, eps=1e-10m, "
                         "leapfrog DKD dt=1e-13s, E_z=1e8V/m"),
    "bh_n65536": dict(n=65536, length=10e-6, method="bh", theta=0.5, leaf=16, seed=1,
                      desc="Barnes-Hut theta=0.5 leaf 16 (stackless warp walk, FP32 forces, FP64 integration), "
                           "N=65536 ions, plume r=20nm z=10um, eps=1e-10m, leapfrog DKD dt=1e-13s, E_z=1e8V/m"),
    "direct_n4096": dict(n=4096, length=1e-6, method="direct", precision="fp64", seed=0,
                         desc="FP64 direct sum, N=4096 ions, plume r=20nm z=1um, eps=1e-10m, "
                              "leapfrog DKD dt=1e-13s, E_z=1e8V/m"),
    "adjoint_n16384": dict(n=16384, length=1e-6, method="adjoint", nsteps=50, every=10, seed=4,
                           desc="adjoint of 50 leapfrog DKD steps (direct sum, mixed precision), N=16384 ions, "
                                "plume r=20nm z=1um, eps=1e-10m, dt=1e-13s, E_z=1e8V/m, checkpoint every 10 steps; "
                                "loss = mean z-momentum + 1e3 x mean transverse radius"),
    "batch256": dict(n=None, nplumes=256, length=1e-6, method="batch", order=6, ws=2, near=2, seed=3,
                     desc="256 independent plumes, N_i uniform in [1024, 65536] (seed 3999), r=20nm z=1um, "
                          "direct sum for N_i < 8192 and FMM p=6 ws=2 (trimmed near field) above, "
                          "4-fold rotational variant on the "
                          "even plumes, eps=1e-10m, leapfrog DKD dt=1e-13s, E_z=1e8V/m, each step one CUDA "
                          "graph"),
}


def plume_seed(wl, rank):
    """Replicas: every rank integrates its own realisation of the workload."""
    return wl["seed"] * 1000 + rank


def max_over_ranks(value, dist, device):
    """Slowest rank's time: the whole job is done when the last replica is."""
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def sample_clocks_start():
    try:
        import tempfile

        path = os.path.join(tempfile.gettempdir(), f"sv_clocks_{os.getpid()}.csv")
        f = open(path, "w")
        p = subprocess.Popen(
            ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
             "--format=csv,noheader,nounits", "-lms", "200"], stdout=f, stderr=subprocess.DEVNULL)
        return p, f
    except Exception:
        return None, None


def sample_clocks_stop(p, f, gpu_index):
    if p is None:
        return None
    p.terminate()
    try:
        p.wait(timeout=5)
    except Exception:
        p.kill()
    f.close()
    path = f.name
    sm, smax, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    try:
        for line in open(path):
            cols = [c.strip() for c in line.split(",")]
            if len(cols) < 9 or cols[0] != str(gpu_index):
                continue
            try:
                sm.append(float(cols[1]))
                smax = max(smax, float(cols[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if cols[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        os.remove(path)
    except Exception:
        pass
    if not sm:
        return None
    loaded = sorted(sm)[len(sm) // 2:]  # upper half: samples under load
    return {"sm_mhz": float(np.median(loaded)), "sm_max_mhz": smax, "reasons": sorted(reasons),
            "samples": len(sm)}


def fp32_peak_tflops(local, sm_max_mhz):
    """FP32 FMA rate of this device: SMs (queried) x 128 lanes x 2 flop x the
    measured maximum SM clock."""
    import torch

    sms = torch.cuda.get_device_properties(local).multi_processor_count
    return sms * 128 * 2 * sm_max_mhz * 1e6 / 1e12, sms


def fp64_sampled_accel(sv, local, cur, targets, sym=0):
    """The plain FP64 GPU direct sum at the sampled targets of a plume (the
    other particles act as sources only)."""
    s2 = np.where(cur["status"] == 1, 2, cur["status"]).astype(np.int32)
    s2[targets] = cur["status"][targets]
    with sv.ForceMethod(softening2=EPS2, method=sv.DIRECT, precision=sv.FP64, device=local, symmetry=sym) as ref:
        ref.upload(dict(cur, status=s2))
        return ref.accel()[targets]


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {}


def cpu_baseline(state, n_sample, threads):
    """The reference's direct sum, restated in C (bit-exact with the reference
    on its FP32 vec4 state), on n_sample targets against all sources, all host
    threads; particle-steps/s."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py as O

    n = state["x"].shape[0]
    pos4, vel4, acc4, _ = plume.to_ref32(state)
    O.direct_ref32(pos4, vel4, acc4, EPS2, i_range=(0, 64), threads=threads)  # warm
    t = time.perf_counter()
    O.direct_ref32(pos4, vel4, acc4, EPS2, i_range=(0, n_sample), threads=threads)
    dt = time.perf_counter() - t
    return {"value": n_sample / dt, "unit": "particle-steps/s", "cores": threads, "kind": "port",
            "sample": f"reference direct sum (DirectForceFunction::direct, direct_force_method.cpp:153-190, "
                      f"restated in C and bit-exact with the reference) for targets 0..{n_sample - 1} of {n} "
                      f"against all {n} sources, one force evaluation ({dt:.2f} s, {threads} threads); the "
                      f"per-target cost does not depend on the target count, so particle-steps/s = "
                      f"targets / time.  The reference's own FMM is not timed: it overflows its heap "
                      f"buffers at this plume size"}


def run_reference(args, wl, rank, world):
    if rank != 0:
        return
    if wl["method"] == "batch":
        return run_reference_batch(args, wl, world)
    if wl["method"] == "adjoint":
        print(json.dumps({"impl": "reference", "unavailable": "the reference has no adjoint: its integrator "
                          "runs forward only"}), flush=True)
        return
    st = plume.make_plume(wl["n"], wl["length"], wl["seed"] * 1000 + 0)
    threads = os.cpu_count() or 1
    n_sample = 2048 if wl["n"] > 100000 else min(wl["n"], 4096)
    vals = []
    cb = None
    for k in range(args.warmup + args.steps):
        cb = cpu_baseline(st, n_sample, threads)
        if k >= args.warmup:
            vals.append(cb["value"])
    v = float(np.mean(vals))
    cb["value"] = v
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": wl["n"] / v * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": args.workload, "desc": wl["desc"], "n": wl["n"]},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0},
            "extrapolated_from": {"targets_timed": n_sample, "targets_total": wl["n"],
                                  "fraction": n_sample / wl["n"],
                                  "how": "one force evaluation of the timed targets against all sources per "
                                         "step; particle-steps/s = targets / time (the per-target cost does not "
                                         "depend on how many targets are timed)"},
            "comparison": "CPU O(N^2) direct sum (the reference's direct method; its FMM overflows its buffers "
                          "at this plume size): a ratio against the GPU FMM is algorithmic as well as hardware"}
    print(json.dumps(line), flush=True)


def run_batch(args, wl, rank, world, local):
    """The batched-plume workload: every step of all plumes is one graph launch."""
    import ctypes as C

    import torch

    import solveit_gpu as sv

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    states, methods, syms = plume.make_batch(wl["nplumes"], config=wl["seed"] + 100 * rank, length=wl["length"])
    counts = np.array([s["x"].shape[0] for s in states])
    n = int(counts.sum())
    fm = sv.ForceMethod(softening2=EPS2, efield=(0.0, 0.0, EZ), device=local, fmm_order=wl["order"],
                        fmm_ws=wl["ws"], fmm_m2l_tc=args.m2l_tc, fmm_near=args.fmm_near or wl.get("near", 0))
    fm.upload_batch(states, methods, syms)
    tuned_ms = None if args.no_tune else fm.tune(None)
    stream = torch.cuda.ExternalStream(fm.stream, device=local)
    t = 0.0
    fm.leapfrog(args.warmup, DT, t)
    t += args.warmup * DT
    fm.sync()
    t_start = t
    snap = fm.download()  # the state at the start of the timed window (the e2e run repeats the window)
    clk_p, clk_f = sample_clocks_start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = fm.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fm.leapfrog(args.steps, DT, t)  # args.steps graph launches, one capacity check at the end
    e1.record(stream)
    torch.cuda.synchronize()
    launches = fm.launches - launches0
    clocks = sample_clocks_stop(clk_p, clk_f, local)
    step_ms = e0.elapsed_time(e1)
    if dist:
        step_ms = max_over_ranks(step_ms, dist, f"cuda:{local}")
    ms_per_step = step_ms / args.steps
    value = world * n * args.steps / (step_ms / 1e3)
    info = fm.batch_info()
    if args.timed_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "ms_per_step": ms_per_step, "timed_only": True,
                              "m2l_weight": info.m2l_weight, "leaf_level": info.leaf_level,
                              "regrows": info.regrows, "m2l_tc": info.m2l_tc}), flush=True)
        fm.close()
        return

    # ---- end to end: the same steps again from the same state, through the C
    # ABI with host buffers: each step uploads the current batch state from
    # pinned host memory (same shape: the plan and graphs are kept), runs one
    # step and downloads positions, velocities and status into the buffers the
    # next step uploads
    cat, _ = plume.concat(states)
    pin = {k: torch.empty(cat[k].shape, dtype=torch.float64 if cat[k].dtype == np.float64 else torch.int32,
                          pin_memory=True) for k in ("x", "v", "q", "m", "status", "t_inj")}
    cnt = np.ascontiguousarray(counts, np.int64)
    meth = np.ascontiguousarray(methods, np.int32)
    sym = np.ascontiguousarray(syms, np.int32)
    L = sv.load()

    def ptr(tn):
        return C.c_void_p(tn.data_ptr())

    def reset_pins():
        for k in ("q", "m", "t_inj"):
            pin[k].numpy()[...] = cat[k]
        pin["x"].numpy()[...] = snap[0]
        pin["v"].numpy()[...] = snap[1]
        pin["status"].numpy()[...] = snap[2]

    def e2e_step(t0):
        for rc in (L.sv_upload_batch(fm.h, len(states), cnt.ctypes.data_as(C.c_void_p),
                                     meth.ctypes.data_as(C.c_void_p), sym.ctypes.data_as(C.c_void_p),
                                     ptr(pin["x"]), ptr(pin["v"]), ptr(pin["q"]), ptr(pin["m"]),
                                     ptr(pin["status"]), ptr(pin["t_inj"])),
                   L.sv_leapfrog(fm.h, 1, DT, t0),
                   L.sv_download(fm.h, ptr(pin["x"]), ptr(pin["v"]), ptr(pin["status"]))):
            if rc != 0:
                raise RuntimeError(L.sv_last_error(fm.h).decode())

    reset_pins()
    e2e_step(t_start)  # warm-up of the host path, then back to the window's first state
    reset_pins()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(t_start + k * DT)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - w0
    if dist:
        e2e_s = max_over_ranks(e2e_s, dist, f"cuda:{local}")
    e2e = {"value": world * n * args.steps / e2e_s, "unit": "particle-steps/s",
           "h2d_bytes_per_step": n * (3 * 8 + 3 * 8 + 8 + 8 + 4 + 8), "d2h_bytes_per_step": n * (3 * 8 + 3 * 8 + 4),
           "steps": args.steps, "window": "the timed steps of value, from the same state"}
    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 pair/expansion arithmetic, f64 state and integration",
            "data": "synthetic (seeded plume generator)",
            "config": {"workload": args.workload, "desc": wl["desc"], "particles_per_gpu": n,
                       "plumes": len(states), "fmm_plumes": info.fmm_plumes, "slots_with_images": info.slots,
                       "leaf_level": info.leaf_level, "tuned_m2l_weight": info.m2l_weight,
                       "tuned_direct_chunk": info.direct_chunk, "kernels_per_step_graph": info.graph_kernels_step,
                       "capacity_regrows": info.regrows, "m2l_on_tensor_cores": bool(info.m2l_tc),
                       "fmm_near_field": "trimmed" if fm.params.fmm_near == 2 else "full 5^3 cube",
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "no flush: the batch state (particles x 48 B plus sorted copies) is far larger than "
                             "L2"},
            "clocks": clocks, "e2e": e2e, "gpu_launches": int(launches), "tuned_force_ms": tuned_ms}
    if rank == 0:
        sm_max = measured_peaks().get("sm_max_mhz", 2070.0)
        fp32_peak, sms = fp32_peak_tflops(local, sm_max)
        p = wl["order"]
        m2l_flop = 8.0 * (2 * sum((k + 1) * (2 * k + 1) for k in range(p)) +
                          sum(p - k for j in range(p) for k in range(j + 1)))
        flops = 20.0 * (info.direct_pairs + info.fmm_pairs) + info.fmm_m2l * m2l_flop + \
            info.fmm_slots * 8.0 * (p * (p + 1) / 2) * 4
        achieved = flops / (ms_per_step * 1e-3) / 1e12
        line["roofline"] = {"kernel": "whole step (direct pairs + P2P pairs at 20 flop, M2L at its flop count, "
                                      "P2M + L2P)", "bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                            "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": None,
                            "pairs_per_step": info.direct_pairs + info.fmm_pairs, "m2l_per_step": info.fmm_m2l,
                            "peak_source": f"FP32 FMA rate: {sms} SMs x 128 lanes x 2 flop x sm_max_mhz "
                                           f"{sm_max:.0f} of MEASURED_PEAKS.json"}
        # force error on sampled targets of a few plumes against the plain FP64 GPU direct sum
        x, v, stt = fm.download()
        a = fm.accel()
        offs = np.concatenate([[0], np.cumsum(counts)])
        rng = np.random.default_rng(11)
        errs = {}
        for i in (0, 1, 2, 3, int(np.argmax(counts)), int(np.argmin(counts))):
            s0, s1 = offs[i], offs[i + 1]
            cur = dict(states[i], x=x[s0:s1], v=v[s0:s1], status=stt[s0:s1])
            tg = np.sort(rng.choice(s1 - s0, min(64, s1 - s0), replace=False))
            ref = fp64_sampled_accel(sv, local, cur, tg, sym=int(syms[i]))
            d = np.sum((a[s0:s1][tg] - ref) ** 2, axis=1) / np.sum(ref ** 2, axis=1)
            errs[f"plume{i}_n{s1 - s0}_{'fmm' if methods[i] == 2 else 'direct'}_{'rot4' if syms[i] else 'none'}"] = \
                float(np.sqrt(np.mean(d)))
        line["force_err_rel_l2_sampled"] = errs
        # plain FP64 GPU direct path: measured pair rate at one plume, applied to every plume's pair count
        big = int(np.argmax(counts))
        with sv.ForceMethod(softening2=EPS2, method=sv.DIRECT, precision=sv.FP64, device=local) as f64:
            f64.upload(states[big])
            f64.accel(out=False)
            f64.sync()
            t0 = time.perf_counter()
            f64.accel(out=False)
            f64.sync()
            t_big = time.perf_counter() - t0
        rate = counts[big] ** 2 / t_big
        pairs_all = float(sum(int(nn) ** 2 * (4 if sy else 1) for nn, sy in zip(counts, syms)))
        t_all = pairs_all / rate
        line["fp64_direct"] = {"value": n / t_all, "unit": "particle-steps/s",
                               "measured": f"FP64 direct force at N={counts[big]}: {t_big * 1e3:.1f} ms "
                                           f"({rate:.3g} pairs/s), applied to the batch's {pairs_all:.3g} "
                                           f"pairs per step (x4 for the rotational plumes)",
                               "extrapolated_from": {"plume_measured": big, "n_measured": int(counts[big]),
                                                     "pairs_measured": float(counts[big]) ** 2,
                                                     "pairs_applied": pairs_all}}
        line["speedup_vs_fp64_direct"] = value / world / (n / t_all)
        # CPU baseline: the oracle's bit-exact restatement of the reference direct sum on a target sample,
        # as a pair rate applied to the whole batch
        threads = os.cpu_count() or 1
        ns = 2048
        cb = cpu_baseline(states[big], ns, threads)
        tc = ns / cb["value"]
        cpu_rate = ns * counts[big] / tc
        line["cpu_baseline"] = {"value": n / (pairs_all / cpu_rate), "unit": "particle-steps/s", "cores": threads,
                                "kind": "port",
                                "sample": f"reference direct sum restated in C (bit-exact with "
                                          f"direct_force_method.cpp:153-190), {ns} targets of plume {big} "
                                          f"(N={counts[big]}) in {tc:.2f} s = {cpu_rate:.3g} pairs/s, applied to "
                                          f"the batch's direct-sum pair count; the reference's FMM is not timed "
                                          f"(its rotational FMM is wrong at these sizes)"}
        print(json.dumps(line), flush=True)
    fm.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_reference_batch(args, wl, world):
    """Reference arm of the batched workload: the reference's direct sum
    (restated in C, bit-exact) as a pair rate, applied to every plume."""
    states, methods, syms = plume.make_batch(wl["nplumes"], config=wl["seed"], length=wl["length"])
    counts = np.array([s["x"].shape[0] for s in states])
    n = int(counts.sum())
    big = int(np.argmax(counts))
    pairs_all = float(sum(int(nn) ** 2 * (4 if sy else 1) for nn, sy in zip(counts, syms)))
    threads = os.cpu_count() or 1
    vals = []
    cb = None
    for k in range(args.warmup + args.steps):
        cb = cpu_baseline(states[big], 2048, threads)
        if k >= args.warmup:
            vals.append(cb["value"] * counts[big] / pairs_all * n)
    v = float(np.mean(vals))
    cb["value"] = v
    cb["sample"] += f"; applied to the batch's {pairs_all:.3g} direct-sum pairs per step"
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "particle-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": n / v * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "desc": wl["desc"], "particles": n},
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                                        "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_adjoint(args, wl, rank, world, local):
    """Gradient throughput: one forward rollout with checkpoints plus the
    backward sweep per step of the metric (particle-steps of the rollout per
    second of forward + backward time)."""
    import torch

    import solveit_gpu as sv

    torch.cuda.set_device(local)
    n, nsteps, every = wl["n"], wl["nsteps"], wl["every"]
    st = plume.make_plume(n, wl["length"], plume_seed(wl, rank))

    def grads(x, v, m):
        gx = np.zeros_like(x)
        gv = np.zeros_like(v)
        gv[:, 2] = m / n
        r = np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2)
        gx[:, 0] = 1e3 / n * x[:, 0] / r
        gx[:, 1] = 1e3 / n * x[:, 1] / r
        return gx, gv

    def one(prec):
        with sv.ForceMethod(softening2=EPS2, precision=prec, efield=(0.0, 0.0, EZ), device=local) as fm:
            for _ in range(args.warmup):  # warm-up sweeps (forward + backward)
                fm.upload(st)
                fm.adjoint_forward(nsteps, DT, 0.0, every)
                x, v, _ = fm.download()
                gx, gv = grads(x, v, st["m"])
                fm.adjoint_backward(gx, gv)
            times, out = [], None
            for _ in range(max(1, args.steps)):
                fm.upload(st)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                fm.adjoint_forward(nsteps, DT, 0.0, every)
                x, v, _ = fm.download()
                out = fm.adjoint_backward(*grads(x, v, st["m"]))
                times.append(time.perf_counter() - t0)
            return float(np.median(times)), out

    t_mixed, g_mixed = one(sv.MIXED)
    t_fp64, g_fp64 = one(sv.FP64)
    err = {k: float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
           for k, a, b in (("dL_dx0", g_mixed[0], g_fp64[0]), ("dL_dv0", g_mixed[1], g_fp64[1]),
                           ("dL_dEz", g_mixed[2][2:], g_fp64[2][2:]))}
    value = world * n * nsteps / t_mixed
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": value, "unit": "particle-steps/s (forward + backward)", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_mixed / nsteps * 1e3,
            "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 pairs (hi/lo splits in the Jacobian), f64 state",
            "data": "synthetic (seeded plume generator)",
            "config": {"workload": args.workload, "desc": wl["desc"], "n": n, "rollout_steps": nsteps,
                       "checkpoint_every": every},
            "e2e": {"value": value, "unit": "particle-steps/s", "note": "the timed region is the C ABI calls with "
                    "host buffers (forward, download of the final state, backward with host gradients)",
                    "h2d_bytes_per_step": 48 * n / nsteps, "d2h_bytes_per_step": 100 * n / nsteps},
            "fp64_adjoint": {"value": world * n * nsteps / t_fp64, "unit": "particle-steps/s",
                             "ms_rollout": t_fp64 * 1e3},
            "speedup_vs_fp64_adjoint": t_fp64 / t_mixed, "grad_rel_diff_mixed_vs_fp64": err}), flush=True)


def run_ours(args, wl, rank, world, local):
    import torch

    import solveit_gpu as sv

    if wl["method"] == "batch":
        return run_batch(args, wl, rank, world, local)
    if wl["method"] == "adjoint":
        return run_adjoint(args, wl, rank, world, local)

    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    n = wl["n"]
    st = plume.make_plume(n, wl["length"], plume_seed(wl, rank))
    if wl["method"] == "fmm":
        kw = dict(method=sv.FMM, precision=sv.MIXED, fmm_order=wl["order"], fmm_ws=wl["ws"],
                  fmm_leaf_target=wl["leaf"], fmm_m2l_tc=args.m2l_tc, fmm_near=args.fmm_near or wl.get("near", 0))
    elif wl["method"] == "bh":
        kw = dict(method=sv.BARNES_HUT, precision=sv.MIXED, theta=wl["theta"], leaf_size=wl["leaf"])
    else:
        kw = dict(method=sv.DIRECT, precision=sv.FP64 if wl.get("precision") == "fp64" else sv.MIXED)
    fm = sv.ForceMethod(softening2=EPS2, efield=(0.0, 0.0, EZ), device=local, profile_phases=1, **kw)
    fm.upload(st)
    root_scale, tune_ms = None, None
    if wl["method"] == "fmm" and args.root_scale is not None:
        fm.set_params(fmm_root_scale=args.root_scale)
        root_scale = args.root_scale
    elif wl["method"] == "fmm" and not args.no_tune:
        # untimed set-up: the root cube's scale (leaf box size) for this plume
        root_scale, tune_ms = fm.fmm_tune()
    stream = torch.cuda.ExternalStream(fm.stream, device=local)
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")

    # ---- device-resident timing
    t = 0.0
    for _ in range(args.warmup):
        fm.leapfrog(1, DT, t)
        t += DT
    fm.sync()
    t_start = t
    snap = fm.download()  # the state at the start of the timed window (the e2e run repeats the window)
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    phase_ms = np.zeros(8)
    clk_p, clk_f = sample_clocks_start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = fm.launches
    wall0 = time.perf_counter()
    for k in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        evs[k][0].record(stream)
        fm.leapfrog(1, DT, t)
        evs[k][1].record(stream)
        t += DT
        fm.sync()
        s = fm.stats()
        phase_ms += np.array(list(s.ms_phase))
    torch.cuda.synchronize()
    wall = time.perf_counter() - wall0
    launches = fm.launches - launches0
    clocks = sample_clocks_stop(clk_p, clk_f, local)
    step_ms = float(sum(a.elapsed_time(b) for a, b in evs))
    if dist:
        step_ms = max_over_ranks(step_ms, dist, f"cuda:{local}")
    ms_per_step = step_ms / args.steps
    value = world * n * args.steps / (step_ms / 1e3)
    phase_ms /= args.steps
    stats = fm.stats()

    if args.timed_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "ms_per_step": ms_per_step,
                              "phases_ms": list(map(float, phase_ms)), "m2l_tc": int(stats.m2l_tc),
                              "m2l": stats.cell_interactions, "timed_only": True}), flush=True)
        fm.close()
        return
    # ---- end to end through the C ABI with pinned host buffers: the same
    # steps again from the same state; each step uploads the current state,
    # runs one step and downloads positions, velocities and status into the
    # buffers the next step uploads
    pin = {k: torch.empty(st[k].shape, dtype=torch.float64 if st[k].dtype == np.float64 else torch.int32,
                          pin_memory=True) for k in ("x", "v", "q", "m", "status", "t_inj")}
    import ctypes as C

    L = sv.load()

    def ptr(tn):
        return C.c_void_p(tn.data_ptr())

    def reset_pins():
        for k in ("q", "m", "t_inj"):
            pin[k].numpy()[...] = st[k]
        pin["x"].numpy()[...] = snap[0]
        pin["v"].numpy()[...] = snap[1]
        pin["status"].numpy()[...] = snap[2]

    def check(rc):
        if rc != 0:
            raise RuntimeError(L.sv_last_error(fm.h).decode())

    def e2e_step(t0):
        # the step's inputs up (positions, velocities, statuses; charges, masses and
        # injection times stay resident), one step, its result down
        check(L.sv_update_state(fm.h, n, ptr(pin["x"]), ptr(pin["v"]), ptr(pin["status"])))
        check(L.sv_leapfrog(fm.h, 1, DT, t0))
        check(L.sv_download(fm.h, ptr(pin["x"]), ptr(pin["v"]), ptr(pin["status"])))

    def load_window_start():
        reset_pins()
        check(L.sv_upload(fm.h, n, ptr(pin["x"]), ptr(pin["v"]), ptr(pin["q"]), ptr(pin["m"]), ptr(pin["status"]),
                          ptr(pin["t_inj"])))

    load_window_start()
    e2e_step(t_start)  # warm-up of the host path, then back to the window's first state
    load_window_start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    e0 = time.perf_counter()
    for k in range(args.steps):
        e2e_step(t_start + k * DT)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - e0
    if dist:
        e2e_s = max_over_ranks(e2e_s, dist, f"cuda:{local}")
    h2d = n * (3 * 8 + 3 * 8 + 4)
    d2h = n * (3 * 8 + 3 * 8 + 4)
    e2e = {"value": world * n * args.steps / e2e_s, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": d2h, "window": "the timed steps of value, from the same state",
           "per_step": "sv_update_state (positions, velocities, statuses from pinned host arrays; charges, "
                       "masses and injection times stay resident), sv_leapfrog(1), sv_download"}

    line = {"metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 pair/expansion arithmetic, f64 state and integration",
            "data": "synthetic (seeded plume generator, seed 1000*workload+rank)",
            "config": {"workload": args.workload, "desc": wl["desc"], "n_per_gpu": n,
                       "parallelism": f"replicas x{world}" if world > 1 else "single GPU",
                       "l2": "512 MB written between timed steps (L2 flush)", "leaf_level": stats.levels,
                       "leaf_boxes": stats.boxes, "fmm_root_scale": root_scale,
                       "tuning": None if tune_ms is None else
                       f"sv_fmm_tune before the warm-up (untimed): root scales 1..1.875, kept {root_scale} "
                       f"({tune_ms:.3f} ms per force evaluation)"},
            "clocks": clocks, "e2e": e2e, "gpu_launches": int(launches // max(1, args.steps)) * args.steps,
            "wall_s_timed_region": wall}

    if rank == 0:
        # ---- phase breakdown and roofline of the dominant kernel
        names = ["sort", "tree", "lists", "upward_p2m_m2m", "downward_m2l_l2l", "l2p", "near_p2p", "scatter"]
        if wl["method"] == "bh":
            names = ["sort", "tree", "-", "cell_properties", "-", "walk", "walk_tail", "scatter"]
        line["phases_ms"] = {nm: round(float(v), 4) for nm, v in zip(names, phase_ms)}
        sm_max = measured_peaks().get("sm_max_mhz", 2070.0)
        fp32_peak, sms = fp32_peak_tflops(local, sm_max)
        if wl["method"] == "fmm":
            near_flop = 20.0 * stats.pair_interactions
            dom_ms = phase_ms[6]
            achieved = near_flop / (dom_ms * 1e-3) / 1e12
            m2l_flop = stats.flops_algorithmic - near_flop - n * 8.0 * (wl["order"] * (wl["order"] + 1) / 2) * 4
            same_cfg = root_scale == P2P_TRAFFIC["root_scale"] and stats.levels == P2P_TRAFFIC["leaf_level"]
            line["roofline"] = {"kernel": "p2p_kernel (near field, 20 flop/pair)", "bound": "fp32",
                                "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                                "frac": achieved / fp32_peak,
                                "traffic": P2P_TRAFFIC["bytes"] if same_cfg else None,
                                "traffic_source": "dram__bytes_read.sum + dram__bytes_write.sum of one p2p_kernel "
                                                  f"launch at root scale {P2P_TRAFFIC['root_scale']} (leaf level "
                                                  f"{P2P_TRAFFIC['leaf_level']}), one ncu capture of this "
                                                  "workload; null when this run's root scale or leaf level differ "
                                                  f"(this run: {root_scale}, level {stats.levels})",
                                "peak_source": f"FP32 FMA rate {sms} SMs x 128 lanes x 2 flop x sm_max_mhz "
                                               f"{sm_max:.0f} of MEASURED_PEAKS.json (no FP32 peak is measured "
                                               "there; the kernel runs on the FP32 pipe, not the tensor cores)",
                                "timing": "CUDA events on the near field's own stream; the kernel shares the "
                                          "GPU with the concurrent upward / downward passes, whose stream has "
                                          "the higher priority, so the span includes their work",
                                "pairs_per_step": stats.pair_interactions,
                                "m2l_per_step": stats.cell_interactions,
                                "m2l_flop_per_step": m2l_flop}
        elif wl["method"] == "bh":
            dom_ms = phase_ms[5]  # the walk (the Barnes-Hut evaluation marks it as phase 5)
            achieved = stats.flops_algorithmic / (dom_ms * 1e-3) / 1e12
            line["roofline"] = {"kernel": "bh_walk_kernel (accepted cells + leaf pairs, 20 flop each)",
                                "bound": "fp32 (a divergent, latency-bound walk)", "achieved": achieved,
                                "peak": fp32_peak, "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": None,
                                "peak_source": f"FP32 FMA rate {sms} SMs x 128 lanes x 2 flop x sm_max_mhz "
                                               f"{sm_max:.0f} of MEASURED_PEAKS.json",
                                "timing": "CUDA events around the walk on the context stream, averaged over the "
                                          "timed steps",
                                "cells_per_step": stats.cell_interactions, "pairs_per_step": stats.pair_interactions}
        else:
            dom_ms = phase_ms[6]
            achieved = stats.flops_algorithmic / (dom_ms * 1e-3) / 1e12
            line["roofline"] = {"kernel": "direct kernel", "bound": "fp64", "achieved": achieved,
                                "peak": None, "unit": "TFLOP/s", "frac": None, "traffic": None}
        # ---- force error against the FP64 GPU direct sum on sampled targets
        if wl["method"] in ("fmm", "bh"):
            x, v, stt = fm.download()
            cur = dict(st, x=x, v=v, status=stt)
            a_fmm = fm.accel()
            tg = np.sort(np.random.default_rng(7).choice(n, 512, replace=False))
            a_ref = fp64_sampled_accel(sv, local, cur, tg)
            d = np.sum((a_fmm[tg] - a_ref) ** 2, axis=1) / np.sum(a_ref ** 2, axis=1)
            line["force_err_rel_l2"] = float(np.sqrt(np.mean(d)))
            line["force_err_max"] = float(np.sqrt(np.max(d)))
            line["force_err_sample"] = ("512 random targets of the state after the timed steps, against the "
                                        "plain FP64 GPU direct sum (pinned to the CPU oracle by the GPU tests)")
            # ---- plain FP64 GPU direct path on the same GPU
            m = min(n, 131072)
            sub = {k: (st[k][:m] if hasattr(st[k], "__len__") else st[k]) for k in st}
            with sv.ForceMethod(softening2=EPS2, method=sv.DIRECT, precision=sv.FP64, device=local,
                                efield=(0.0, 0.0, EZ)) as f64:
                f64.upload(sub)
                f64.leapfrog(1, DT)
                f64.sync()
                t0 = time.perf_counter()
                f64.leapfrog(1, DT)
                f64.sync()
                t_m = time.perf_counter() - t0
            t_n = t_m * (n / m) ** 2
            line["fp64_direct"] = {"value": n / t_n, "unit": "particle-steps/s",
                                   "measured": f"one FP64 direct leapfrog step at N={m}: {t_m * 1e3:.1f} ms, "
                                               f"scaled by (N/{m})^2 to N={n}",
                                   "ms_per_step_at_n": t_n * 1e3,
                                   "extrapolated_from": {"n_measured": m, "n": n, "scaled_by": f"(N/{m})^2",
                                                         "timing": "one step, host wall clock around a "
                                                                   "synchronised call"}}
            line["speedup_vs_fp64_direct"] = value / world / (n / t_n)
        # ---- CPU baseline (C oracle FP64 direct sum, bounded sample)
        threads = os.cpu_count() or 1
        line["cpu_baseline"] = cpu_baseline(st, 2048 if n > 100000 else min(n, 4096), threads)
        print(json.dumps(line), flush=True)
    fm.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="fmm_n1m", choices=sorted(WORKLOADS))
    ap.add_argument("--root-scale", type=float, default=None,
                    help="FMM: this root-cube scale instead of sv_fmm_tune's (profiling a fixed configuration)")
    ap.add_argument("--timed-only", action="store_true",
                    help="only the device-resident timed steps (for profiler launch lists)")
    ap.add_argument("--fmm-near", type=int, default=0, choices=[0, 1, 2],
                    help="FMM near field at ws 2: 1 full cube, 2 trimmed, 0 the workload's choice")
    ap.add_argument("--m2l-tc", type=int, default=0, choices=[-1, 0, 1],
                    help="FMM M2L: 1 tensor cores, -1 FP32 rotation kernel, 0 the library default")
    ap.add_argument("--no-tune", action="store_true",
                    help="skip the autotuner (batch: default depth-model weight; FMM: power-of-two root cube)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    rank, world, local = dist_env()
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        run_reference(args, wl, rank, world)
    else:
        run_ours(args, wl, rank, world, local)


if __name__ == "__main__":
    main()
