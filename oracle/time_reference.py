"""Time the reference's own force methods on a seeded plume (CPU baseline).

TEST INFRASTRUCTURE ONLY: runs oracle/_ref/<variant>/ref_harness (the
reference's sources compiled where they lie by `make -C oracle ref`), which
calls the reference's updateAcceleration() once and prints its wall time.
The reference tree is needed to build the harness, so this runs where the
reference sources are present, not on a machine that only has this
repository.

usage: python oracle/time_reference.py [--mode fmm|bh|direct] [--n 65536]
           [--length 50e-6] [--p 8] [--threads 0] [--seed 2000]

Prints one JSON line: the evaluation's wall time, particle-steps/s of the
force evaluation (n / time), and its per-particle relative-L2 error against
the FP64 direct sum of the C oracle on sampled targets.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import re
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "solveit-code_gb300"))
sys.path.insert(0, HERE)

import oracle_py as O  # noqa: E402
import plume  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--mode", default="fmm", choices=["fmm", "bh", "direct"])
    ap.add_argument("--n", type=int, default=65536)
    ap.add_argument("--length", type=float, default=50e-6)
    ap.add_argument("--p", type=int, default=8)
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--seed", type=int, default=2000)
    ap.add_argument("--variant", default="eps20", choices=["eps20", "stock"])
    args = ap.parse_args()
    threads = args.threads or os.cpu_count() or 1
    harness = os.path.join(HERE, "_ref", args.variant, "ref_harness")
    if not os.path.exists(harness):
        sys.exit("reference harness not built: make -C oracle ref (needs the reference tree)")
    st = plume.make_plume(args.n, args.length, args.seed)
    pos4, vel4, acc4, tinj = plume.to_ref32(st)
    scratch = os.path.join(HERE, "_ref", "scratch")
    os.makedirs(scratch, exist_ok=True)
    with tempfile.TemporaryDirectory(dir=scratch) as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fin, "wb") as f:
            np.array([args.n], np.int32).tofile(f)
            for a in (pos4, vel4, acc4, tinj):
                np.ascontiguousarray(a).tofile(f)
        kw = [f"threads={threads}"]
        if args.mode == "fmm":
            kw.append(f"p={args.p}")
        if args.mode == "bh":
            kw.append(f"theta={args.theta}")
        r = subprocess.run([harness, args.mode, fin, fout] + kw, capture_output=True, text=True)
        if r.returncode != 0:
            sys.exit(f"harness failed ({r.returncode}): {r.stderr[-500:]}")
        sec = float(re.search(r"update_s=([0-9.eE+-]+)", r.stderr).group(1))
        out = np.fromfile(fout, np.float32)[: 12 * args.n].reshape(3, args.n, 4)
    acc = out[2][:, :3].astype(np.float64)
    eps2 = 1e-20 if args.variant == "eps20" else 6.4e-19
    tg = np.arange(0, args.n, max(1, args.n // 1024))
    ref = O.direct_f64(st, eps2, targets=tg)
    err = O.rel_l2(acc[tg], ref, st["status"][tg])[0]
    print(json.dumps({"mode": args.mode, "n": args.n, "length_m": args.length, "p": args.p if args.mode == "fmm"
                      else None, "threads": threads, "cpu": platform.processor() or platform.machine(),
                      "update_s": sec, "particle_steps_per_s_force": args.n / sec,
                      "force_err_rel_l2_sampled": float(err), "targets_sampled": int(tg.size)}))


if __name__ == "__main__":
    main()
