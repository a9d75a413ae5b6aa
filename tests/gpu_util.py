"""Shared helpers of the GPU parity tests."""
import numpy as np

import oracle_py as O
import plume
import solveit_gpu as sv


def run_accel(state, **kw):
    with sv.ForceMethod(**kw) as fm:
        fm.upload(state)
        a = fm.accel()
        st = fm.stats()
        return a, st


def rel_l2(a, ref, status):
    return O.rel_l2(a, ref, status)[0]
