"""Geometry of the FMM's interaction lists with separation 2, full and
trimmed near field (sv_params.fmm_near), restated on the CPU.

The library's list builder (build_lists_box / near_lists_kernel) classifies a
box's candidates, the children of its parent's near boxes, into its near list
and its interaction (M2L) list; trimming moves the (2,2,1)- and (2,2,2)-type
offsets from the first to the second (fmm_trimmable).  These tests check the
rules themselves:
  - 32 offsets of the 5^3 cube are trimmed;
  - none of them has a larger separation ratio than the full cube's closest
    M2L offsets, (3,0,0);
  - on a small octree every (target, source) pair of leaf boxes is counted
    exactly once: by the near field at the leaf level, or by one M2L at the
    level where the pair's ancestors first leave each other's near field.
The GPU tests check the accuracy of the lists the library builds.
"""
import itertools
import math

import numpy as np
import pytest

WS = 2


def trimmable(o):
    a = sorted(abs(v) for v in o)
    return WS == 2 and a[2] == 2 and a[1] == 2 and a[0] >= 1


def near(o, trim):
    return max(abs(v) for v in o) <= WS and not (trim and trimmable(o))


def ratio(o):
    """Sum of the two unit boxes' circumradii over the centre distance."""
    return math.sqrt(3.0) / math.sqrt(sum(v * v for v in o))


def test_trimmed_offsets():
    cube = list(itertools.product(range(-WS, WS + 1), repeat=3))
    trimmed = [o for o in cube if trimmable(o)]
    assert len(trimmed) == 32
    assert sorted({tuple(sorted(abs(v) for v in o)) for o in trimmed}) == [(1, 2, 2), (2, 2, 2)]
    worst_m2l = ratio((3, 0, 0))
    assert max(ratio(o) for o in trimmed) <= worst_m2l + 1e-12
    assert math.isclose(ratio((2, 2, 1)), worst_m2l) and math.isclose(ratio((2, 2, 2)), 0.5)


@pytest.mark.parametrize("trim", [False, True])
def test_near_boxes_have_near_parents(trim):
    """A box's near boxes are children of its parent's near boxes (the
    parent offsets lie in [-1, 1]^3, which trimming never removes), so the
    candidate set of the builder contains every near box."""
    for parity in itertools.product((0, 1), repeat=3):
        for o in itertools.product(range(-WS, WS + 1), repeat=3):
            if not near(o, trim):
                continue
            # target child at coordinates `parity` inside parent 0, source child at parity - o
            po = tuple(0 - ((p - d) // 2) for p, d in zip(parity, o))
            assert max(abs(v) for v in po) <= 1
            assert near(po, trim)


@pytest.mark.parametrize("trim", [False, True])
def test_every_pair_counted_once(trim):
    """Full octree of depth 4 (16^3 leaf boxes): for each target leaf box and
    each source leaf box, count the levels at which the pair is handled."""
    depth = 4
    side = 1 << depth
    rng = np.random.default_rng(1)
    targets = [tuple(int(v) for v in rng.integers(0, side, 3)) for _ in range(6)]
    for t in targets:
        for s in itertools.product(range(side), repeat=3):
            if s == t:
                continue
            handled = 0
            # near field at the leaf level
            if near(tuple(a - b for a, b in zip(t, s)), trim):
                handled += 1
            # M2L at level l: the boxes' ancestors at l are not near each other,
            # but their parents are (the candidate rule of the builder); level 1
            # pairs are all near (no offset exceeds 1 there)
            for l in range(2, depth + 1):
                sh = depth - l
                ta = tuple(v >> sh for v in t)
                sa = tuple(v >> sh for v in s)
                tp = tuple(v >> 1 for v in ta)
                sp = tuple(v >> 1 for v in sa)
                o = tuple(a - b for a, b in zip(ta, sa))
                po = tuple(a - b for a, b in zip(tp, sp))
                if not near(o, trim) and near(po, trim):
                    handled += 1
            assert handled == 1, (trim, t, s, handled)
