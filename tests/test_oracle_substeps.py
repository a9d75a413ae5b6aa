"""The multi-rate leapfrog (LeapfrogDKDSubsteps) and the single-rate loop:
the oracle pinned against the reference's own integrators
(LeapfrogDKD::runSimulation and LeapfrogDKDSubsteps::runSimulation driven
headlessly, tests/golden/substeps.npz)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
import oracle_py as O  # noqa: E402

# the substep requests of the fixture: (dt, BoundaryConditionOptions, (|x|, |y|, |z|, r), time limit)
SUBSTEP_CASES = {
    "core": [(1e-13, 1, (0.0, 0.0, 0.0, 1e-8), 0.0)],
    "nested": [(3.4e-13, 1, (0.0, 0.0, 0.0, 1.4e-8), 0.0), (1.2e-13, 3, (0.0, 0.0, 0.0, 8e-9), 2.9e-12)],
}


def fixture():
    return np.load(os.path.join(HERE, "golden", "substeps.npz"))


def args_of(g):
    return (g["pos4"], g["vel4"], g["acc4"], g["tinj"], int(g["steps"]), float(g["dt"]), float(g["eps"]))


def test_single_rate_loop_is_the_reference_integrator():
    """orc_leapfrog_ref32 (injection window, force, kick) against the
    reference's own LeapfrogDKD::runSimulation."""
    g = fixture()
    p, v, a = O.leapfrog_ref32(*args_of(g))
    assert np.array_equal(p, g["single_pos4_out"])
    assert np.array_equal(v, g["single_vel4_out"])
    assert np.array_equal(a, g["single_acc4_out"])


@pytest.mark.parametrize("name", sorted(SUBSTEP_CASES))
def test_substeps_bit_exact(name):
    g = fixture()
    p, v, a, lev = O.leapfrog_substeps_ref32(*args_of(g), SUBSTEP_CASES[name])
    assert np.array_equal(p, g[name + "_pos4_out"])
    assert np.array_equal(v, g[name + "_vel4_out"])
    assert np.array_equal(a, g[name + "_acc4_out"])
    assert len(np.unique(lev)) >= 2  # particles on more than one level


def test_single_level_table_rewrites_source_only_status():
    """With a table that resolves to one level, setParticleStatus makes every
    active particle a target, the source-only ones included, as the
    reference's substep integrator does."""
    g = fixture()
    p, v, a, lev = O.leapfrog_substeps_ref32(*args_of(g), [(2e-12, 0, (0, 0, 0, 0), 0.0)])
    assert np.all(lev == 0)
    assert np.all(a[:, 3] == 1.0) and np.any(g["acc4"][:, 3] == 2.0)
