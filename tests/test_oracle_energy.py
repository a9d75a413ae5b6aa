"""The energy bookkeeping (Integrator::toggleEnergy): the oracle's FP32
restatement pinned against the reference's own LeapfrogDKD::runSimulation
with the energy file (tests/golden/energy.npz), bit for bit."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
import oracle_py as O  # noqa: E402
from test_oracle_emitter_field import field_of  # noqa: E402

CASES = ("plain", "field", "window")


def fixture():
    return dict(np.load(os.path.join(HERE, "golden", "energy.npz")))


def run_case(g, name, **over):
    init, each, interval, fld = (int(v) for v in g[f"{name}_setup"])
    kw = dict(init_steps=init, steps=each, interval=interval)
    kw.update(over)
    return O.leapfrog_ref32_energy(g[f"{name}_pos4"], g[f"{name}_vel4"], g[f"{name}_acc4"], g[f"{name}_tinj"],
                                   int(g["steps"]), float(g["dt"]), float(g["eps"]), kw["init_steps"], kw["steps"],
                                   kw["interval"], fld=field_of(g) if fld else None, threads=4)


@pytest.mark.parametrize("name", CASES)
def test_energy_records_are_the_reference_file(name):
    g = fixture()
    p, v, a, rec = run_case(g, name)
    ref = g[f"{name}_records"]
    assert rec.shape == ref.shape and rec.shape[0] >= 2
    assert np.array_equal(rec, ref)
    # the bookkeeping leaves the trajectory alone
    assert np.array_equal(p, g[f"{name}_pos4_out"]) and np.array_equal(v, g[f"{name}_vel4_out"])
    assert np.array_equal(a, g[f"{name}_acc4_out"])


def test_fixture_exercises_every_term():
    g = fixture()
    plain, field, window = (g[f"{k}_records"] for k in CASES)
    assert np.all(plain[:, [2, 5]] == 0) and np.all(plain[:, [0, 1, 3, 4]] > 0)  # no field: FE = 0
    assert np.all(field > 0)
    # the injected totals grow as the groups of the plume are injected
    assert np.all(np.diff(field[:, 0]) > 0) and np.all(np.diff(field[:, 1]) > 0)
    # the last record of both is at step 6: the injected totals count every
    # injected particle, the window's sums leave out the five in front of the
    # first active one
    assert window[-1, 0] == field[-1, 0] and window[-1, 2] == field[-1, 2]
    assert window[-1, 3] < field[-1, 3] and window[-1, 5] < field[-1, 5]


def test_energy_depends_on_its_settings():
    """A planted change in the restatement's settings moves the records."""
    g = fixture()
    ref = g["field_records"]
    _, _, _, rec = run_case(g, "field", steps=7)
    assert not np.array_equal(rec[:, 5], ref[:, 5]) and np.array_equal(rec[:, :5], ref[:, :5])
    _, _, _, rec = run_case(g, "field", init_steps=13)
    assert not np.array_equal(rec[:, 2], ref[:, 2])
    _, _, _, rec = run_case(g, "field", interval=3)
    assert rec.shape[0] == 2
