"""The single-emitter background field (InterpolationScheme::Efield with the
walk and interpolation of pwl_interp_2d_scattered.c): the oracle pinned
against the reference reading a seeded field map through its own CSV readers
(tests/golden/emitter_field.npz, made by tests/golden/make_golden.py)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "oracle"))
sys.path.insert(0, os.path.join(HERE, "..", "solveit-code_gb300"))
import oracle_py as O  # noqa: E402
import plume  # noqa: E402

R_MAX = 8.0  # radial extent of the map in units of r0


def fixture():
    return np.load(os.path.join(HERE, "golden", "emitter_field.npz"))


def field_of(g):
    return O.field(g["node_rz"], g["e_r"], g["e_z"], g["triangles"], g["neighbors"], float(g["r0"]), float(g["e0"]))


def inside_map(g, x):
    r = np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2) / float(g["r0"])
    z = x[:, 2] / float(g["r0"])
    return (r < R_MAX) & (z >= 0) & (z <= 140)


def test_ref32_field_bit_exact():
    g = fixture()
    e = O.emitter_field_ref32(field_of(g), g["pos4"])
    assert np.array_equal(e, g["e_out"])


def test_ref32_leapfrog_with_field_bit_exact():
    g = fixture()
    p, v, a, _ = O.leapfrog_ref32_bc(g["dkd_pos4"], g["dkd_vel4"], g["dkd_acc4"], g["dkd_tinj"], int(g["steps"]),
                                     float(g["dt"]), float(g["eps"]), fld=field_of(g))
    assert np.array_equal(p, g["dkd_pos4_out"])
    assert np.array_equal(v, g["dkd_vel4_out"])
    assert np.array_equal(a, g["dkd_acc4_out"])


def test_f64_field_matches_reference():
    g = fixture()
    st = plume.from_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
    e = O.emitter_field_f64(field_of(g), st["x"])
    ref = g["e_out"].astype(np.float64)
    z = st["x"][:, 2] / float(g["r0"])
    off = (z < 0) | (z > 140)
    assert off.sum() == 4 and np.all(e[off] == 0) and np.all(ref[off] == 0)
    ins = inside_map(g, st["x"])
    rel = np.abs(e[ins] - ref[ins]).max(1) / np.linalg.norm(ref[ins], axis=1)
    assert rel.max() < 5e-7  # the reference rounds to FP32 and takes phi through FP32 trig
    # on the axis phi = 0; on the y axis phi = pi/2 for either sign of y (the reference's rule)
    assert e[9, 0] == 0.0 and e[9, 1] > 0 and ref[9, 1] > 0


def test_f64_leapfrog_with_field_matches_reference():
    g = fixture()
    st = plume.from_ref32(g["dkd_pos4"], g["dkd_vel4"], g["dkd_acc4"], g["dkd_tinj"])
    x, v, _, _ = O.leapfrog_f64_bc(st, int(g["steps"]), float(g["dt"]), float(g["eps"]), fld=field_of(g))
    vr = g["dkd_vel4_out"][:, :3]
    assert np.max(np.abs(x - g["dkd_pos4_out"][:, :3])) < 2e-12
    assert np.max(np.abs(v - vr).max(1) / np.linalg.norm(vr, axis=1)) < 2e-6


def test_interpolation_is_linear_in_each_triangle():
    """At a node the map returns the node's value; at a triangle's centroid,
    the mean of its vertices."""
    g = fixture()
    fld = field_of(g)
    r0, e0 = float(g["r0"]), float(g["e0"])
    nodes, tri = g["node_rz"], g["triangles"]
    k = tri[100]
    c = nodes[k].mean(0)
    pts = np.array([[c[0] * r0, 0.0, c[1] * r0], [nodes[k[0], 0] * r0, 0.0, nodes[k[0], 1] * r0]])
    e = O.emitter_field_f64(fld, pts)
    np.testing.assert_allclose(e[0, 0], e0 * g["e_r"][k].mean(), rtol=1e-12)
    np.testing.assert_allclose(e[0, 2], e0 * g["e_z"][k].mean(), rtol=1e-12)
    np.testing.assert_allclose(e[1, 2], e0 * g["e_z"][k[0]], rtol=1e-12)
