"""Pin the C oracle against fixtures produced by running the reference itself.

The fixtures in tests/golden/ were written by tests/golden/make_golden.py from
the reference compiled from its own sources; the *_ref32 restatements must
reproduce them bit for bit (same FP32 state, same operation order).
"""
import os

import numpy as np
import pytest

import oracle_py as O
import plume


def load(golden_dir, name):
    return dict(np.load(os.path.join(golden_dir, name)))


def test_constants():
    # K = e^2/(4 pi eps0 amu) as the reference evaluates it (constants.h:46)
    assert abs(O.k_const() - 1.3895e-1) / 1.3895e-1 < 1e-3 or O.k_const() > 0
    e = 1.6021766e-19
    eps0 = 8.85419e-12
    amu = 1.66053904e-27
    k = np.float32(e) * np.float32(e) / (4 * np.pi * np.float32(eps0) * np.float32(amu))
    assert abs(O.k_const() - float(k)) / float(k) < 1e-6
    assert O.lib().orc_species_mass(0) == 111.0
    assert O.lib().orc_species_mass(1) == 309.0


@pytest.mark.parametrize("sym", [0, 1, 2])
def test_direct_bit_exact(golden_dir, sym):
    g = load(golden_dir, "direct_n512.npz")
    images = O.trans_images(2, (1, 1, 0), lattice=g["lattice"]) if sym == 2 else None
    acc = O.direct_ref32(g["pos4"], g["vel4"], g["acc4"], float(g["eps"]), sym=sym, images=images,
                         domain_size=g["domain"])
    assert np.array_equal(acc, g[f"acc_sym{sym}"])


def test_trans_image_list():
    img = O.trans_images(2, (1, 1, 0))
    assert img.shape == (81, 3)
    assert len({tuple(r) for r in img}) == 81
    assert set(np.unique(img[:, 0])) == set(range(-4, 5))
    assert np.all(img[:, 2] == 0)
    # one axis periodic: 2n+1 images
    assert O.trans_images(2, (0, 0, 1)).shape == (9, 3)
    # three axes: (2n+1)^3
    assert O.trans_images(1, (1, 1, 1)).shape == (27, 3)


def test_status_handling(golden_dir):
    g = load(golden_dir, "direct_n512.npz")
    acc = g["acc_sym0"]
    # out-of-bounds and crashed targets are untouched, source-only receives no force
    for i in (5, 7, 9):
        assert np.all(acc[i, :3] == 0.0)


def test_leapfrog_bit_exact(golden_dir):
    g = load(golden_dir, "dkd_n256.npz")
    p, v, a = O.leapfrog_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"], int(g["steps"]),
                               float(g["dt"]), float(g["eps"]), (0.0, 0.0, float(g["ez"])))
    assert np.array_equal(p, g["pos4_out"])
    assert np.array_equal(v, g["vel4_out"])
    assert np.array_equal(a, g["acc4_out"])


def test_f64_matches_reference_direct(golden_dir):
    g = load(golden_dir, "direct_n512.npz")
    st = plume.from_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
    for sym in (0, 1, 2):
        off = None
        if sym == 2:
            img = O.trans_images(2, (1, 1, 0), lattice=g["lattice"])
            off = img * g["domain"].astype(np.float64)
        a = O.direct_f64(st, float(g["eps"]), sym=sym, img_off=off)
        ref = g[f"acc_sym{sym}"][:, :3].astype(np.float64)
        l2, mx, _, _ = O.rel_l2(a, ref, st["status"])
        # the reference forms coordinate differences in FP32
        assert l2 < 1e-6, (sym, l2)


def test_f64_leapfrog_close_to_reference(golden_dir):
    g = load(golden_dir, "dkd_n256.npz")
    st = plume.from_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
    x, v, a = O.leapfrog_f64(st, int(g["steps"]), float(g["dt"]), float(g["eps"]),
                             (0.0, 0.0, float(g["ez"])))
    vr = g["vel4_out"][:, :3].astype(np.float64)
    xr = g["pos4_out"][:, :3].astype(np.float64)
    assert np.max(np.abs(v - vr) / np.linalg.norm(vr, axis=1)[:, None]) < 1e-5
    assert np.max(np.abs(x - xr)) < 1e-12


def test_bh_and_fmm_envelopes(golden_dir):
    """Accuracy of the reference's own BH (theta 0.5) and FMM (p 8) against
    the FP64 direct sum: the envelopes the GPU methods are held to."""
    g = load(golden_dir, "bh_n4096.npz")
    st = plume.from_ref32(g["pos4"], g["vel4"], g["acc4"], g["tinj"])
    ref = O.direct_f64(st, float(g["eps"]))
    l2_bh = O.rel_l2(g["acc_bh"][:, :3], ref, st["status"])[0]
    f = load(golden_dir, "fmm_n4096.npz")
    l2_fmm = O.rel_l2(f["acc_fmm"][:, :3], ref, st["status"])[0]
    assert 1e-3 < l2_bh < 2e-2
    assert 1e-5 < l2_fmm < 1e-3


def test_energy_two_body():
    st = {"x": np.array([[0.0, 0, 0], [1e-9, 0, 0]]), "v": np.array([[1.0, 0, 0], [0, 2.0, 0]]),
          "q": np.ones(2), "m": np.array([111.0, 309.0])}
    ke, pe = O.energy_f64(st, 0.0)
    amu = O.lib().orc_amu()
    assert abs(ke - 0.5 * amu * (111.0 * 1 + 309.0 * 4)) / ke < 1e-12
    e = O.lib().orc_elem_charge()
    kc = O.lib().orc_coulomb_ke()
    assert abs(pe - e * e * kc / 1e-9) / pe < 1e-12


@pytest.mark.parametrize("name", ["bh_n65536_sampled.npz", "fmm_n65536_z50_sampled.npz"])
def test_sampled_fixture_plume_and_reference_error(golden_dir, name):
    """The seeded plume generator reproduces the fixture's plume here (the
    sampled particles' FP32 positions, bit for bit), and the reference's own
    Barnes-Hut / FMM error on it against the oracle's FP64 direct sum is the
    envelope the GPU tests hold the GPU methods to."""
    g = load(golden_dir, name)
    n, tg = int(g["n"]), g["targets"]
    st = plume.make_plume(n, float(g["length"]), int(g["seed"]))
    pos4 = plume.to_ref32(st)[0]
    assert np.array_equal(pos4[tg], g["pos4_targets"])
    ref = O.direct_f64(st, float(g["eps"]), targets=tg)
    err = O.rel_l2(g["acc_ref"].astype(np.float64), ref, st["status"][tg])[0]
    # the reference's monopole Barnes-Hut and uniform-depth ws-1 FMM
    assert (3e-3 < err < 2e-2) if "bh" in name else (5e-5 < err < 1e-3), err
