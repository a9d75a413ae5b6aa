"""The hand-written adjoint of the leapfrog + direct-sum rollout.

The rollout is wrapped in a torch.autograd.Function here, in the test
harness only: forward = sv_adjoint_forward (keeping checkpoints), backward =
sv_adjoint_backward.  Loss, at the final step:
    L = mean_i(m_i v_z,i)  [amu m/s]  +  1e3 * mean_i(sqrt(x_i^2 + y_i^2))  [m].
Gradients w.r.t. initial positions, velocities and the E_z amplitude are
checked against central finite differences of the FP64 rollout with relative
step 1e-6, to 1e-4.  The two loss terms are checked separately: internal
Coulomb forces cancel in the total momentum, so the momentum term's
dependence on positions is zero up to round-off, which would swamp a
finite difference of the (much smaller) radius term.
"""
import numpy as np
import pytest

import oracle_py as O
import plume
import solveit_gpu as sv

pytestmark = pytest.mark.gpu

EPS20 = 1e-20
DT = 1e-13
EZ = 1e8


def loss_terms(x, v, m):
    mom = float(np.mean(m * v[:, 2]))
    rad = 1e3 * float(np.mean(np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2)))
    return mom, rad


def loss_grads(x, v, m, w_mom, w_rad):
    n = x.shape[0]
    gx = np.zeros_like(x)
    gv = np.zeros_like(v)
    gv[:, 2] = w_mom * m / n
    r = np.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2)
    gx[:, 0] = w_rad * 1e3 / n * x[:, 0] / r
    gx[:, 1] = w_rad * 1e3 / n * x[:, 1] / r
    return gx, gv


def rollout(state, nsteps, ez, prec, ckpt=5):
    with sv.ForceMethod(softening2=EPS20, precision=prec, efield=(0.0, 0.0, ez)) as fm:
        fm.upload(state)
        fm.adjoint_forward(nsteps, DT, 0.0, ckpt)
        x, v, _ = fm.download()
    return x, v


def adjoint(state, nsteps, ez, prec, w_mom, w_rad, ckpt=5):
    with sv.ForceMethod(softening2=EPS20, precision=prec, efield=(0.0, 0.0, ez)) as fm:
        fm.upload(state)
        fm.adjoint_forward(nsteps, DT, 0.0, ckpt)
        x, v, _ = fm.download()
        gx, gv = loss_grads(x, v, state["m"], w_mom, w_rad)
        return fm.adjoint_backward(gx, gv)


@pytest.fixture(scope="module")
def small():
    st = plume.make_plume(384, 0.3e-6, 4004)
    return st


def test_radius_term_directional_fd(small):
    nsteps = 20
    gx0, gv0, _ = adjoint(small, nsteps, EZ, sv.FP64, 0.0, 1.0)
    rng = np.random.default_rng(1)
    for _ in range(3):
        dx = rng.normal(size=small["x"].shape)
        dv = rng.normal(size=small["v"].shape)
        ex = 1e-6 * np.linalg.norm(small["x"]) / np.linalg.norm(dx)
        ev = 1e-6 * np.linalg.norm(small["v"]) / np.linalg.norm(dv)
        for d_x, d_v, eps in ((dx, 0 * dv, ex), (0 * dx, dv, ev)):
            sp = dict(small, x=small["x"] + eps * d_x, v=small["v"] + eps * d_v)
            sm = dict(small, x=small["x"] - eps * d_x, v=small["v"] - eps * d_v)
            rp = loss_terms(*rollout(sp, nsteps, EZ, sv.FP64), small["m"])[1]
            rm = loss_terms(*rollout(sm, nsteps, EZ, sv.FP64), small["m"])[1]
            fd = (rp - rm) / (2 * eps)
            ad = float(np.sum(gx0 * d_x) + np.sum(gv0 * d_v))
            assert abs(ad - fd) <= 1e-4 * abs(fd), (ad, fd)


def test_momentum_term_field_and_velocity(small):
    nsteps = 20
    gx0, gv0, ge = adjoint(small, nsteps, EZ, sv.FP64, 1.0, 0.0)
    h = 1e-6 * EZ
    mp = loss_terms(*rollout(small, nsteps, EZ + h, sv.FP64), small["m"])[0]
    mm = loss_terms(*rollout(small, nsteps, EZ - h, sv.FP64), small["m"])[0]
    fd = (mp - mm) / (2 * h)
    assert abs(ge[2] - fd) <= 1e-4 * abs(fd), (ge[2], fd)
    # dL/dv0_z = m/N exactly; internal forces cancel in the total momentum
    np.testing.assert_allclose(gv0[:, 2], small["m"] / small["m"].size, rtol=1e-9)
    assert np.max(np.abs(gx0)) < 1e-6 * np.max(np.abs(gv0)) / DT


def test_field_gradient_matches_oracle_fd(small):
    """dL/dE_z of the GPU adjoint against central differences of the CPU
    oracle's FP64 leapfrog (the FP64 reference gradient)."""
    nsteps = 10
    _, _, ge = adjoint(small, nsteps, EZ, sv.FP64, 1.0, 1.0)
    h = 1e-6 * EZ
    vals = []
    for e in (EZ + h, EZ - h):
        x, v, _ = O.leapfrog_f64(small, nsteps, DT, EPS20, (0.0, 0.0, e))
        vals.append(sum(loss_terms(x, v, small["m"])))
    fd = (vals[0] - vals[1]) / (2 * h)
    assert abs(ge[2] - fd) <= 1e-4 * abs(fd), (ge[2], fd)


def test_checkpoint_interval_does_not_change_gradient(small):
    g1 = adjoint(small, 12, EZ, sv.FP64, 1.0, 1.0, ckpt=1)
    g2 = adjoint(small, 12, EZ, sv.FP64, 1.0, 1.0, ckpt=5)
    g3 = adjoint(small, 12, EZ, sv.FP64, 1.0, 1.0, ckpt=12)
    for a, b in ((g1, g2), (g1, g3)):
        for u, w in zip(a, b):
            np.testing.assert_allclose(u, w, rtol=1e-9, atol=1e-30)


def test_autograd_function_and_mixed_precision():
    torch = pytest.importorskip("torch")
    st = plume.make_plume(16384, 1e-6, 4000)
    nsteps, ckpt = 50, 10
    m = torch.tensor(st["m"])

    class Rollout(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x0, v0, ez, prec):
            fm = sv.ForceMethod(softening2=EPS20, precision=prec, efield=(0.0, 0.0, float(ez)))
            fm.upload(dict(st, x=x0.detach().numpy(), v=v0.detach().numpy()))
            fm.adjoint_forward(nsteps, DT, 0.0, ckpt)
            x, v, _ = fm.download()
            ctx.fm = fm
            return torch.from_numpy(x), torch.from_numpy(v)

        @staticmethod
        def backward(ctx, gx, gv):
            ox, ov, oe = ctx.fm.adjoint_backward(gx.numpy(), gv.numpy())
            ctx.fm.close()
            return torch.from_numpy(ox), torch.from_numpy(ov), torch.tensor(oe[2], dtype=torch.float64), None

    grads = {}
    for prec in (sv.FP64, sv.MIXED):
        x0 = torch.tensor(st["x"], requires_grad=True)
        v0 = torch.tensor(st["v"], requires_grad=True)
        ez = torch.tensor(EZ, dtype=torch.float64, requires_grad=True)
        x, v = Rollout.apply(x0, v0, ez, prec)
        loss = torch.mean(m * v[:, 2]) + 1e3 * torch.mean(torch.sqrt(x[:, 0] ** 2 + x[:, 1] ** 2))
        loss.backward()
        grads[prec] = (x0.grad.numpy(), v0.grad.numpy(), float(ez.grad))
    gx64, gv64, ge64 = grads[sv.FP64]
    gxm, gvm, gem = grads[sv.MIXED]
    assert np.linalg.norm(gxm - gx64) <= 1e-4 * np.linalg.norm(gx64)
    assert np.linalg.norm(gvm - gv64) <= 1e-4 * np.linalg.norm(gv64)
    assert abs(gem - ge64) <= 1e-4 * abs(ge64)


def test_c4_adjoint_against_finite_differences():
    """The adjoint workload's own configuration: N = 16,384, 50 steps,
    checkpoint every 10.  The FP64 and the mixed-precision adjoint gradients
    of the radius term (x0, v0) and of the momentum term (E_z) against
    central finite differences of the FP64 rollout, to 1e-4.

    Steps are h = 1e-6 of the perturbed vector's norm and h / 2, combined by
    Richardson extrapolation (4 D(h/2) - D(h)) / 3: along positions the
    rollout is stiff (pairs pass within a few softening lengths), and the
    plain central difference at h = 1e-6 keeps an O(h^2) truncation error of
    ~1e-3 that the extrapolation removes.  Directions: a seeded random one and
    the radial one (x, y, 0)/r per particle.  The reference function is the
    FP64 rollout; a finite difference of the mixed-precision rollout itself is
    limited by its FP32 force rounding (the rollout is not smooth at the
    1e-6 scale along random directions), and is checked along the radial
    directions only."""
    st = plume.make_plume(16384, 1e-6, 4000)
    nsteps, ckpt = 50, 10
    gx64, gv64, _ = adjoint(st, nsteps, EZ, sv.FP64, 0.0, 1.0, ckpt)
    gxm, gvm, _ = adjoint(st, nsteps, EZ, sv.MIXED, 0.0, 1.0, ckpt)
    r = np.sqrt(st["x"][:, 0] ** 2 + st["x"][:, 1] ** 2)
    radial = np.stack([st["x"][:, 0] / r, st["x"][:, 1] / r, np.zeros_like(r)], axis=1)
    rng = np.random.default_rng(16384)

    def radius(s, prec):
        return loss_terms(*rollout(s, nsteps, EZ, prec, ckpt), st["m"])[1]

    def fd(key, d, rel, prec):
        eps = rel * np.linalg.norm(st[key]) / np.linalg.norm(d)
        return (radius(dict(st, **{key: st[key] + eps * d}), prec) -
                radius(dict(st, **{key: st[key] - eps * d}), prec)) / (2 * eps)

    for key, g64, gm in (("x", gx64, gxm), ("v", gv64, gvm)):
        for name, d in (("random", rng.normal(size=st[key].shape)), ("radial", radial)):
            ref = (4 * fd(key, d, 5e-7, sv.FP64) - fd(key, d, 1e-6, sv.FP64)) / 3
            for g in (g64, gm):
                ad = float(np.sum(g * d))
                assert abs(ad - ref) <= 1e-4 * abs(ref), (key, name, ad, ref)
            if name == "radial":
                mix = (4 * fd(key, d, 5e-7, sv.MIXED) - fd(key, d, 1e-6, sv.MIXED)) / 3
                assert abs(float(np.sum(gm * d)) - mix) <= 1e-4 * abs(mix), (key, mix)
    # the field amplitude, through the momentum term
    _, _, ge64 = adjoint(st, nsteps, EZ, sv.FP64, 1.0, 0.0, ckpt)
    _, _, gem = adjoint(st, nsteps, EZ, sv.MIXED, 1.0, 0.0, ckpt)
    h = 1e-6 * EZ
    fde = (loss_terms(*rollout(st, nsteps, EZ + h, sv.FP64, ckpt), st["m"])[0] -
           loss_terms(*rollout(st, nsteps, EZ - h, sv.FP64, ckpt), st["m"])[0]) / (2 * h)
    for g in (ge64, gem):
        assert abs(g[2] - fde) <= 1e-4 * abs(fde), (g[2], fde)
