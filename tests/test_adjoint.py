"""Differentiable form: the discrete adjoint of the time step (cnv_adjoint_*).

The gradient of J = 1/2 sum w(T)^2 dx dy with respect to the initial vorticity and the lid speed,
from the hand-written adjoint kernels, must match central finite differences of the forward run
(eps = 1e-6, seeded random directions in (w0, lid)) to FD_RTOL relative per direction. The
forward run of the adjoint form must be the step of cnv_step with the direct Poisson solve, bit
for bit, and the converged reference step of the oracle to 1e-10. The checkpoint interval must
not change the gradient.
"""
from __future__ import annotations

import numpy as np
import pytest

FD_EPS = 1e-6
FD_RTOL = 1e-6        # |fd - adjoint| / |adjoint| per direction
ORACLE_TOL = 1e-10    # adjoint-form forward vs the oracle's converged SOR steps


def stable_dt(n, re, lid=1.0):
    h = 1.0 / n
    return 0.2 * min(h * h * re / 4, h / abs(lid))


def make_cfg(cnv, n, re=400.0, lid=1.0, order=6):
    return cnv.default_config(nx=n, ny=n, Re=re, u4=lid, dt=stable_dt(n, re, lid), order=order)


def directions(n, count, seed):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = np.zeros((n, n))
        d[1:-1, 1:-1] = rng.standard_normal((n - 2, n - 2))
        out.append((d, float(rng.standard_normal())))
    return out


def fd_check(cnv, adj, w0, lid, nsteps, dirs, eps=FD_EPS):
    """Relative error per direction between the adjoint gradient and central differences."""
    J, gw, glid = adj.enstrophy_gradient(w0, lid, nsteps)
    h2 = adj.h2

    def objective(w, l):
        wT = adj.forward(w, l, nsteps)
        return 0.5 * h2 * float(np.sum(wT * wT))

    errs = []
    for d, dl in dirs:
        fd = (objective(w0 + eps * d, lid + eps * dl) - objective(w0 - eps * d, lid - eps * dl)) / (2 * eps)
        ad = float(np.sum(gw * d)) + glid * dl
        errs.append(abs(fd - ad) / abs(ad))
    return J, gw, glid, errs


@pytest.mark.gpu
@pytest.mark.parametrize("n,order,steps,every", [(32, 6, 60, 10), (48, 4, 40, 7), (64, 2, 30, 30)])
def test_adjoint_matches_finite_differences(cnv, n, order, steps, every):
    w0 = cnv.noise_field(n, seed=n, sigma=1.0, passes=4)
    with cnv.Adjoint(make_cfg(cnv, n, order=order), every) as adj:
        J, gw, glid, errs = fd_check(cnv, adj, w0, 1.0, steps, directions(n, 4, seed=7))
    assert J > 0 and np.all(gw[0] == 0) and np.all(gw[:, -1] == 0)
    assert max(errs) <= FD_RTOL, errs


@pytest.mark.gpu
def test_lid_gradient_alone(cnv):
    n, steps = 40, 50
    w0 = np.zeros((n, n))  # flow driven by the lid alone: J depends on the lid speed only
    with cnv.Adjoint(make_cfg(cnv, n), 9) as adj:
        _, gw, glid, errs = fd_check(cnv, adj, w0, 1.0, steps, [(np.zeros((n, n)), 1.0)])
    assert glid > 0 and errs[0] <= FD_RTOL


@pytest.mark.gpu
def test_checkpoint_interval_does_not_change_the_gradient(cnv):
    n, steps = 32, 45
    w0 = cnv.noise_field(n, seed=3, sigma=1.0, passes=2)
    ref = None
    for every in (1, 7, 45, 100):
        with cnv.Adjoint(make_cfg(cnv, n), every) as adj:
            J, gw, glid = adj.enstrophy_gradient(w0, 0.8, steps)
        if ref is None:
            ref = (J, gw, glid)
        else:
            assert J == ref[0] and glid == ref[2] and np.array_equal(gw, ref[1]), every


@pytest.mark.gpu
def test_adjoint_forward_is_the_direct_step(cnv):
    n, steps = 64, 12
    cfg = make_cfg(cnv, n, lid=1.3)
    w0 = cnv.noise_field(n, seed=11, sigma=0.5, passes=3)
    with cnv.Adjoint(cfg, 5) as adj:
        wT = adj.forward(w0, 1.3, steps)
    cfg.poisson_type = cnv.POISSON_DIRECT
    with cnv.Cavity(cfg) as cav:
        cav.set_fields(w=w0)
        cav.step(steps)
        w = cav.get_fields()[0]
    assert np.array_equal(wT, w)


@pytest.mark.gpu
def test_adjoint_forward_matches_converged_oracle(cnv, orc):
    n, steps, re, lid = 24, 10, 400.0, 0.9
    dt = stable_dt(n, re, lid)
    w0 = cnv.noise_field(n, seed=5, sigma=1.0, passes=2)
    p = orc.make_params(n, re=re, dt=dt, u_bc=(0.0, 0.0, 0.0, lid), itmax=2000000, tol=1e-14, exact_norm=0)
    W, U, V, PSI = orc.initial_state(n)
    W[...] = w0
    assert orc.run(p, steps, W, U, V, PSI)[0] == 0
    with cnv.Adjoint(make_cfg(cnv, n, re=re, lid=lid), 4) as adj:
        wT = adj.forward(w0, lid, steps)
    assert np.max(np.abs(wT - W)) <= ORACLE_TOL * np.max(np.abs(W))


@pytest.mark.gpu
def test_adjoint_gradient_matches_oracle_finite_differences(cnv, orc):
    # finite differences of the oracle's own step (the reference's algorithm, SOR converged to
    # rounding) against the GPU adjoint: ties the gradient to the reference's time step
    n, steps, re, lid = 16, 12, 400.0, 1.0
    dt = stable_dt(n, re, lid)
    w0 = cnv.noise_field(n, seed=9, sigma=1.0, passes=2)
    h2 = (1.0 / n) ** 2

    def oracle_J(w, l):
        p = orc.make_params(n, re=re, dt=dt, u_bc=(0.0, 0.0, 0.0, l), itmax=2000000, tol=1e-15, exact_norm=0)
        W, U, V, PSI = orc.initial_state(n)
        W[...] = w
        assert orc.run(p, steps, W, U, V, PSI)[0] == 0
        return 0.5 * h2 * float(np.sum(W * W))

    with cnv.Adjoint(make_cfg(cnv, n, re=re, lid=lid), 5) as adj:
        _, gw, glid = adj.enstrophy_gradient(w0, lid, steps)
    for d, dl in directions(n, 3, seed=21):
        fd = (oracle_J(w0 + FD_EPS * d, lid + FD_EPS * dl) - oracle_J(w0 - FD_EPS * d, lid - FD_EPS * dl)) / (2 * FD_EPS)
        ad = float(np.sum(gw * d)) + glid * dl
        assert abs(fd - ad) <= 1e-5 * abs(ad), (fd, ad)


@pytest.mark.gpu
def test_torch_autograd_function(cnv):
    torch = pytest.importorskip("torch")
    import cnv_torch

    n, steps = 32, 20
    w0n = cnv.noise_field(n, seed=13, sigma=1.0, passes=3)
    with cnv.Adjoint(make_cfg(cnv, n), 6) as adj:
        J_ref, gw_ref, glid_ref = adj.enstrophy_gradient(w0n, 1.0, steps)
        w0 = torch.tensor(w0n, dtype=torch.float64, device="cuda", requires_grad=True)
        lid = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
        wT = cnv_torch.CavityRollout.apply(w0, lid, adj, steps)
        J = cnv_torch.enstrophy(wT, adj.h2)
        J.backward()
    assert abs(J.item() - J_ref) <= 1e-14 * J_ref
    assert np.allclose(w0.grad.cpu().numpy(), gw_ref, rtol=0, atol=1e-15 * np.max(np.abs(gw_ref)))
    assert abs(lid.grad.item() - glid_ref) <= 1e-12 * abs(glid_ref)


@pytest.mark.gpu
def test_enstrophy_gradient_config_256(cnv):
    """The full workload: 256 x 256, Re 400, 2000 steps, checkpoints every 100, 16 directions."""
    n, steps = 256, 2000
    w0 = cnv.noise_field(n, seed=2025, sigma=1.0, passes=16)
    with cnv.Adjoint(make_cfg(cnv, n), 100) as adj:
        J, gw, glid, errs = fd_check(cnv, adj, w0, 1.0, steps, directions(n, 16, seed=2026))
        fwd_ms, bwd_ms, state_bytes = adj.stats()
    assert max(errs) <= FD_RTOL, errs
    assert fwd_ms + bwd_ms <= 4 * fwd_ms, (fwd_ms, bwd_ms)  # gradient at most 4x the forward cost


def _dense_model(orc, n, order=6, re=400.0, u_bc=(0.0, 0.0, 0.0), v_bc=(0.0, 0.0, 0.0, 0.0)):
    import adjoint  # oracle/adjoint.py

    return adjoint.DenseStep(n, order=order, re=re, dt=stable_dt(n, re), u_bc=u_bc, v_bc=v_bc)


@pytest.mark.parametrize("order", [2, 4, 6])
def test_dense_adjoint_matches_finite_differences(orc, order):
    # the adjoint equations themselves, on the CPU: dense restatement vs central differences
    n, steps, lid = 10, 8, 1.2
    model = _dense_model(orc, n, order=order, u_bc=(0.1, -0.2, 0.05), v_bc=(0.02, 0.0, -0.1, 0.3))
    rng = np.random.default_rng(order)
    w0 = np.zeros((n, n))
    w0[1:-1, 1:-1] = rng.standard_normal((n - 2, n - 2))
    J, gw, glid = model.enstrophy_gradient(w0, lid, steps)
    h2 = model.dx * model.dy
    Jf = lambda w, l: 0.5 * h2 * float(np.sum(model.run(w, l, steps)[0] ** 2))
    for d, dl in directions(n, 3, seed=order):
        fd = (Jf(w0 + FD_EPS * d, lid + FD_EPS * dl) - Jf(w0 - FD_EPS * d, lid - FD_EPS * dl)) / (2 * FD_EPS)
        ad = float(np.sum(gw * d)) + glid * dl
        assert abs(fd - ad) <= 1e-7 * abs(ad), (fd, ad)


@pytest.mark.gpu
@pytest.mark.parametrize("n,order", [(12, 6), (17, 4), (20, 2)])
def test_adjoint_kernels_match_dense_adjoint(cnv, orc, n, order):
    steps, lid = 15, 0.9
    u_bc, v_bc = (0.1, -0.2, 0.05), (0.02, 0.0, -0.1, 0.3)
    model = _dense_model(orc, n, order=order, u_bc=u_bc, v_bc=v_bc)
    w0 = cnv.noise_field(n, seed=n, sigma=1.0, passes=1)
    J_ref, gw_ref, glid_ref = model.enstrophy_gradient(w0, lid, steps)
    cfg = make_cfg(cnv, n, order=order)
    cfg.u1, cfg.u2, cfg.u3 = u_bc
    cfg.v1, cfg.v2, cfg.v3, cfg.v4 = v_bc
    with cnv.Adjoint(cfg, 4) as adj:
        J, gw, glid = adj.enstrophy_gradient(w0, lid, steps)
    assert abs(J - J_ref) <= 1e-12 * J_ref
    assert np.max(np.abs(gw - gw_ref)) <= 1e-10 * np.max(np.abs(gw_ref))
    assert abs(glid - glid_ref) <= 1e-10 * abs(glid_ref)


def test_adjoint_rejects_bad_arguments(cnv):
    cfg = cnv.default_config(nx=64, ny=32)
    with pytest.raises(cnv.CnvError) as e:
        cnv.Adjoint(cfg, 10)
    assert e.value.status == cnv.CNV_BAD_ARG
    with pytest.raises(cnv.CnvError) as e:
        cnv.Adjoint(cnv.default_config(nx=64, ny=64), 0)
    assert e.value.status == cnv.CNV_BAD_ARG


def test_noise_field_is_seeded_and_smoothed(cnv):
    a = cnv.noise_field(40, seed=1, sigma=2.0, passes=0)
    b = cnv.noise_field(40, seed=1, sigma=2.0, passes=0)
    c = cnv.noise_field(40, seed=2, sigma=2.0, passes=0)
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    assert 1.8 < a.std() < 2.2
    s = cnv.noise_field(40, seed=1, sigma=2.0, passes=8)
    assert np.array_equal(s[0], a[0]) and s[1:-1, 1:-1].std() < 0.5 * a.std()
