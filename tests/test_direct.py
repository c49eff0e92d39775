"""CNV_POISSON_DIRECT: the exact sine-transform solve of the reference's discrete Poisson equation.

It must give the answer the reference's SOR converges to: the oracle's red-black SOR run to a
stop norm near rounding (sum|dpsi| < 1e-15 for one solve, < 1e-13 in time steps) is the check, to 1e-11 normwise
relative for a solve and 1e-10 for whole time steps. It must also beat the FP64 SOR path's own
error against that converged answer by orders of magnitude. On grids too large for the oracle's
SOR it must match the sine-transform solve psi = S((S R S) ./ Lambda) S done densely in numpy FP64,
with the eigenvalues as sums of squared sines (accurate to a few units of rounding against an
extended-precision solve), to 1e-13, on both of its row-transform paths: the FFT (2(n-1) has only
prime factors up to 251) and the dense products (n = 258: 2 * 257). The eigenvalues written as
den - 2 dy^2 cos - 2 dx^2 cos instead lose accuracy as n grows (about 2e-12 at n = 1024).
"""
from __future__ import annotations

import numpy as np
import pytest

SOLVE_TOL = 1e-11   # direct solve vs converged oracle SOR, normwise relative
STEP_TOL = 1e-10    # fields after several steps
DENSE_TOL = 1e-13   # direct solve vs the dense sine-transform solve in numpy


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.gpu
@pytest.mark.parametrize("n", [5, 17, 64, 130])
def test_direct_solve_matches_converged_sor(cnv, orc, n):
    rng = np.random.default_rng(n)
    f = rng.standard_normal((n, n))
    p = orc.make_params(n, itmax=2000000, tol=1e-15 * n * n / 256, exact_norm=0)
    want, it, err, rc = orc.poisson(p, f)
    assert rc == 0
    cfg = cnv.default_config(nx=n, ny=n, poisson_type=cnv.POISSON_DIRECT)
    with cnv.Cavity(cfg) as cav:
        rc, got, iters, e = cav.poisson(f)
    assert rc == 0 and iters == 0 and e == 0.0
    assert np.all(got[0] == 0) and np.all(got[-1] == 0) and np.all(got[:, 0] == 0) and np.all(got[:, -1] == 0)
    assert _rel(got, want) <= SOLVE_TOL


def _dense_sine_solve(f, dx, dy):
    """psi for the reference's right-hand side f (the equation den psi - dy^2 (psi_i+1 + psi_i-1)
    - dx^2 (psi_j+1 + psi_j-1) = -c4 f on the interior, psi = 0 on the edge) by four dense
    products with the orthonormal DST-I matrix, in numpy FP64; the eigenvalues
    4 dy^2 sin^2(pi a / 2(m+1)) + 4 dx^2 sin^2(pi b / 2(m+1))."""
    n = f.shape[0]
    m = n - 2
    k = np.arange(1, m + 1)
    arg = np.outer(k, k) % (2 * (m + 1))  # exact argument reduction
    S = np.sqrt(2.0 / (m + 1)) * np.sin(np.pi * arg / (m + 1))
    sk = np.sin(np.pi * k / (2 * (m + 1)))
    lam = 4 * dy * dy * (sk * sk)[:, None] + 4 * dx * dx * (sk * sk)[None, :]
    R = -(dx * dx * dy * dy) * f[1:-1, 1:-1]
    out = np.zeros_like(f)
    out[1:-1, 1:-1] = S @ ((S @ R @ S) / lam) @ S
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("n,L", [(37, 1), (96, 2), (258, 1), (1024, 1)])
def test_direct_solve_matches_dense_sine_transform_solve(cnv, n, L):
    rng = np.random.default_rng(n + 7)
    f = rng.standard_normal((n, n))
    cfg = cnv.default_config(nx=n, ny=n, Lx=L, Ly=1, poisson_type=cnv.POISSON_DIRECT)
    with cnv.Cavity(cfg) as cav:
        rc, got, _, _ = cav.poisson(f)
    assert rc == 0
    want = _dense_sine_solve(f, L / n, 1.0 / n)
    assert _rel(got, want) <= DENSE_TOL


@pytest.mark.gpu
def test_direct_solve_unequal_spacing(cnv, orc):
    n = 48
    rng = np.random.default_rng(1)
    f = rng.standard_normal((n, n))
    p = orc.make_params(n, Lx=2, Ly=1, itmax=2000000, tol=1e-14, exact_norm=0)
    want, _, _, rc = orc.poisson(p, f)
    assert rc == 0
    cfg = cnv.default_config(nx=n, ny=n, Lx=2, Ly=1, poisson_type=cnv.POISSON_DIRECT)
    with cnv.Cavity(cfg) as cav:
        rc, got, _, _ = cav.poisson(f)
    assert rc == 0 and _rel(got, want) <= SOLVE_TOL


@pytest.mark.gpu
@pytest.mark.parametrize("n,order", [(32, 6), (41, 4), (64, 2)])
def test_direct_steps_match_converged_oracle(cnv, orc, n, order):
    h = 1.0 / n
    dt = 0.2 * min(h * h * 400 / 4, h)
    steps = 6
    p = orc.make_params(n, order=order, re=400.0, dt=dt, itmax=2000000, tol=1e-13, exact_norm=0)
    W, U, V, PSI = orc.initial_state(n)
    rc, _ = orc.run(p, steps, W, U, V, PSI)
    assert rc == 0
    cfg = cnv.default_config(nx=n, ny=n, order=order, Re=400.0, dt=dt, poisson_type=cnv.POISSON_DIRECT)
    with cnv.Cavity(cfg) as cav:
        _, info = cav.step(steps)
        w, u, v, psi = cav.get_fields()
    assert all(r["iters"] == 0 and r["status"] == 0 for r in info)
    for name, a, b in zip("w u v psi".split(), (w, u, v, psi), (W, U, V, PSI)):
        assert _rel(a, b) <= STEP_TOL, name


@pytest.mark.gpu
def test_direct_is_closer_to_converged_answer_than_sor_1e6(cnv, orc):
    # the reference's stop rule (sum|dpsi| < 1e-6) leaves an error the direct solve does not have
    n = 128
    h = 1.0 / n
    dt = 0.2 * min(h * h * 1000 / 4, h)
    p = orc.make_params(n, re=1000.0, dt=dt, itmax=5000000, tol=1e-13, threads=4, exact_norm=0)
    W, U, V, PSI = orc.initial_state(n)
    assert orc.run(p, 3, W, U, V, PSI)[0] == 0
    errs = {}
    for name, ptype in (("sor", cnv.POISSON_SOR), ("direct", cnv.POISSON_DIRECT)):
        cfg = cnv.default_config(nx=n, ny=n, Re=1000.0, dt=dt, poisson_type=ptype, poisson_tol=1e-6,
                                 poisson_max_it=1000000)
        with cnv.Cavity(cfg) as cav:
            cav.step(3)
            errs[name] = _rel(cav.get_fields()[3], PSI)
    assert errs["direct"] <= STEP_TOL
    assert errs["direct"] * 1e3 < errs["sor"], errs


def test_direct_rejects_mixed_precision(cnv):
    # argument checks run before any device call
    cfg = cnv.default_config(nx=64, ny=64, poisson_type=cnv.POISSON_DIRECT, precision=cnv.PREC_MIXED)
    with pytest.raises(cnv.CnvError) as e:
        cnv.Cavity(cfg)
    assert e.value.status == cnv.CNV_BAD_ARG
