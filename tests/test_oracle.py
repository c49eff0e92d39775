"""The oracle is pinned before it is trusted.

1. Against the reference's shipped run logs (tests/golden/logs_kat.json, made by
   tests/golden/make_golden.py from output/logs/*.txt): every logged step's Poisson iteration
   count, stop norm and continuity max/min, as printed digits. Runs everywhere.
2. Against the unmodified reference code itself (oracle/_ref, compiled from the reference
   tree): fields bit for bit after several steps, for every FD order, both SOR orderings and
   Gauss-Seidel. Skipped where the reference tree is absent (the GPU machine).
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "logs_kat.json")


def _fmt(step):
    return dict(iters=step["iters"], err="%E" % step["err"], cont_max="%E" % step["cont_max"],
                cont_min="%E" % step["cont_min"])


@pytest.mark.parametrize("run", ["testRunNOOMP", "testRunOMP", "testRunNOOMPHIGHRES", "testRunOMPHIGHRES"])
def test_oracle_reproduces_shipped_logs(orc, run):
    spec = json.load(open(GOLDEN))[run]
    n = spec["n"]
    ordering = orc.ORDER_REDBLACK if spec["ordering"] == "redblack" else orc.ORDER_LEX
    p = orc.make_params(n, re=spec["re"], dt=spec["dt"], tol=spec["tol"], itmax=spec["itmax"],
                        ordering=ordering, exact_norm=1)
    w, u, v, psi = orc.initial_state(n)
    steps = spec["steps"]
    rc, got = orc.run(p, len(steps), w, u, v, psi)
    assert rc == 0
    for t, (a, b) in enumerate(zip(got, steps)):
        assert _fmt(a) == b, f"step {t}"


def test_fd_band_rejects_bad_order_and_size(orc):
    with pytest.raises(ValueError):
        orc.fd_band(16, 3, 1, 1 / 16)  # src/finitediff.c:148-152 exits on other orders
    with pytest.raises(ValueError):
        orc.fd_band(4, 6, 1, 1 / 4)  # order 6 writes D[2][4]: needs n >= 5
    orc.fd_band(5, 6, 2, 1 / 5)
    orc.fd_band(4, 4, 2, 1 / 4)


def test_fd_band_interior_stencil_values(orc):
    n, h = 32, 1 / 32
    b1 = orc.fd_band(n, 6, 1, h)
    b2 = orc.fd_band(n, 6, 2, h)
    # src/finitediff.c:126-132 and :263-269, evaluated as ((double)p / q) / h
    want1 = [-1 / 60 / h, 3 / 20 / h, -3 / 4 / h, 0 / h, 3 / 4 / h, -3 / 20 / h, 1 / 60 / h]
    want2 = [1 / 90 / (h * h), -3 / 20 / (h * h), 3 / 2 / (h * h), -49 / 18 / (h * h),
             3 / 2 / (h * h), -3 / 20 / (h * h), 1 / 90 / (h * h)]
    assert b1[10].tolist() == want1
    assert b2[10].tolist() == want2
    # first and last rows: one-sided first difference, 4-point second difference
    assert b1[0].tolist() == [0, 0, 0, -1 / h, 1 / h, 0, 0]
    assert b1[n - 1].tolist() == [0, 0, -1 / h, 1 / h, 0, 0, 0]
    assert b2[n - 1].tolist() == [-1 / (h * h), 4 / (h * h), -5 / (h * h), 2 / (h * h), 0, 0, 0]


ref_only = pytest.mark.skipif("not __import__('orc').ref_available()",
                              reason="reference tree not present (oracle/_ref not built)")


@ref_only
@pytest.mark.parametrize("n", [5, 6, 7, 8, 16, 33, 64])
@pytest.mark.parametrize("order", [2, 4, 6])
@pytest.mark.parametrize("deriv", [1, 2])
def test_band_equals_reference_dense_operator(orc, n, order, deriv):
    h = 1.0 / n
    band = orc.fd_band(n, order, deriv, h)
    dense = orc.ref_fd_dense(n, order, deriv, h)
    rebuilt = np.zeros((n, n))
    for r in range(n):
        for o in range(-3, 4):
            if 0 <= r + o < n:
                rebuilt[r, r + o] = band[r, o + 3]
    assert np.array_equal(rebuilt, dense)
    assert np.count_nonzero(dense) == np.count_nonzero(rebuilt)


@ref_only
@pytest.mark.parametrize("n,order,ptype,rb", [
    (16, 6, 2, 1), (32, 6, 2, 1), (33, 6, 2, 1), (32, 6, 2, 0), (32, 4, 2, 1),
    (16, 2, 2, 0), (32, 6, 1, 0), (64, 6, 2, 1), (24, 6, 2, 1),
])
def test_restatement_bitwise_equals_reference_steps(orc, n, order, ptype, rb):
    nsteps = 4
    (w, u, v, psi), rsteps = orc.ref_run(n, order=order, re=1000.0, dt=0.005, poisson_type=ptype,
                                         tol=1e-3, openmp=rb, nsteps=nsteps)
    p = orc.make_params(n, order=order, re=1000.0, dt=0.005, poisson_type=ptype, ordering=rb,
                        tol=1e-3, exact_norm=1)
    W, U, V, PSI = orc.initial_state(n)
    rc, osteps = orc.run(p, nsteps, W, U, V, PSI)
    assert rc == 0
    for a, b in [(w, W), (u, U), (v, V), (psi, PSI)]:
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
    for a, b in zip(rsteps, osteps):
        assert a["iters"] == b["iters"]
        assert "%E" % a["err"] == "%E" % b["err"]
        assert a["cont_max"] == b["cont_max"] and a["cont_min"] == b["cont_min"]


@ref_only
def test_restatement_nonzero_lid_and_side_walls(orc):
    """All eight velocity BCs non-zero and Lx != Ly (dx != dy) exercise every BC branch."""
    n = 24
    ubc, vbc = (0.1, -0.2, 0.3, 1.0), (0.05, -0.05, 0.02, -0.03)
    (w, u, v, psi), rsteps = orc.ref_run(n, Lx=2, Ly=1, re=400.0, dt=0.001, u_bc=ubc, v_bc=vbc,
                                         tol=1e-6, openmp=1, nsteps=3)
    p = orc.make_params(n, Lx=2, Ly=1, re=400.0, dt=0.001, u_bc=ubc, v_bc=vbc, tol=1e-6, exact_norm=1)
    W, U, V, PSI = orc.initial_state(n)
    orc.run(p, 3, W, U, V, PSI)
    for a, b in [(w, W), (u, U), (v, V), (psi, PSI)]:
        assert np.array_equal(a, b)
