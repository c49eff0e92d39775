"""CUDA path vs the CPU oracle, through the C ABI of libcnv.

Both FP64 SOR/GS kernels are checked where it matters (sor_blocking = 1: border exchange every
half-sweep; 2 or 4: that many sweeps per exchange on shared-memory tiles, grids with
n - 2 >= 2 * sweeps).

Tolerances: the FP64 path with reference arithmetic (precision = fp64) must match the oracle
bit for bit on every field (same operation order, round-to-nearest, no FMA contraction);
iteration counts must be equal; the stop norm is summed in a different order on the GPU, so it
is compared to 1e-12 relative. The FMA form must agree to 1e-10 normwise relative
(max|a-b| / max|b|) per field, well inside the 1e-8 relative bound the FMA form is held to.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "logs_kat.json")
REL_ERR_TOL = 1e-12       # stop norm, GPU vs oracle (different summation order)
FMA_FIELD_TOL = 1e-10     # FMA form, normwise relative per field


def make_cfg(cnv, n, **kw):
    base = dict(nx=n, ny=n, Re=1000.0, dt=0.005, poisson_tol=1e-3, poisson_max_it=10000, order=6)
    base.update(kw)
    return cnv.default_config(**base)


def oracle_params(orc, cfg, ordering=1):
    return orc.make_params(cfg.nx, order=cfg.order, Lx=cfg.Lx, Ly=cfg.Ly, re=cfg.Re, dt=cfg.dt,
                           u_bc=(cfg.u1, cfg.u2, cfg.u3, cfg.u4), v_bc=(cfg.v1, cfg.v2, cfg.v3, cfg.v4),
                           poisson_type=cfg.poisson_type, ordering=ordering,
                           beta=(cfg.sor_omega if cfg.sor_omega > 0 else None), itmax=cfg.poisson_max_it,
                           tol=cfg.poisson_tol, threads=0, exact_norm=0)


BLOCKING = [1, 2, 4]


def blocking_ok(n, blocking):
    return blocking == 1 or n - 2 >= 2 * blocking


def bitwise(a, b):
    return np.array_equal(np.asarray(a).view(np.uint64), np.asarray(b).view(np.uint64))


def run_both(cnv, orc, cfg, nsteps):
    with cnv.Cavity(cfg) as cav:
        rc, gsteps = cav.step(nsteps)
        gw, gu, gv, gpsi = cav.get_fields()
    p = oracle_params(orc, cfg)
    w, u, v, psi = orc.initial_state(cfg.nx, cfg.ui, cfg.vi)
    orc_rc, osteps = orc.run(p, nsteps, w, u, v, psi)
    assert rc == 0 and orc_rc == 0
    return (gw, gu, gv, gpsi), gsteps, (w, u, v, psi), osteps


@pytest.mark.parametrize("blocking", BLOCKING)
@pytest.mark.parametrize("n,order", [(7, 6), (8, 6), (16, 6), (33, 6), (64, 6), (32, 4), (32, 2), (5, 6), (4, 4)])
def test_step_bitwise_equals_oracle(cnv, orc, n, order, blocking):
    if not blocking_ok(n, blocking):
        pytest.skip("grid smaller than one shared-memory tile")
    cfg = make_cfg(cnv, n, order=order, sor_blocking=blocking)
    g, gs, o, os_ = run_both(cnv, orc, cfg, 6)
    for name, a, b in zip("w u v psi".split(), g, o):
        assert bitwise(a, b), f"{name} differs: max abs {np.max(np.abs(a - b))}"
    for a, b in zip(gs, os_):
        assert a["iters"] == b["iters"]
        assert abs(a["err"] - b["err"]) <= REL_ERR_TOL * abs(b["err"])
        assert bitwise(a["cont_max"], b["cont_max"]) and bitwise(a["cont_min"], b["cont_min"])


@pytest.mark.parametrize("blocking", BLOCKING)
@pytest.mark.parametrize("n,blocks", [(64, 4), (64, 16), (64, 37), (64, 152), (50, 9), (130, 304), (31, 6),
                                      (100, 7), (200, 60)])
def test_step_bitwise_with_forced_tilings(cnv, orc, n, blocks, blocking):
    """Many solver tiles on small grids: every tile frame, halo and neighbour wait is exercised
    (the shared-memory kernel lowers the block count until tiles are at least 8 cells wide)."""
    cfg = make_cfg(cnv, n, solver_blocks=blocks, poisson_tol=1e-6, sor_blocking=blocking)
    g, gs, o, os_ = run_both(cnv, orc, cfg, 4)
    for name, a, b in zip("w u v psi".split(), g, o):
        assert bitwise(a, b), f"{name} differs: max abs {np.max(np.abs(a - b))}"
    assert [s["iters"] for s in gs] == [s["iters"] for s in os_]


@pytest.mark.parametrize("ptype,blocking", [(1, 1), (1, 2), (1, 4), (3, 1)])
def test_gs_and_jacobi_steps_with_tiles(cnv, orc, ptype, blocking):
    cfg = make_cfg(cnv, 48, poisson_type=ptype, solver_blocks=12, poisson_tol=1e-5, poisson_max_it=100000,
                   sor_blocking=blocking)
    g, gs, o, os_ = run_both(cnv, orc, cfg, 3)
    for name, a, b in zip("w u v psi".split(), g, o):
        assert bitwise(a, b), name


@pytest.mark.parametrize("blocking", BLOCKING)
def test_step_all_boundary_values_and_rectangular_spacing(cnv, orc, blocking):
    cfg = make_cfg(cnv, 24, Lx=2, Ly=1, Re=400.0, dt=0.001, poisson_tol=1e-6, u1=0.1, u2=-0.2, u3=0.3,
                   u4=1.0, v1=0.05, v2=-0.05, v3=0.02, v4=-0.03, ui=0.01, vi=-0.02, sor_blocking=blocking)
    g, gs, o, os_ = run_both(cnv, orc, cfg, 4)
    for a, b in zip(g, o):
        assert bitwise(a, b)


@pytest.mark.parametrize("run", ["testRunOMP", "testRunOMPHIGHRES"])
def test_gpu_reproduces_shipped_redblack_logs(cnv, run):
    """The reference's own red-black run logs, every logged step, printed digits."""
    spec = json.load(open(GOLDEN))[run]
    n = spec["n"]
    cfg = make_cfg(cnv, n, Re=spec["re"], dt=spec["dt"], poisson_tol=spec["tol"], poisson_max_it=spec["itmax"])
    steps = spec["steps"]
    with cnv.Cavity(cfg) as cav:
        rc, got = cav.step(len(steps))
    assert rc == 0
    for t, (a, b) in enumerate(zip(got, steps)):
        assert a["iters"] == b["iters"], f"step {t}"
        assert "%E" % a["err"] == b["err"], f"step {t}"
        assert "%E" % a["cont_max"] == b["cont_max"] and "%E" % a["cont_min"] == b["cont_min"], f"step {t}"


def test_config1_64_re100_sor15(cnv, orc):
    """The CPU workload: 64^2, Re 100, dt 1e-3, SOR beta 1.5, tol 1e-6 (first 20 of its 1000 steps)."""
    cfg = make_cfg(cnv, 64, Re=100.0, dt=1e-3, poisson_tol=1e-6, sor_omega=1.5)
    g, gs, o, os_ = run_both(cnv, orc, cfg, 20)
    for a, b in zip(g, o):
        assert bitwise(a, b)
    assert [s["iters"] for s in gs] == [s["iters"] for s in os_]


def test_config1_all_1000_steps(cnv, orc):
    """The whole CPU workload (64^2, Re 100, dt 1e-3, SOR beta 1.5, tol 1e-6, tf = 1 -> 1000
    steps, about 1.7 M SOR sweeps): every step's iteration count equal to the oracle's and the
    fields after the last step equal bit for bit."""
    steps = 1000
    cfg = make_cfg(cnv, 64, Re=100.0, dt=1e-3, poisson_tol=1e-6, sor_omega=1.5)
    g, gs, o, os_ = run_both(cnv, orc, cfg, steps)
    assert len(gs) == len(os_) == steps
    assert [s["iters"] for s in gs] == [s["iters"] for s in os_]
    for name, a, b in zip("w u v psi".split(), g, o):
        assert bitwise(a, b), f"{name} differs: max abs {np.max(np.abs(a - b))}"


@pytest.mark.parametrize("ptype,blocking", [(1, 1), (2, 1), (3, 1), (1, 2), (2, 2), (1, 4), (2, 4)])
@pytest.mark.parametrize("n", [16, 37, 96])
def test_poisson_alone_matches_oracle(cnv, orc, ptype, n, blocking):
    rng = np.random.default_rng(n * 10 + ptype)
    f = rng.standard_normal((n, n))
    cfg = make_cfg(cnv, n, poisson_type=ptype, poisson_tol=1e-9, poisson_max_it=200000, sor_blocking=blocking)
    with cnv.Cavity(cfg) as cav:
        rc, psi, it, err = cav.poisson(f)
        sweeps, ms, poisson_ms = cav.stats()  # the standalone solve's sweeps and kernel time
    p = oracle_params(orc, cfg)
    opsi, oit, oerr, orc_rc = orc.poisson(p, f)
    assert rc == 0 and orc_rc == 0
    assert it == oit
    assert sweeps == it + 1 and poisson_ms > 0
    assert bitwise(psi, opsi)
    assert abs(err - oerr) <= REL_ERR_TOL * oerr


@pytest.mark.parametrize("blocking", BLOCKING)
@pytest.mark.parametrize("n", [64, 100, 128])
def test_fma_form_within_tolerance(cnv, orc, n, blocking):
    cfg = make_cfg(cnv, n, precision=1, poisson_tol=1e-8, sor_blocking=blocking)
    g, gs, o, os_ = run_both(cnv, orc, cfg, 5)
    for name, a, b in zip("w u v psi".split(), g, o):
        scale = max(np.max(np.abs(b)), 1e-300)
        assert np.max(np.abs(a - b)) / scale <= FMA_FIELD_TOL, name
    for a, b in zip(gs, os_):
        assert abs(a["iters"] - b["iters"]) <= 1


@pytest.mark.parametrize("blocking", BLOCKING)
def test_1024_single_step_matches_oracle(cnv, orc, blocking):
    """The benchmark workload's grid (1024^2, Re 1000, dt by the stability rule, tol 1e-6), step 0."""
    n = 1024
    h = 1.0 / n
    dt = 0.2 * min(h * h * 1000.0 / 4, h / 1.0)
    cfg = make_cfg(cnv, n, Re=1000.0, dt=dt, poisson_tol=1e-6, poisson_max_it=100000, sor_blocking=blocking)
    g, gs, o, os_ = run_both(cnv, orc, cfg, 1)
    for name, a, b in zip("w u v psi".split(), g, o):
        assert bitwise(a, b), name
    assert gs[0]["iters"] == os_[0]["iters"]


def test_1024_four_steps_match_oracle(cnv, orc):
    """The benchmark workload with its default solver, 4 steps (about 9,600 SOR sweeps): fields bit
    for bit and every step's iteration count, against the oracle run on all host cores with its
    exact (order-free) stop norm, the same sum the GPU forms."""
    n = 1024
    h = 1.0 / n
    dt = 0.2 * min(h * h * 1000.0 / 4, h / 1.0)
    cfg = make_cfg(cnv, n, Re=1000.0, dt=dt, poisson_tol=1e-6, poisson_max_it=100000)
    with cnv.Cavity(cfg) as cav:
        rc, gsteps = cav.step(4)
        g = cav.get_fields()
    assert rc == 0
    p = orc.make_params(n, order=cfg.order, re=cfg.Re, dt=cfg.dt, tol=cfg.poisson_tol, itmax=cfg.poisson_max_it,
                        threads=os.cpu_count() or 1, exact_norm=1)
    w, u, v, psi = orc.initial_state(n)
    orc_rc, osteps = orc.run(p, 4, w, u, v, psi)
    assert orc_rc == 0
    assert [s["iters"] for s in gsteps] == [s["iters"] for s in osteps]
    for name, a, b in zip("w u v psi".split(), g, (w, u, v, psi)):
        assert bitwise(a, b), name


def test_1024_fifty_steps_match_oracle(cnv, orc):
    """The benchmark workload for 50 steps (about 125,000 SOR sweeps, into the range the
    benchmark times): every step's iteration count, continuity max and min, and the final fields
    bit for bit, against the oracle on all host cores (its parallel row-sum stop norm; the GPU's
    is order-free, and the two could differ only at a tie of the norm with tol within rounding)."""
    n, steps = 1024, 50
    h = 1.0 / n
    dt = 0.2 * min(h * h * 1000.0 / 4, h / 1.0)
    cfg = make_cfg(cnv, n, Re=1000.0, dt=dt, poisson_tol=1e-6, poisson_max_it=100000)
    with cnv.Cavity(cfg) as cav:
        rc, gsteps = cav.step(steps)
        g = cav.get_fields()
    assert rc == 0
    p = orc.make_params(n, order=cfg.order, re=cfg.Re, dt=cfg.dt, tol=cfg.poisson_tol, itmax=cfg.poisson_max_it,
                        threads=os.cpu_count() or 1, exact_norm=0)
    w, u, v, psi = orc.initial_state(n)
    orc_rc, osteps = orc.run(p, steps, w, u, v, psi)
    assert orc_rc == 0
    assert [s["iters"] for s in gsteps] == [s["iters"] for s in osteps]
    for a, b in zip(gsteps, osteps):
        assert a["cont_max"] == b["cont_max"] and a["cont_min"] == b["cont_min"]
    for name, a, b in zip("w u v psi".split(), g, (w, u, v, psi)):
        assert bitwise(a, b), name


@pytest.mark.parametrize("blocking", [1, 4])
@pytest.mark.parametrize("ptype", [1, 2])
def test_poisson_with_streamfunction_beyond_2_46(cnv, orc, ptype, blocking):
    """A right-hand side scaled by 2^70 drives |psi| far past 2^46, where the stop norm's cells
    leave the fixed-point sum for its FP64 part. Scaling by a power of two is exact in every
    operation of the update, so the solve must give exactly 2^70 times the unscaled iterates:
    the same sweep count (tol scaled too) and psi bit for bit; and it must equal the oracle,
    which sums the norm in FP64 throughout, as the reference does."""
    n = 64
    scale = 2.0 ** 70
    rng = np.random.default_rng(4646 + ptype)
    f = rng.standard_normal((n, n))
    tol = 1e-9
    out = []
    for s in (1.0, scale):
        cfg = make_cfg(cnv, n, poisson_type=ptype, poisson_tol=tol * s, poisson_max_it=200000, sor_blocking=blocking)
        with cnv.Cavity(cfg) as cav:
            out.append(cav.poisson(f * s))
    (rc_a, psi_a, it_a, err_a), (rc_b, psi_b, it_b, err_b) = out
    assert rc_a == 0 and rc_b == 0, (rc_a, rc_b)
    assert np.max(np.abs(psi_b)) >= 2.0 ** 46
    assert it_b == it_a
    assert bitwise(psi_b, psi_a * scale)
    assert abs(err_b - err_a * scale) <= REL_ERR_TOL * err_a * scale
    p = oracle_params(orc, make_cfg(cnv, n, poisson_type=ptype, poisson_tol=tol * scale, poisson_max_it=200000))
    opsi, oit, oerr, orc_rc = orc.poisson(p, f * scale)
    assert orc_rc == 0 and oit == it_b
    assert bitwise(psi_b, opsi)
    assert abs(err_b - oerr) <= REL_ERR_TOL * oerr


# ------------------------------------------------------------------------- failure paths
@pytest.mark.parametrize("kind", [2, 3], ids=["sor", "jacobi"])
def test_stalled_block_times_out_and_device_stays_usable(cnv, kind):
    """A solver block that never raises its progress flags (the test hook test_stall_block):
    its neighbours' bounded waits run out after solver_timeout_ms, every block leaves through the
    same barrier sequence, the step reports CNV_TIMEOUT, and the device runs the next solve."""
    import time

    cfg = make_cfg(cnv, 256, poisson_type=kind, sor_blocking=1, solver_blocks=16, poisson_tol=1e-12,
                   poisson_max_it=200000, solver_timeout_ms=50, test_stall_block=1 + 5)
    with cnv.Cavity(cfg) as cav:
        t0 = time.perf_counter()
        rc, steps = cav.step(1, raise_on_error=False)
        elapsed = time.perf_counter() - t0
    assert rc == cnv.CNV_TIMEOUT, rc
    assert elapsed < 30, elapsed
    with cnv.Cavity(make_cfg(cnv, 64, poisson_type=kind, sor_blocking=1, solver_blocks=4)) as cav:
        rc, steps = cav.step(2)
    assert rc == 0 and all(s["status"] == 0 for s in steps)
@pytest.mark.parametrize("blocking", BLOCKING)
@pytest.mark.parametrize("itmax", [2, 9])
def test_itmax_reports_not_converged_and_stops(cnv, blocking, itmax):
    cfg = make_cfg(cnv, 32, poisson_max_it=itmax, poisson_tol=1e-12, sor_blocking=blocking)
    with cnv.Cavity(cfg) as cav:
        rc, steps = cav.step(3, raise_on_error=False)
    assert rc == cnv.CNV_NOT_CONVERGED
    assert steps[0]["status"] == cnv.CNV_NOT_CONVERGED and steps[0]["iters"] == itmax


@pytest.mark.parametrize("blocking", BLOCKING)
@pytest.mark.parametrize("tol", [1e3, 1e-1, 2e-3])
def test_early_convergence_matches_oracle(cnv, orc, blocking, tol):
    """Loose tolerances stop in the first sweeps (the shared-memory kernel then replays its first
    epoch from zero) and at every position inside an epoch."""
    rng = np.random.default_rng(7)
    n = 40
    f = rng.standard_normal((n, n))
    cfg = make_cfg(cnv, n, poisson_tol=tol, sor_blocking=blocking)
    with cnv.Cavity(cfg) as cav:
        rc, psi, it, err = cav.poisson(f)
    opsi, oit, oerr, orc_rc = orc.poisson(oracle_params(orc, cfg), f)
    assert rc == 0 and orc_rc == 0 and it == oit
    assert bitwise(psi, opsi)


def test_blocking_flag_checks(cnv):
    # argument checks need no GPU work: an unknown value, or blocking with a solver it cannot run
    for kw in (dict(sor_blocking=3), dict(sor_blocking=4, poisson_type=3), dict(sor_blocking=4, nx=8, ny=8)):
        with pytest.raises(cnv.CnvError) as e:
            cnv.Cavity(make_cfg(cnv, kw.pop("nx", 32), **kw))
        assert e.value.status == cnv.CNV_BAD_ARG


@pytest.mark.parametrize("n,kw,want", [
    (256, {}, "sor-tiled sweeps=4"),                       # the tiled kernel below 300^2
    (320, {}, "sor-tiled sweeps=2"),                       # two sweeps per exchange from 300^2
    (352, {}, "sor-exchange"),                             # the exchange kernel from 336^2
    (512, {}, "sor-exchange grid=152 tiles=8x19"),         # one block per SM (not 127 strips)
    (1024, {}, "sor-exchange grid=152 tiles=8x19"),        # one block of 1024 threads per SM
    (2048, {}, "sor-exchange grid=152 tiles=8x19"),
    (1024, {"precision": 2}, "mixed grid=152"),
    (256, {"poisson_type": 4}, "direct-sine-transform"),
    (256, {"sor_blocking": 1}, "sor-exchange"),
])
def test_solver_choice_and_geometry(cnv, n, kw, want):
    """cnv_solver_info names the solver a state picked; the defaults follow the measured
    crossovers (tiled kernel below 336^2, then one block per SM)."""
    with cnv.Cavity(make_cfg(cnv, n, **kw)) as cav:
        info = cav.solver_info()
    assert info.startswith(want), info


def test_nonfinite_input_rejected(cnv):
    cfg = make_cfg(cnv, 16)
    with cnv.Cavity(cfg) as cav:
        before = cav.get_fields()
        w = np.zeros((16, 16))
        w[3, 4] = np.nan
        assert cav.set_fields(w=w) == cnv.CNV_NONFINITE
        w[3, 4] = np.inf
        assert cav.set_fields(w=w) == cnv.CNV_NONFINITE
        # a finite field next to a non-finite one is not applied either: the state is untouched
        v = np.zeros((16, 16))
        v[0, 0] = -np.inf
        assert cav.set_fields(u=np.full((16, 16), 0.5), v=v) == cnv.CNV_NONFINITE
        for a, b in zip(cav.get_fields(), before):
            assert bitwise(a, b)
        # the standalone solve rejects a non-finite right-hand side before solving
        f = np.ones((16, 16))
        f[5, 5] = np.nan
        assert cav.poisson(f)[0] == cnv.CNV_NONFINITE
        rc, steps = cav.step(1)
        assert rc == 0


def test_time_passes_leaves_the_next_step_unchanged(cnv):
    """cnv_time_passes replays the pre- and post-solve passes on the current fields; the following
    step must give the same bits as without that call."""
    out = []
    for timed in (False, True):
        cfg = make_cfg(cnv, 96, poisson_tol=1e-6)
        with cnv.Cavity(cfg) as cav:
            cav.step(2)
            if timed:
                pre_ms, post_ms = cav.time_passes(5)
                assert pre_ms > 0 and post_ms > 0
            rc, info = cav.step(2)
            assert rc == 0
            out.append(([s["iters"] for s in info], cav.get_fields()))
    assert out[0][0] == out[1][0]
    for name, a, b in zip("w u v psi".split(), out[0][1], out[1][1]):
        assert bitwise(a, b), name


def test_step_rows_matches_step(cnv):
    n = 20
    cfg = make_cfg(cnv, n)
    with cnv.Cavity(cfg) as a:
        a.step(3)
        ref = a.get_fields()
    with cnv.Cavity(cfg) as b:
        w, u, v, psi = b.get_fields()
        for _ in range(3):
            rc, info = b.step_rows(w, u, v, psi)
            assert rc == 0
    for x, y in zip(ref, (w, u, v, psi)):
        assert bitwise(x, y)


def test_reset_and_repeat_is_deterministic(cnv):
    cfg = make_cfg(cnv, 48)
    with cnv.Cavity(cfg) as cav:
        _, s1 = cav.step(4)
        f1 = cav.get_fields()
        cav.reset()
        _, s2 = cav.step(4)
        f2 = cav.get_fields()
    assert s1 == s2
    for a, b in zip(f1, f2):
        assert bitwise(a, b)


# ----------------------------------------------------------------------- mixed precision
def fp64_residual(psi, f, Lx=1, Ly=1):
    """||g - A psi||_2 / ||g||_2 over the interior, g = dx^2 dy^2 f (the reference's scaling)."""
    n = psi.shape[0]
    dx, dy = Lx / n, Ly / n
    c4 = dx * dx * dy * dy
    den = 2 * (dx * dx + dy * dy)
    P = psi
    ap = (dy * dy * (P[2:, 1:-1] + P[:-2, 1:-1]) + dx * dx * (P[1:-1, 2:] + P[1:-1, :-2])
          - den * P[1:-1, 1:-1])
    g = c4 * f[1:-1, 1:-1]
    return np.linalg.norm(g - ap) / np.linalg.norm(g)


MIXED_RTOL = 1e-10        # the mixed form's stop rule (relative FP64 residual)
MIXED_FIELD_TOL = 1e-7    # mixed vs tightly converged FP64, normwise relative per field


@pytest.mark.parametrize("n", [24, 64, 96, 256, 1024])
def test_mixed_poisson_reaches_fp64_residual(cnv, orc, n):
    rng = np.random.default_rng(n)
    f = rng.standard_normal((n, n))
    cfg = make_cfg(cnv, n, precision=cnv.PREC_MIXED, mixed_rtol=MIXED_RTOL)
    with cnv.Cavity(cfg) as cav:
        rc, psi, outer, rel = cav.poisson(f)
    assert rc == 0, rel
    assert rel <= MIXED_RTOL
    assert fp64_residual(psi, f) <= 1.05 * MIXED_RTOL  # independent FP64 check of the iterate
    assert np.all(psi[0, :] == 0) and np.all(psi[-1, :] == 0) and np.all(psi[:, 0] == 0) and np.all(psi[:, -1] == 0)
    if n <= 256:
        p = oracle_params(orc, cfg)
        p.poisson_type, p.tol, p.itmax = 2, 1e-13 * n * n, 10_000_000
        opsi, _, _, orc_rc = orc.poisson(p, f)
        assert orc_rc == 0
        assert np.max(np.abs(psi - opsi)) <= MIXED_FIELD_TOL * np.max(np.abs(opsi))


@pytest.mark.parametrize("n", [64, 128])
@pytest.mark.parametrize("warm", [0, 1])
def test_mixed_steps_match_fp64_fields(cnv, orc, n, warm):
    """Time steps with the mixed solve (zero start or warm start from the previous step's psi)
    against the FP64 oracle run to a tight tolerance."""
    cfg = make_cfg(cnv, n, precision=cnv.PREC_MIXED, mixed_rtol=MIXED_RTOL, dt=0.001, mixed_warm_start=warm)
    with cnv.Cavity(cfg) as cav:
        rc, steps = cav.step(5)
        g = cav.get_fields()
    assert rc == 0 and all(s["err"] <= MIXED_RTOL for s in steps)
    p = oracle_params(orc, cfg)
    p.tol = 1e-13 * n * n
    p.itmax = 10_000_000
    w, u, v, psi = orc.initial_state(n)
    orc.run(p, 5, w, u, v, psi)
    for name, a, b in zip("w u v psi".split(), g, (w, u, v, psi)):
        assert np.max(np.abs(a - b)) <= MIXED_FIELD_TOL * np.max(np.abs(b)), name


def test_mixed_warm_start_needs_fewer_corrections(cnv):
    # a slowly changing flow (tiny dt on a smooth noise field): the previous step's psi is
    # already close, so the warm start needs fewer FP64 corrections to the same residual
    n = 128
    counts = {}
    for warm in (0, 1):
        cfg = make_cfg(cnv, n, precision=cnv.PREC_MIXED, mixed_rtol=MIXED_RTOL, dt=1e-7, mixed_warm_start=warm,
                       init_field=cnv.INIT_NOISE, init_sigma=1.0, init_smooth_passes=8, seed=3)
        with cnv.Cavity(cfg) as cav:
            rc, steps = cav.step(6)
        assert rc == 0
        counts[warm] = sum(s["iters"] for s in steps[1:])
    assert counts[1] < counts[0], counts


def test_fp64_probe_reports_device_rates(cnv):
    """cnv_probe_fp64: positive rates of the right order for a GB300-class part (FP64 is
    about 1/60 of FP32 there: 1e11-1e13 operations per second), FMA chains not slower than
    multiply-then-add chains by more than rounding of the timing."""
    add_mul, fma_rate = cnv.probe_fp64(0)
    assert 1e11 < add_mul < 1e13 and 1e11 < fma_rate < 1e13
    assert fma_rate > 0.5 * add_mul
