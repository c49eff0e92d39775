"""Out-of-bounds writes, checked without a sanitizer: guard cells around every buffer.

With the testing-only config field test_guard_cells, every field and work buffer of a cavity
(w, u, v, psi, the split-layout solver arrays, the mixed form's FP32 arrays, the tiled solver's
snapshots, the reduction partials, ...) sits between two 4 KB regions of 0xFF bytes, a NaN in
every lane width, and the library compares them after each step and Poisson call. A kernel that
writes past either end of its buffer makes the call return CNV_CUDA_ERROR naming the buffer.
Each case below runs steps and a standalone Poisson solve with guards on small odd and even grids
and with every solver and precision, and checks that (1) no guard changed and (2) the fields
equal, bit for bit, those of the same run without guards.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    (7, {}), (8, {}), (33, {}), (64, {}),
    (33, {"order": 4}), (40, {"order": 2}),
    (64, {"poisson_type": 1}),                        # Gauss-Seidel
    (64, {"poisson_type": 3}),                        # Jacobi
    (66, {"sor_blocking": 1}), (66, {"sor_blocking": 2}), (130, {"sor_blocking": 4}),
    (320, {}),                                        # the exchange kernel, 2 blocks per SM
    (64, {"precision": 1}),                           # FP64 with FMA
    (64, {"precision": 2}), (130, {"precision": 2}),  # mixed
    (66, {"poisson_type": 4}),                        # direct
]


def run(cnv, n, guards, kw):
    cfg = cnv.default_config(nx=n, ny=n, Re=1000.0, dt=0.002, poisson_tol=1e-6, poisson_max_it=200000,
                             test_guard_cells=guards, **kw)
    f = np.random.default_rng(n).standard_normal((n, n))
    with cnv.Cavity(cfg) as cav:
        rc, _ = cav.step(3)
        assert rc == cnv.CNV_OK, cnv.last_error()
        fields = cav.get_fields()
        rc, psi, _, _ = cav.poisson(f)
        assert rc == cnv.CNV_OK, cnv.last_error()
    return fields + (psi,)


@pytest.mark.parametrize("n,kw", CASES, ids=[f"{n}-{'-'.join(f'{k}{v}' for k, v in kw.items()) or 'sor'}"
                                             for n, kw in CASES])
def test_no_kernel_writes_outside_its_buffers(cnv, n, kw):
    plain = run(cnv, n, 0, kw)
    guarded = run(cnv, n, 1, kw)
    for a, b in zip(plain, guarded):
        assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_guard_check_reports_a_changed_byte(cnv):
    """test_guard_cells = 2 changes one byte of the guard after u at creation (from the host): the
    first step must report it, naming u."""
    cfg = cnv.default_config(nx=32, ny=32, test_guard_cells=2)
    with cnv.Cavity(cfg) as cav:
        rc, _ = cav.step(1, raise_on_error=False)
        assert rc == cnv.CNV_CUDA_ERROR
        assert "after s->u" in cnv.last_error()


# ------------------------------------------------------------------------------ batched form
BATCH = [dict(n=384, Re=1500.0, lid=1.2), dict(n=256, Re=300.0, lid=0.7), dict(n=96, Re=900.0, lid=1.0),
         dict(n=40, Re=1200.0, lid=0.8), dict(n=33, Re=150.0, lid=1.4)]


def run_batch(cnv, guards, split):
    base = cnv.default_config(mixed_rtol=1e-10, test_guard_cells=guards)
    with cnv.Batch(base, BATCH) as bt:
        if split:
            bt.split(4, 1)
        groups = bt.groups()
        rc, _ = bt.step(2)
        assert rc == cnv.CNV_OK, cnv.last_error()
        return groups, [bt.get_fields(k) for k in range(len(BATCH))]


@pytest.mark.parametrize("split", [False, True], ids=["model-strips", "4x-strips"])
def test_no_batch_kernel_writes_outside_its_buffers(cnv, split):
    """Every buffer of every cavity in the batch arena is followed by a guard region: one-block
    cavities, row-strip groups of the cost model's sizes, and 2- to 4-strip groups of small
    cavities leave all of them intact, with the same fields as the unguarded batch."""
    g0, plain = run_batch(cnv, 0, split)
    g1, guarded = run_batch(cnv, 1, split)
    assert g0 == g1 and max(g1) > 1
    for fa, fb in zip(plain, guarded):
        for a, b in zip(fa, fb):
            assert np.array_equal(a.view(np.uint64), b.view(np.uint64))


def test_batch_guard_check_reports_a_changed_byte(cnv):
    base = cnv.default_config(mixed_rtol=1e-10, test_guard_cells=2)
    with cnv.Batch(base, BATCH[2:]) as bt:
        rc, _ = bt.step(1, raise_on_error=False)
        assert rc == cnv.CNV_CUDA_ERROR
        assert "after cavity 0's u" in cnv.last_error()


# --------------------------------------------------------------------------- differentiable form
@pytest.mark.parametrize("n,order", [(33, 6), (64, 4)])
def test_no_adjoint_kernel_writes_outside_its_buffers(cnv, n, order):
    """Forward run with checkpoints and the backward run's segment recomputation, with guards
    around every field, checkpoint and segment buffer: none changed, and J and the gradients equal
    those of the unguarded run bit for bit."""
    w0 = cnv.noise_field(n, seed=5, sigma=1.0, passes=4)
    out = []
    for guards in (0, 1):
        cfg = cnv.default_config(nx=n, ny=n, Re=400.0, dt=0.2 * min((1 / n) ** 2 * 100.0, 1 / n), order=order,
                                 test_guard_cells=guards)
        with cnv.Adjoint(cfg, 3) as adj:
            out.append(adj.enstrophy_gradient(w0, 1.0, 8))
    (j0, g0, l0), (j1, g1, l1) = out
    assert j0 == j1 and l0 == l1 and np.array_equal(g0.view(np.uint64), g1.view(np.uint64))


def test_adjoint_guard_check_reports_a_changed_byte(cnv):
    cfg = cnv.default_config(nx=32, ny=32, Re=400.0, dt=1e-4, test_guard_cells=2)
    with cnv.Adjoint(cfg, 4) as adj:
        with pytest.raises(cnv.CnvError) as ei:
            adj.forward(np.zeros((32, 32)), 1.0, 2)
    assert ei.value.status == cnv.CNV_CUDA_ERROR and "after u changed" in str(ei.value)
