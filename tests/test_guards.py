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
