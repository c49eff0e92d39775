"""cnv_poisson_noalloc: the Poisson solve for callers that may not allocate device memory.

Some callers cannot allocate GPU memory while they run. One example is an application whose
memory pool owns the whole device; another is a real-time loop where cudaMalloc/cudaFree are
forbidden because they synchronise the device and take unbounded time. For them this entry
point keeps its working arrays in one fixed device array inside the library. These tests call
it through the C ABI twice in a row, on different right-hand sides, and compare each result
with the regular entry point (cnv_poisson_device on a cnv_state). They use the same
tolerance as the other parity tests: fields to 1e-12 normwise relative (the two paths run the
same kernels, so they normally agree bit for bit) and equal iteration counts. A further test
checks the property the entry point exists for: once a first call has run on the device (that
call loads the library's kernels and places the fixed array there, under CUDA's default lazy
module loading), a call leaves the device's free memory unchanged.

This file is named so that pytest collects it last.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

FIELD_TOL = 1e-12


def _solve_noalloc(cnv, torch, f_dev, psi_dev, n, h, ptype, precision):
    it, err = C.c_int(-1), C.c_double(-1.0)
    stream = torch.cuda.current_stream().cuda_stream
    rc = cnv.load().cnv_poisson_noalloc(f_dev.data_ptr(), psi_dev.data_ptr(), n, h, h, ptype, precision,
                                        0.0, 200000, 1e-9, C.byref(it), C.byref(err), stream or None)
    return rc, it.value, err.value


@pytest.mark.gpu
@pytest.mark.parametrize("n,ptype,precision", [(200, 2, 0), (256, 2, 1), (97, 1, 0), (128, 3, 0), (512, 2, 0)])
def test_noalloc_matches_state_entry_point_on_two_calls(cnv, n, ptype, precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    h = 1.0 / n
    cfg = cnv.default_config(nx=n, ny=n, poisson_type=ptype, precision=precision, poisson_tol=1e-9,
                             poisson_max_it=200000)
    gen = torch.Generator(device="cpu").manual_seed(n)
    with cnv.Cavity(cfg) as cav:
        for call in range(2):
            f = torch.randn((n, n), dtype=torch.float64, generator=gen).cuda()
            psi_a = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
            psi_b = torch.full((n, n), float("nan"), dtype=torch.float64, device="cuda")
            torch.cuda.synchronize()
            rc_a, it_a, err_a = _solve_noalloc(cnv, torch, f, psi_a, n, h, ptype, precision)
            it_b, err_b = C.c_int(-1), C.c_double(-1.0)
            rc_b = cav._lib.cnv_poisson_device(cav._h, f.data_ptr(), psi_b.data_ptr(), C.byref(it_b),
                                              C.byref(err_b))
            torch.cuda.synchronize()
            assert rc_a == 0 and rc_b == 0, (call, rc_a, rc_b)
            a = psi_a.cpu().numpy()
            b = psi_b.cpu().numpy()
            assert np.all(np.isfinite(a))
            assert np.max(np.abs(a - b)) <= FIELD_TOL * np.max(np.abs(b)), f"call {call}"
            assert it_a == it_b.value, f"call {call}"
            assert abs(err_a - err_b.value) <= FIELD_TOL * abs(err_b.value), f"call {call}"


@pytest.mark.gpu
def test_noalloc_call_after_the_first_takes_no_device_memory(cnv):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    n = 256
    h = 1.0 / n
    gen = torch.Generator(device="cpu").manual_seed(7)
    f = torch.randn((n, n), dtype=torch.float64, generator=gen).cuda()
    psi = torch.empty((n, n), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    # first call on this device: may load modules and place the fixed array
    assert _solve_noalloc(cnv, torch, f, psi, n, h, 2, 0)[0] == 0
    torch.cuda.synchronize()
    results = []
    for _ in range(2):
        free_before, _total = torch.cuda.mem_get_info()
        rc, it, _err = _solve_noalloc(cnv, torch, f, psi, n, h, 2, 0)
        torch.cuda.synchronize()
        free_after, _total = torch.cuda.mem_get_info()
        assert rc == 0
        assert free_after == free_before, f"device free memory changed by {free_before - free_after} bytes"
        results.append((it, psi.cpu().numpy().copy()))
    assert results[0][0] == results[1][0]
    assert np.array_equal(results[0][1], results[1][1])


def test_noalloc_rejects_grids_beyond_its_scratch_size(cnv):
    # argument checks run before any CUDA call, so this needs no GPU
    it, err = C.c_int(0), C.c_double(0)
    rc = cnv.load().cnv_poisson_noalloc(C.c_void_p(8), C.c_void_p(8), 513, 1 / 513, 1 / 513, 2, 0, 0.0,
                                        100, 1e-6, C.byref(it), C.byref(err), None)
    assert rc == cnv.CNV_BAD_ARG
    rc = cnv.load().cnv_poisson_noalloc(C.c_void_p(8), C.c_void_p(8), 64, 1 / 64, 1 / 64, 4, 0, 0.0,
                                        100, 1e-6, C.byref(it), C.byref(err), None)
    assert rc == cnv.CNV_BAD_ARG
