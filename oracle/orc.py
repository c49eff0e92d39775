"""ctypes binding of the CPU oracle (liboracle.so) and of the reference harness (oracle/_ref).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and by the
CPU-baseline leg of ``bench.py``. The product library never uses it.

``liboracle.so`` is the banded C restatement of cnavier's step (cnv_oracle.c). ``_ref/`` holds
the unmodified reference code compiled from the reference tree (``make -C oracle ref``); it
exists only where that tree exists, and every user of it checks ``ref_available()`` first.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libcnv_ref.so")

POISSON_GS, POISSON_SOR, POISSON_JACOBI = 1, 2, 3
ORDER_LEX, ORDER_REDBLACK = 0, 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Params(C.Structure):
    _fields_ = [
        ("n", C.c_int), ("order", C.c_int), ("dx", C.c_double), ("dy", C.c_double),
        ("re", C.c_double), ("dt", C.c_double), ("u_bc", C.c_double * 4),
        ("v_bc", C.c_double * 4), ("poisson_type", C.c_int), ("ordering", C.c_int),
        ("beta", C.c_double), ("itmax", C.c_int), ("tol", C.c_double), ("threads", C.c_int),
        ("exact_norm", C.c_int),
    ]


class StepInfo(C.Structure):
    _fields_ = [("iters", C.c_int), ("err", C.c_double), ("cont_max", C.c_double),
                ("cont_min", C.c_double), ("status", C.c_int)]


def reference_tree() -> str | None:
    """The reference's source tree, or None where it is absent: $CNV_REFERENCE_TREE when set,
    else a checkout named ``reference`` beside this repository (the same rule as oracle/Makefile)."""
    ref = os.environ.get("CNV_REFERENCE_TREE") or os.path.join(os.path.dirname(HERE), "..", "reference")
    ref = os.path.abspath(ref)
    return ref if os.path.isdir(os.path.join(ref, "src")) else None


def build(force: bool = False) -> None:
    """Compile liboracle.so (and the reference harness when the reference tree exists)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    ref = reference_tree()
    if ref and (force or not os.path.exists(REF_LIB_PATH)):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={ref}"], check=True)


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB_PATH)
        _lib.orc_fd_band.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp]
        _lib.orc_poisson.argtypes = [C.POINTER(Params), _dp, _dp, _ip, _dp]
        _lib.orc_run.argtypes = [C.POINTER(Params), C.c_int, _dp, _dp, _dp, _dp, C.POINTER(StepInfo)]
        _lib.orc_sor_beta.argtypes = [C.c_int, C.c_int]
        _lib.orc_sor_beta.restype = C.c_double
        _lib.orc_apply_i.argtypes = [C.c_int, _dp, _dp, _dp]
        _lib.orc_apply_j.argtypes = [C.c_int, _dp, _dp, _dp]
        _lib.orc_smooth_pass.argtypes = [C.c_int, _dp, _dp]
    return _lib


def ref_available() -> bool:
    try:
        build()
    except Exception:
        return False
    return os.path.exists(REF_LIB_PATH)


def ref_lib():
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_LIB_PATH)
        _ref.ref_run.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, _dp,
                                 C.c_int, C.c_double, C.c_int, C.c_double, C.c_int, C.c_int,
                                 _dp, _dp, _dp, _dp, _ip, _dp, _dp, _dp]
        _ref.ref_fd_dense.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, _dp]
    return _ref


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def sor_beta(nx: int, ny: int | None = None) -> float:
    return lib().orc_sor_beta(nx, nx if ny is None else ny)


def make_params(n, order=6, Lx=1, Ly=1, re=1000.0, dt=0.005, u_bc=(0.0, 0.0, 0.0, 1.0),
                v_bc=(0.0, 0.0, 0.0, 0.0), poisson_type=POISSON_SOR, ordering=ORDER_REDBLACK,
                beta=None, itmax=10000, tol=1e-3, threads=1, exact_norm=1) -> Params:
    p = Params()
    p.n, p.order = n, order
    p.dx, p.dy = float(Lx) / n, float(Ly) / n  # src/main.c:138-139
    p.re, p.dt = re, dt
    for k in range(4):
        p.u_bc[k], p.v_bc[k] = u_bc[k], v_bc[k]
    p.poisson_type, p.ordering = poisson_type, ordering
    p.beta = sor_beta(n) if beta is None else beta
    p.itmax, p.tol, p.threads, p.exact_norm = itmax, tol, threads, exact_norm
    return p


def fd_band(n, order, deriv, h) -> np.ndarray:
    out = np.zeros((n, 7))
    rc = lib().orc_fd_band(n, order, deriv, h, _ptr(out))
    if rc != 0:
        raise ValueError(f"orc_fd_band rc={rc}")
    return out


def apply_i(band, x):
    n = x.shape[0]
    d = np.zeros_like(x)
    lib().orc_apply_i(n, _ptr(np.ascontiguousarray(band)), _ptr(np.ascontiguousarray(x)), _ptr(d))
    return d


def apply_j(band, x):
    n = x.shape[0]
    d = np.zeros_like(x)
    lib().orc_apply_j(n, _ptr(np.ascontiguousarray(band)), _ptr(np.ascontiguousarray(x)), _ptr(d))
    return d


def poisson(p: Params, f: np.ndarray):
    psi = np.zeros_like(f)
    it, err = C.c_int(0), C.c_double(0)
    rc = lib().orc_poisson(C.byref(p), _ptr(np.ascontiguousarray(f)), _ptr(psi), C.byref(it), C.byref(err))
    return psi, it.value, err.value, rc


def initial_state(n, ui=0.0, vi=0.0):
    """Fields as src/main.c:178-221 leaves them before the first step."""
    w = np.zeros((n, n))
    psi = np.zeros((n, n))
    u = np.zeros((n, n))
    v = np.zeros((n, n))
    u[1:-1, 1:-1] = ui
    v[1:-1, 1:-1] = vi
    return w, u, v, psi


def run(p: Params, nsteps: int, w, u, v, psi):
    """Advance the state in place; returns (rc, list of per-step dicts)."""
    info = (StepInfo * max(nsteps, 1))()
    rc = lib().orc_run(C.byref(p), nsteps, _ptr(w), _ptr(u), _ptr(v), _ptr(psi), info)
    steps = [dict(iters=info[t].iters, err=info[t].err, cont_max=info[t].cont_max,
                  cont_min=info[t].cont_min, status=info[t].status) for t in range(nsteps)]
    return rc, steps


def smooth_pass(x):
    n = x.shape[0]
    d = np.zeros_like(x)
    lib().orc_smooth_pass(n, _ptr(np.ascontiguousarray(x)), _ptr(d))
    return d


# ---------------------------------------------------------------- reference harness (_ref)
def ref_fd_dense(n, order, deriv, h) -> np.ndarray:
    out = np.zeros((n, n))
    ref_lib().ref_fd_dense(n, order, deriv, h, _ptr(out))
    return out


def ref_run(n, order=6, Lx=1, Ly=1, re=1000.0, dt=0.005, u_bc=(0.0, 0.0, 0.0, 1.0),
            v_bc=(0.0, 0.0, 0.0, 0.0), poisson_type=POISSON_SOR, beta=None, itmax=10000,
            tol=1e-3, openmp=1, nsteps=1, w=None, u=None, v=None):
    """Run the reference's own dense step (src/main.c:283-395) through ref_harness.c."""
    w0, u0, v0, _ = initial_state(n)
    w = w0 if w is None else np.ascontiguousarray(w, dtype=np.float64).copy()
    u = u0 if u is None else np.ascontiguousarray(u, dtype=np.float64).copy()
    v = v0 if v is None else np.ascontiguousarray(v, dtype=np.float64).copy()
    psi = np.zeros((n, n))
    bc = np.array(list(u_bc) + list(v_bc), dtype=np.float64)
    it = (C.c_int * nsteps)()
    err = (C.c_double * nsteps)()
    cmax = (C.c_double * nsteps)()
    cmin = (C.c_double * nsteps)()
    if beta is None:
        beta = sor_beta(n)
    ref_lib().ref_run(n, order, Lx, Ly, re, dt, _ptr(bc), poisson_type, beta, itmax, tol, openmp,
                      nsteps, _ptr(w), _ptr(u), _ptr(v), _ptr(psi), it, err, cmax, cmin)
    steps = [dict(iters=it[t], err=err[t], cont_max=cmax[t], cont_min=cmin[t]) for t in range(nsteps)]
    return (w, u, v, psi), steps
