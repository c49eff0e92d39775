"""Thin ctypes binding of libcnv (include/cnv.h) for tests, the benchmark and Python callers.

This mirrors the C ABI one to one; the GPU work all happens inside libcnv.so. If the library is
missing or fails to load, every entry point raises: there is no Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libcnv.so")

CNV_OK, CNV_NOT_CONVERGED, CNV_NONFINITE, CNV_BAD_ARG = 0, 1, 2, 3
CNV_CUDA_ERROR, CNV_TIMEOUT, CNV_NO_DEVICE, CNV_IO_ERROR = 4, 5, 6, 7
STATUS_NAMES = {0: "OK", 1: "NOT_CONVERGED", 2: "NONFINITE", 3: "BAD_ARG", 4: "CUDA_ERROR",
                5: "TIMEOUT", 6: "NO_DEVICE", 7: "IO_ERROR"}
POISSON_GS, POISSON_SOR, POISSON_JACOBI, POISSON_DIRECT = 1, 2, 3, 4
PREC_FP64, PREC_FP64_FMA, PREC_MIXED = 0, 1, 2
INIT_REFERENCE, INIT_NOISE = 0, 1


class CnvError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Config(C.Structure):
    _fields_ = [
        ("Re", C.c_double), ("Lx", C.c_int), ("Ly", C.c_int), ("nx", C.c_int), ("ny", C.c_int),
        ("dt", C.c_double), ("tf", C.c_double), ("max_co", C.c_double), ("order", C.c_int),
        ("poisson_max_it", C.c_int), ("poisson_tol", C.c_double), ("output_interval", C.c_int),
        ("poisson_type", C.c_int), ("openmp_enabled", C.c_int),
        ("ui", C.c_double), ("vi", C.c_double),
        ("u1", C.c_double), ("u2", C.c_double), ("u3", C.c_double), ("u4", C.c_double),
        ("v1", C.c_double), ("v2", C.c_double), ("v3", C.c_double), ("v4", C.c_double),
        ("sor_omega", C.c_double), ("nsteps", C.c_int), ("precision", C.c_int),
        ("mixed_rtol", C.c_double), ("init_field", C.c_int), ("seed", C.c_ulonglong),
        ("init_sigma", C.c_double), ("init_smooth_passes", C.c_int), ("device", C.c_int),
        ("solver_blocks", C.c_int), ("mixed_inner_sweeps", C.c_int), ("mixed_max_outer", C.c_int),
        ("sor_blocking", C.c_int), ("mixed_warm_start", C.c_int), ("solver_timeout_ms", C.c_int),
        ("test_stall_block", C.c_int), ("test_guard_cells", C.c_int),
    ]


class StepInfo(C.Structure):
    _fields_ = [("iters", C.c_int), ("status", C.c_int), ("err", C.c_double),
                ("cont_max", C.c_double), ("cont_min", C.c_double)]


class CavitySpec(C.Structure):
    _fields_ = [("n", C.c_int), ("Re", C.c_double), ("lid", C.c_double), ("dt", C.c_double)]


_dp = C.POINTER(C.c_double)
_lib = None

# name -> (restype, argtypes)
_SIGS = {
    "cnv_config_default": (C.c_int, [C.POINTER(Config)]),
    "cnv_config_load": (C.c_int, [C.c_char_p, C.POINTER(Config)]),
    "cnv_config_set": (C.c_int, [C.POINTER(Config), C.c_char_p, C.c_char_p]),
    "cnv_config_steps": (C.c_int, [C.POINTER(Config)]),
    "cnv_create": (C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    "cnv_destroy": (None, [C.c_void_p]),
    "cnv_reset": (C.c_int, [C.c_void_p]),
    "cnv_grid_size": (C.c_int, [C.c_void_p]),
    "cnv_set_fields": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "cnv_get_fields": (C.c_int, [C.c_void_p, _dp, _dp, _dp, _dp]),
    "cnv_set_fields_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cnv_get_fields_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "cnv_step": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(StepInfo)]),
    "cnv_step_async": (C.c_int, [C.c_void_p, C.c_int]),
    "cnv_sync": (C.c_int, [C.c_void_p, C.POINTER(StepInfo), C.c_int]),
    "cnv_step_rows": (C.c_int, [C.c_void_p, C.POINTER(_dp), C.POINTER(_dp), C.POINTER(_dp),
                                C.POINTER(_dp), C.POINTER(StepInfo)]),
    "cnv_poisson": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(C.c_int), _dp]),
    "cnv_poisson_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.POINTER(C.c_int), _dp]),
    "cnv_last_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), _dp, _dp]),
    "cnv_time_passes": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp]),
    "cnv_solver_info": (C.c_int, [C.c_void_p, C.c_char_p, C.c_size_t]),
    "cnv_probe_fp64": (C.c_int, [C.c_int, _dp, _dp]),
    "cnv_check_mul_rn": (C.c_int, [C.c_int, _dp, C.c_int, C.c_double, _dp]),
    "cnv_check_div_rn": (C.c_int, [C.c_int, _dp, C.c_int, C.c_double, _dp, C.POINTER(C.c_longlong)]),
    "cnv_poisson_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int,
                                      C.c_int, C.c_double, C.c_int, C.c_double, C.POINTER(C.c_int), _dp,
                                      C.c_void_p]),
    "cnv_batch_specs": (C.c_int, [C.c_int, C.c_ulonglong, C.POINTER(CavitySpec)]),
    "cnv_batch_create": (C.c_int, [C.POINTER(Config), C.c_int, C.POINTER(CavitySpec), C.POINTER(C.c_void_p)]),
    "cnv_batch_destroy": (None, [C.c_void_p]),
    "cnv_batch_reset": (C.c_int, [C.c_void_p]),
    "cnv_batch_tune": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "cnv_batch_step": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(StepInfo)]),
    "cnv_batch_split": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "cnv_batch_groups": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "cnv_batch_plan": (C.c_int, [C.c_int, C.POINTER(CavitySpec), C.c_int, C.c_int, C.POINTER(C.c_int), _dp]),
    "cnv_batch_get_fields": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp]),
    "cnv_batch_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong), _dp]),
    "cnv_adjoint_create": (C.c_int, [C.POINTER(Config), C.c_int, C.POINTER(C.c_void_p)]),
    "cnv_adjoint_destroy": (None, [C.c_void_p]),
    "cnv_adjoint_forward": (C.c_int, [C.c_void_p, _dp, C.c_double, C.c_int, _dp]),
    "cnv_adjoint_backward": (C.c_int, [C.c_void_p, _dp, _dp, _dp]),
    "cnv_adjoint_forward_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_double, C.c_int, C.c_void_p]),
    "cnv_adjoint_backward_device": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, _dp]),
    "cnv_adjoint_enstrophy_gradient": (C.c_int, [C.c_void_p, _dp, C.c_double, C.c_int, _dp, _dp, _dp]),
    "cnv_adjoint_stats": (C.c_int, [C.c_void_p, _dp, _dp, C.POINTER(C.c_longlong)]),
    "cnv_noise_field": (C.c_int, [C.c_int, C.c_ulonglong, C.c_double, C.c_int, _dp]),
    "cnv_last_error": (C.c_char_p, []),
    "cnv_version": (C.c_char_p, []),
}


def load(path: str | None = None):
    """Load libcnv.so (building it first if it is missing). Raises if it cannot be loaded."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        import importlib.util

        spec = importlib.util.spec_from_file_location("cnv_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        mod.build()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols() -> list[str]:
    return list(_SIGS)


def last_error() -> str:
    return load().cnv_last_error().decode(errors="replace")


def check(status: int, what: str = "") -> None:
    if status != CNV_OK:
        raise CnvError(status, f"{what}: {last_error()}")


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "fields must be C-contiguous float64"
    return a.ctypes.data_as(_dp)


def default_config(**overrides) -> Config:
    cfg = Config()
    check(load().cnv_config_default(C.byref(cfg)), "cnv_config_default")
    for k, v in overrides.items():
        setattr(cfg, k, v)
    return cfg


def load_config(path: str) -> tuple[int, Config]:
    cfg = Config()
    rc = load().cnv_config_load(path.encode(), C.byref(cfg))
    return rc, cfg


def config_steps(cfg: Config) -> int:
    return load().cnv_config_steps(C.byref(cfg))


class Cavity:
    """One device-resident cavity (cnv_state)."""

    def __init__(self, cfg: Config):
        self._lib = load()
        self.cfg = cfg
        h = C.c_void_p()
        check(self._lib.cnv_create(C.byref(cfg), C.byref(h)), "cnv_create")
        self._h = h
        self.n = cfg.nx

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.cnv_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def reset(self):
        check(self._lib.cnv_reset(self._h), "cnv_reset")

    def set_fields(self, w=None, u=None, v=None) -> int:
        return self._lib.cnv_set_fields(self._h, _ptr(w), _ptr(u), _ptr(v))

    def get_fields(self):
        n = self.n
        w, u, v, psi = (np.empty((n, n)) for _ in range(4))
        check(self._lib.cnv_get_fields(self._h, _ptr(w), _ptr(u), _ptr(v), _ptr(psi)), "cnv_get_fields")
        return w, u, v, psi

    def step(self, nsteps: int = 1, raise_on_error: bool = True):
        """Advance nsteps; returns (status, list of per-step dicts)."""
        info = (StepInfo * max(nsteps, 1))()
        rc = self._lib.cnv_step(self._h, nsteps, info)
        if rc != CNV_OK and raise_on_error:
            raise CnvError(rc, last_error())
        return rc, [dict(iters=info[t].iters, status=info[t].status, err=info[t].err,
                         cont_max=info[t].cont_max, cont_min=info[t].cont_min) for t in range(nsteps)]

    def step_async(self, nsteps: int) -> None:
        check(self._lib.cnv_step_async(self._h, nsteps), "cnv_step_async")

    def sync(self, nsteps: int = 0):
        info = (StepInfo * max(nsteps, 1))()
        rc = self._lib.cnv_sync(self._h, info, nsteps)
        return rc, [dict(iters=info[t].iters, status=info[t].status, err=info[t].err,
                         cont_max=info[t].cont_max, cont_min=info[t].cont_min) for t in range(nsteps)]

    def step_rows(self, w, u, v, psi):
        """cnv_step_rows on row-pointer arrays built from the given (n, n) numpy fields."""
        rows = lambda a: (_dp * self.n)(*[a[i].ctypes.data_as(_dp) for i in range(self.n)])
        info = StepInfo()
        rc = self._lib.cnv_step_rows(self._h, rows(w), rows(u), rows(v), rows(psi), C.byref(info))
        return rc, dict(iters=info.iters, status=info.status, err=info.err, cont_max=info.cont_max,
                        cont_min=info.cont_min)

    def poisson(self, f):
        psi = np.empty_like(f)
        it, err = C.c_int(0), C.c_double(0.0)
        rc = self._lib.cnv_poisson(self._h, _ptr(np.ascontiguousarray(f)), _ptr(psi), C.byref(it), C.byref(err))
        return rc, psi, it.value, err.value

    def time_passes(self, reps: int = 20):
        """(ms of the pre-solve pass, ms of the post-solve pass), mean over reps launches each
        (cnv_time_passes)."""
        pre, post = C.c_double(0), C.c_double(0)
        check(self._lib.cnv_time_passes(self._h, reps, C.byref(pre), C.byref(post)), "cnv_time_passes")
        return pre.value, post.value

    def solver_info(self) -> str:
        """The Poisson solver this cavity runs and its geometry (cnv_solver_info)."""
        buf = C.create_string_buffer(256)
        check(self._lib.cnv_solver_info(self._h, buf, 256), "cnv_solver_info")
        return buf.value.decode()

    def stats(self):
        """(sweeps, ms of the last call, ms of the last Poisson kernel) -- CUDA-event times."""
        sw, ms, pms = C.c_longlong(0), C.c_double(0), C.c_double(0)
        check(self._lib.cnv_last_stats(self._h, C.byref(sw), C.byref(ms), C.byref(pms)), "cnv_last_stats")
        return sw.value, ms.value, pms.value

    # device-pointer variants (torch tensors or any CUDA allocation); pointers are ints
    def set_fields_device(self, w=0, u=0, v=0) -> int:
        return self._lib.cnv_set_fields_device(self._h, w or None, u or None, v or None)

    def get_fields_device(self, w=0, u=0, v=0, psi=0) -> int:
        return self._lib.cnv_get_fields_device(self._h, w or None, u or None, v or None, psi or None)


def batch_specs(count: int, seed: int = 0):
    """Cavities of the batched workload: n over {64,96,128,192,256,384}, Re in [100,2000], lid in [0.5,1.5]."""
    arr = (CavitySpec * count)()
    check(load().cnv_batch_specs(count, seed, arr), "cnv_batch_specs")
    return [dict(n=a.n, Re=a.Re, lid=a.lid, dt=a.dt) for a in arr]


def batch_plan(specs, blocks: int = 152, smem_bytes: int = 231424):
    """cnv_batch_plan (host only): the row strips per cavity that a batch of these cavities gets on
    a device running `blocks` blocks of `smem_bytes` bytes of shared memory (defaults: a GB300),
    and the schedule's estimated step time in microseconds."""
    arr = (CavitySpec * len(specs))(*[CavitySpec(s["n"], s["Re"], s["lid"], s.get("dt", 0.0)) for s in specs])
    groups = (C.c_int * len(specs))()
    us = C.c_double(0.0)
    check(load().cnv_batch_plan(len(specs), arr, blocks, smem_bytes, groups, C.byref(us)), "cnv_batch_plan")
    return list(groups), us.value


class Batch:
    """Many cavities advanced by one persistent launch (cnv_batch)."""

    def __init__(self, base: Config, specs):
        self._lib = load()
        self.specs = [dict(x) for x in specs]
        arr = (CavitySpec * len(specs))()
        for a, x in zip(arr, specs):
            a.n, a.Re, a.lid, a.dt = x["n"], x["Re"], x["lid"], x.get("dt", 0.0)
        h = C.c_void_p()
        check(self._lib.cnv_batch_create(C.byref(base), len(specs), arr, C.byref(h)), "cnv_batch_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.cnv_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def reset(self):
        check(self._lib.cnv_batch_reset(self._h), "cnv_batch_reset")

    def tune(self):
        t, b = C.c_int(0), C.c_int(0)
        check(self._lib.cnv_batch_tune(self._h, C.byref(t), C.byref(b)), "cnv_batch_tune")
        return t.value, b.value

    def split(self, factor: int, min_n: int = 1):
        check(self._lib.cnv_batch_split(self._h, factor, min_n), "cnv_batch_split")

    def groups(self):
        out = (C.c_int * len(self.specs))()
        check(self._lib.cnv_batch_groups(self._h, out), "cnv_batch_groups")
        return list(out)

    def step(self, nsteps: int = 1, raise_on_error: bool = True):
        info = (StepInfo * len(self.specs))()
        rc = self._lib.cnv_batch_step(self._h, nsteps, info)
        if rc != CNV_OK and raise_on_error:
            raise CnvError(rc, last_error())
        return rc, [dict(iters=i.iters, status=i.status, err=i.err, cont_max=i.cont_max, cont_min=i.cont_min)
                    for i in info]

    def get_fields(self, index: int):
        n = self.specs[index]["n"]
        w, u, v, psi = (np.empty((n, n)) for _ in range(4))
        check(self._lib.cnv_batch_get_fields(self._h, index, _ptr(w), _ptr(u), _ptr(v), _ptr(psi)),
              "cnv_batch_get_fields")
        return w, u, v, psi

    def stats(self):
        cells, sweeps, ms = C.c_longlong(0), C.c_longlong(0), C.c_double(0)
        check(self._lib.cnv_batch_stats(self._h, C.byref(cells), C.byref(sweeps), C.byref(ms)), "cnv_batch_stats")
        return cells.value, sweeps.value, ms.value


def probe_fp64(device: int = 0):
    """(multiply-then-add chains, FMA chains): FP64 lane-operations per second of the device."""
    a, f = C.c_double(0), C.c_double(0)
    check(load().cnv_probe_fp64(device, C.byref(a), C.byref(f)), "cnv_probe_fp64")
    return a.value, f.value


def check_mul_rn(x, c: float, device: int = 0):
    """c * x on the device the way the exact update multiplies by its constants."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    check(load().cnv_check_mul_rn(device, _ptr(x), x.size, c, _ptr(out)), "cnv_check_mul_rn")
    return out


def check_div_rn(x, b: float, device: int = 0):
    """(x / b on the device the way the exact update divides by a constant, how many quotients
    the three-operation path proved correctly rounded)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.empty_like(x)
    fast = C.c_longlong(0)
    check(load().cnv_check_div_rn(device, _ptr(x), x.size, b, _ptr(out), C.byref(fast)), "cnv_check_div_rn")
    return out, fast.value


def noise_field(n: int, seed: int, sigma: float = 1.0, passes: int = 0):
    """The CNV_INIT_NOISE field: sigma * N(0,1) per cell, then `passes` Jacobi averaging passes."""
    out = np.empty((n, n))
    check(load().cnv_noise_field(n, seed, sigma, passes, _ptr(out)), "cnv_noise_field")
    return out


class Adjoint:
    """Discrete adjoint of the time step (cnv_adjoint): forward runs keep checkpoints every
    `checkpoint_every` steps; backward returns dJ/dw0 and dJ/dlid for a given dJ/dw(T)."""

    def __init__(self, cfg: Config, checkpoint_every: int = 100):
        self._lib = load()
        self.n = cfg.nx
        self.h2 = (cfg.Lx / cfg.nx) * (cfg.Ly / cfg.ny)
        self.generation = 0  # counts forward runs (the checkpoints belong to the last one)
        h = C.c_void_p()
        check(self._lib.cnv_adjoint_create(C.byref(cfg), checkpoint_every, C.byref(h)), "cnv_adjoint_create")
        self._h = h

    def close(self):
        if getattr(self, "_h", None) and self._h.value:
            self._lib.cnv_adjoint_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def forward(self, w0, lid: float, nsteps: int):
        w0 = np.ascontiguousarray(w0, dtype=np.float64)
        wT = np.empty_like(w0)
        check(self._lib.cnv_adjoint_forward(self._h, _ptr(w0), float(lid), nsteps, _ptr(wT)), "cnv_adjoint_forward")
        self.generation += 1
        return wT

    def backward(self, g_final):
        g = np.ascontiguousarray(g_final, dtype=np.float64)
        gw0 = np.empty_like(g)
        glid = C.c_double(0)
        check(self._lib.cnv_adjoint_backward(self._h, _ptr(g), _ptr(gw0), C.byref(glid)), "cnv_adjoint_backward")
        return gw0, glid.value

    def forward_device(self, w0_ptr: int, lid: float, nsteps: int, wT_ptr: int):
        check(self._lib.cnv_adjoint_forward_device(self._h, w0_ptr, float(lid), nsteps, wT_ptr),
              "cnv_adjoint_forward_device")
        self.generation += 1

    def backward_device(self, g_ptr: int, gw0_ptr: int) -> float:
        glid = C.c_double(0)
        check(self._lib.cnv_adjoint_backward_device(self._h, g_ptr, gw0_ptr, C.byref(glid)),
              "cnv_adjoint_backward_device")
        return glid.value

    def enstrophy_gradient(self, w0, lid: float, nsteps: int):
        """J = 1/2 sum w(T)^2 dx dy, dJ/dw0, dJ/dlid."""
        w0 = np.ascontiguousarray(w0, dtype=np.float64)
        gw0 = np.empty_like(w0)
        J, glid = C.c_double(0), C.c_double(0)
        check(self._lib.cnv_adjoint_enstrophy_gradient(self._h, _ptr(w0), float(lid), nsteps, C.byref(J), _ptr(gw0),
                                                       C.byref(glid)), "cnv_adjoint_enstrophy_gradient")
        self.generation += 1
        return J.value, gw0, glid.value

    def stats(self):
        f, b, by = C.c_double(0), C.c_double(0), C.c_longlong(0)
        check(self._lib.cnv_adjoint_stats(self._h, C.byref(f), C.byref(b), C.byref(by)), "cnv_adjoint_stats")
        return f.value, b.value, by.value
