"""The reference-facing layer: the reference's own entry points (libcnv_compat.so), its program
(cnavier_gpu) and its output formats (log lines, VTK files).

- cnv_format_step_log prints the reference's lines (src/poisson.c:275, src/main.c:401-414)
  byte for byte; cnv_write_vtk writes src/utils.c's VTK layout byte for byte.
- cnavier_gpu run on the configurations of the reference's shipped red-black logs reproduces
  every logged step: iteration count, stop norm and continuity max/min as printed.
- The reference's own program sources, compiled where they lie, link against the compatibility
  library in place of src/poisson.c and src/fluiddyn.c (both builds; CPU only).
- The compatibility library's euler() and poisson_SOR_log(), driven by a copy of the
  reference's time loop (src/main.c:283-383) whose derivative products come from the oracle,
  give the oracle's fields bit for bit; cnavier_gpu's VTK files hold the oracle's fields.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
PKG = os.path.join(ROOT, "fluid-dynamics1_gb300")
APP = os.path.join(PKG, "cnavier_gpu")
COMPAT = os.path.join(PKG, "libcnv_compat.so")
GOLDEN = os.path.join(HERE, "golden", "logs_kat.json")


def parse_log(text):
    import sys

    sys.path.insert(0, os.path.join(HERE, "golden"))
    from make_golden import parse_log as p

    return p(text)


# --------------------------------------------------------------------------- formats (CPU)
def reference_step_lines(iters, err, t, dt, it_max, cmax, cmin, iter_s, elapsed):
    s = "Poisson equation solved with %d iterations - root-sum-of-squares error: %E\n" % (iters, err)
    s += "Iteration: %d | " % t + "Time: %f | " % (t * dt) + "Progress: %.2f%% | " % (100.0 * t / it_max)
    s += "Iter time: %.3f s\n" % iter_s
    s += "Continuity max: %E | " % cmax + "Continuity min: %E | " % cmin + "Elapsed: %.1f s | " % elapsed
    s += ("Est. remaining: %.1f s\n" % (elapsed / (t + 1) * (it_max - t))) if t > 0 else "Est. remaining: -- s\n"
    return s


@pytest.mark.parametrize("t", [0, 1, 57])
def test_step_log_lines_match_reference_format(cnv, t):
    info = cnv.StepInfo(iters=48, status=0, err=9.813335e-04, cont_max=1.991679e-16, cont_min=-1.743397e-16)
    buf = C.create_string_buffer(4096)
    lib = cnv.load()
    lib.cnv_format_step_log.argtypes = [C.POINTER(cnv.StepInfo), C.c_int, C.c_double, C.c_int, C.c_double,
                                        C.c_double, C.c_char_p, C.c_size_t]
    assert lib.cnv_format_step_log(C.byref(info), t, 0.005, 3999, 0.0123, 4.56, buf, 4096) == 0
    want = reference_step_lines(48, 9.813335e-04, t, 0.005, 3999, 1.991679e-16, -1.743397e-16, 0.0123, 4.56)
    assert buf.value.decode() == want
    info.status = cnv.CNV_NOT_CONVERGED
    assert lib.cnv_format_step_log(C.byref(info), t, 0.005, 3999, 0.0, 0.0, buf, 4096) == 0
    assert buf.value.decode() == "Error: maximum number of iterations achieved for Poisson equation.\n"
    assert lib.cnv_format_step_log(C.byref(info), t, 0.005, 3999, 0.0, 0.0, buf, 8) == cnv.CNV_BAD_ARG


def reference_vtk(field):
    """src/utils.c:62-96 written out in Python (printf %.6lf is correctly rounded on glibc)."""
    m, n = field.shape
    out = ["# vtk DataFile Version 2.0\n", "test\n", "ASCII\n", "DATASET STRUCTURED_POINTS\n",
           "DIMENSIONS %d %d 1\n" % (m, n), "ORIGIN 0 0 0\n", "SPACING 1 1 1\n", "POINT_DATA %d\n" % (m * n),
           "SCALARS values float\n", "LOOKUP_TABLE default"]
    for i in range(m):
        out.append("\n" + " ".join("%.6f" % field[i, j] for j in range(n)))
    return "".join(out)


def test_vtk_writer_matches_reference_layout(cnv, tmp_path):
    rng = np.random.default_rng(0)
    f = rng.standard_normal((5, 7)) * np.array([1e-9, 1e-3, 1, 1e3, 1e9, -0.5e-6, 2.5e-7])
    f[0, 0], f[1, 1], f[2, 2] = -0.0, 1e300, -1e-300
    lib = cnv.load()
    lib.cnv_write_vtk.argtypes = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_double), C.c_int, C.c_int]
    d = str(tmp_path / "out" / "run")
    assert lib.cnv_write_vtk(d.encode(), b"vorticity", 7, f.ctypes.data_as(C.POINTER(C.c_double)), 5, 7) == 0
    text = open(os.path.join(d, "vorticity-1-7.vtk")).read()
    assert text == reference_vtk(f)


# ------------------------------------------------------------------------- the program (GPU)
CONFIGS = {
    # config_default.txt / config_high_re.txt of the reference with OpenMP (red-black) enabled
    "testRunOMP": "Re = 1000.0\nnx = 64\nny = 64\ndt = 0.005\npoisson_max_it = 10000\npoisson_tol = 1E-3\n"
                  "order = 6\npoisson_type = 2\nopenmp_enabled = 1\n",
    "testRunOMPHIGHRES": "Re = 5000.0\nnx = 128\nny = 128\ndt = 0.001\npoisson_max_it = 15000\n"
                         "poisson_tol = 5E-4\norder = 6\npoisson_type = 2\nopenmp_enabled = 1\n",
}


def run_app(tmp_path, cfg_text, run_name):
    (tmp_path / "cfg.txt").write_text(cfg_text)
    r = subprocess.run([APP, "cfg.txt", run_name], cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r


@pytest.mark.gpu
@pytest.mark.parametrize("run", sorted(CONFIGS))
def test_program_reproduces_shipped_redblack_logs(tmp_path, run):
    golden = json.load(open(GOLDEN))[run]
    steps = len(golden["steps"])
    dt = golden["dt"]
    # the extension key nsteps fixes the step count (tf / dt rounds either way near an integer)
    cfg = CONFIGS[run] + f"tf = {(steps + 1) * dt!r}\nnsteps = {steps}\noutput_interval = 1000000\n"
    run_app(tmp_path, cfg, "kat")
    got = parse_log(open(tmp_path / "output" / "logs" / "kat.txt").read())
    assert len(got) == steps
    assert got == golden["steps"]


@pytest.mark.gpu
def test_program_writes_reference_vtk_files(tmp_path, orc):
    n, steps, interval, dt = 32, 7, 3, 0.004
    cfg = (f"Re = 400.0\nnx = {n}\nny = {n}\ndt = {dt!r}\ntf = {(steps + 1) * dt!r}\nnsteps = {steps}\n"
           f"poisson_tol = 1E-8\n"
           f"poisson_max_it = 100000\noutput_interval = {interval}\n")
    run_app(tmp_path, cfg, "vtk")
    files = sorted(os.listdir(tmp_path / "output" / "vtk"))
    # steps 0, 3, 6; four fields each; one counter (src/main.c:429-436)
    titles = ["stream-function", "vorticity", "x-velocity", "y-velocity"]
    assert files == sorted(f"{titles[k % 4]}-1-{k}.vtk" for k in range(12))
    p = orc.make_params(n, re=400.0, dt=dt, tol=1e-8, itmax=100000, exact_norm=1)
    W, U, V, PSI = orc.initial_state(n)
    assert orc.run(p, 7, W, U, V, PSI)[0] == 0  # the files of step 6 (the last ones)
    for k, field in zip(range(8, 12), (PSI, W, U, V)):
        assert open(tmp_path / "output" / "vtk" / f"{titles[k % 4]}-1-{k}.vtk").read() == reference_vtk(field)


# ------------------------------------------------------- the compatibility library, linked (CPU)
def test_reference_program_links_against_compat_library():
    """The reference's own main.c, linearalg.c, finitediff.c, utils.c and config.c, compiled where
    they lie (oracle/Makefile, target ab), link against libcnv_compat.so + libcnv.so in place of
    src/poisson.c and src/fluiddyn.c, in both of the reference's builds: the compatibility library
    defines every function the program takes from those two files. The programs only print their
    usage here (no GPU)."""
    import orc  # the oracle's helpers locate the reference tree

    ref = orc.reference_tree()
    if ref is None:
        pytest.skip("reference tree absent")
    import build as product_build  # fluid-dynamics1_gb300/build.py

    product_build.build()
    oracle_dir = os.path.join(ROOT, "oracle")
    subprocess.run(["make", "-s", "-B", "-C", oracle_dir, "ab", f"REF={ref}", f"LIBCNV={PKG}"], check=True)
    for exe in ("cnavier_ab", "cnavier_ab_seq"):
        path = os.path.join(oracle_dir, "_ref", exe)
        undefined = subprocess.run(["nm", "-D", "--undefined-only", path], capture_output=True, text=True,
                                   check=True).stdout.split()
        for name in ("euler", "poisson_SOR_log", "poisson_log", "continuity"):
            assert name in undefined, (exe, name)  # taken from the library, not compiled in
        r = subprocess.run([path, "--help"], capture_output=True, text=True, timeout=60)
        assert r.returncode == 0 and r.stdout.startswith("Usage:"), (exe, r.stdout[:200], r.stderr[:200])


# --------------------------------------------------------------- the compatibility library (GPU)
class Mtrx(C.Structure):
    _fields_ = [("M", C.POINTER(C.POINTER(C.c_double))), ("m", C.c_int), ("n", C.c_int)]


def as_mtrx(a):
    rows = (C.POINTER(C.c_double) * a.shape[0])(*[a[i].ctypes.data_as(C.POINTER(C.c_double))
                                                  for i in range(a.shape[0])])
    m = Mtrx(C.cast(rows, C.POINTER(C.POINTER(C.c_double))), a.shape[0], a.shape[1])
    m._keep = (rows, a)
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("n,order", [(48, 6), (33, 4)])
def test_compat_entry_points_reproduce_reference_loop(orc, n, order):
    lib = C.CDLL(COMPAT)
    lib.euler.argtypes = [Mtrx] * 7 + [C.c_double, C.c_double]
    lib.euler.restype = None
    lib.poisson_SOR_log.argtypes = [Mtrx, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double, C.c_void_p]
    lib.poisson_SOR_log.restype = Mtrx
    libc = C.CDLL(None)
    libc.free.argtypes = [C.c_void_p]
    re_, dt, tol, itmax, steps = 1000.0, 0.002, 1e-7, 100000, 5
    h = 1.0 / n
    beta = orc.sor_beta(n)
    b1, b2 = orc.fd_band(n, order, 1, h), orc.fd_band(n, order, 2, h)
    DX = lambda x, b=b1: orc.apply_j(b, x)
    DY = lambda x, b=b1: orc.apply_i(b, x)
    w, u, v, psi = orc.initial_state(n)
    for _ in range(steps):  # src/main.c:283-383
        u[:, 0] = u[:, -1] = 0.0
        v[:, 0] = v[:, -1] = 0.0
        u[0, :], u[-1, :] = 0.0, 1.0
        v[0, :] = v[-1, :] = 0.0
        u[:, 0] = u[:, -1] = 0.0
        wall = DX(v) - DY(u)
        w[0, :], w[-1, :], w[:, 0], w[:, -1] = wall[0, :], wall[-1, :], wall[:, 0], wall[:, -1]
        derivs = [DX(w), DY(w), DX(w, b2), DY(w, b2)]
        lib.euler(as_mtrx(w), *[as_mtrx(d) for d in derivs], as_mtrx(u), as_mtrx(v), re_, dt)
        f = -w
        res = lib.poisson_SOR_log(as_mtrx(f), h, h, itmax, tol, beta, None)
        psi = np.array([[res.M[i][j] for j in range(n)] for i in range(n)])
        for i in range(n):
            libc.free(C.cast(res.M[i], C.c_void_p))
        libc.free(C.cast(res.M, C.c_void_p))
        u = DY(psi)
        v = -DX(psi)
    p = orc.make_params(n, order=order, re=re_, dt=dt, tol=tol, itmax=itmax, exact_norm=1)
    W, U, V, PSI = orc.initial_state(n)
    assert orc.run(p, steps, W, U, V, PSI)[0] == 0
    for a, b in ((w, W), (u, U), (v, V), (psi, PSI)):
        assert np.array_equal(a, b)
