"""Host-side checks that need no GPU: the library builds, loads and exports every entry point
declared in include/*.h; the config parser follows src/config.c; argument validation."""
from __future__ import annotations

import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


# header -> the library that must export its functions
LIBRARIES = {"cnv.h": "libcnv.so", "cnv_compat.h": "libcnv_compat.so"}


def declared_symbols(header=None):
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h") or (header and h != header):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text):
            name = m.group(1)
            if name not in {"if", "while", "for", "return", "sizeof"}:
                names.add(name)
    return names


def test_every_header_is_mapped_to_a_library():
    headers = {h for h in os.listdir(os.path.join(ROOT, "include")) if h.endswith(".h")}
    assert headers == set(LIBRARIES)


@pytest.mark.parametrize("header", sorted(LIBRARIES))
def test_library_exports_every_declared_symbol(cnv, header):
    import ctypes

    lib = ctypes.CDLL(os.path.join(os.path.dirname(cnv.LIB_PATH), LIBRARIES[header]))
    declared = declared_symbols(header)
    missing = [s for s in sorted(declared) if not hasattr(lib, s)]
    assert declared and not missing, missing


def test_compat_library_mirrors_reference_signatures():
    # the reference's call shapes (include/poisson.h:10-15, include/fluiddyn.h:5-7, :10)
    text = open(os.path.join(ROOT, "include", "cnv_compat.h")).read()
    for decl in ["mtrx poisson(mtrx f, double dx, double dy, int itmax, double tol);",
                 "mtrx poisson_SOR(mtrx f, double dx, double dy, int itmax, double tol, double beta);",
                 "mtrx poisson_log(mtrx f, double dx, double dy, int itmax, double tol, FILE *log_file);",
                 "mtrx poisson_SOR_log(mtrx f, double dx, double dy, int itmax, double tol, double beta, FILE *log_file);",
                 "void euler(mtrx w, mtrx dwdx, mtrx dwdy, mtrx d2wdx2, mtrx d2wdy2, mtrx u, mtrx v, double Re, double dt);",
                 "mtrx continuity(mtrx dudx, mtrx dvdy);", "double error(mtrx u1, mtrx u2);"]:
        assert decl in text, decl


def test_config_defaults_match_reference(cnv):
    c = cnv.default_config()
    # src/config.c:47-87
    assert (c.Re, c.Lx, c.Ly, c.nx, c.ny, c.dt, c.tf, c.max_co) == (1000.0, 1, 1, 64, 64, 0.005, 20.0, 1.0)
    assert (c.order, c.poisson_max_it, c.poisson_tol, c.output_interval, c.poisson_type) == (6, 10000, 1e-3, 10, 2)
    assert (c.u1, c.u2, c.u3, c.u4, c.v1, c.v2, c.v3, c.v4, c.ui, c.vi) == (0, 0, 0, 1.0, 0, 0, 0, 0, 0, 0)
    assert cnv.config_steps(c) == 4000  # it_max + 1 with it_max = (int)(20/0.005 - 1)


def test_config_parser_follows_reference_rules(cnv, tmp_path, capfd):
    p = tmp_path / "cfg.txt"
    p.write_text(
        "# comment\n"
        "; also a comment\n"
        "\n"
        "Re = 5000.0\n"
        "   nx=128\n"
        "ny = 128   \n"
        "Lx = 2.9\n"                 # atoi -> 2
        "dt = 0.001 # trailing text\n"
        "tf = 10.0\n"
        "poisson_tol = 5E-4\n"
        "poisson_max_it = 15000\n"
        "u4 = 1.5\n"
        "v2 = -0.25\n"
        "unknown_key = 3\n"
        "sor_omega = 1.5\n"
        "precision = fp64_fma\n"
        "nsteps = 7\n"
        "no equals sign here\n"
    )
    rc, c = cnv.load_config(str(p))
    out = capfd.readouterr().out
    assert rc == 0
    assert (c.Re, c.nx, c.ny, c.Lx, c.dt, c.tf, c.poisson_tol, c.poisson_max_it) == (5000.0, 128, 128, 2, 0.001, 10.0, 5e-4, 15000)
    assert (c.u4, c.v2, c.sor_omega, c.precision, c.nsteps) == (1.5, -0.25, 1.5, 1, 7)
    assert "Warning: Unknown configuration parameter 'unknown_key'" in out
    assert cnv.config_steps(c) == 7


def test_missing_config_file_keeps_defaults(cnv, tmp_path):
    rc, c = cnv.load_config(str(tmp_path / "nope.txt"))
    assert rc == cnv.CNV_IO_ERROR
    assert c.nx == 64 and c.Re == 1000.0


@pytest.mark.parametrize("field,value", [("ny", 63), ("order", 3), ("poisson_type", 5), ("nx", 3),
                                         ("precision", 9), ("dt", 0.0), ("u1", 1e6), ("test_guard_cells", 3),
                                         ("test_stall_block", -1)])
def test_create_rejects_bad_arguments_without_touching_the_gpu(cnv, field, value):
    cfg = cnv.default_config()
    setattr(cfg, field, value)
    if field == "nx":
        cfg.ny = value
    with pytest.raises(cnv.CnvError) as ei:
        cnv.Cavity(cfg)
    assert ei.value.status == cnv.CNV_BAD_ARG
