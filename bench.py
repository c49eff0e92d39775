#!/usr/bin/env python
"""Benchmark of the vorticity-streamfunction time step on GB300.

Workload (one "step" = one explicit time step of cnavier's solver, src/main.c:283-395): the
lid-driven cavity on a 1024 x 1024 grid, Re = 1000, lid u = 1, w = psi = 0 at t = 0,
dt = 0.2*min(h^2 Re/4, h/|u|max), red-black SOR with the reference's factor
(src/main.c:134) to sum|d psi| < 1e-6 from a zero start every step (src/poisson.c). Inputs are
synthetic: the cavity's own initial condition, nothing is read from disk.

Prints one JSON line. value = Mcell-steps/s = n^2 * steps / (sum of per-step device times),
each step timed with CUDA events on the library's stream, with L2 flushed (a 256 MB write)
before every timed step. e2e = the same metric through the C ABI with host buffers: every step
uploads w, u, v from pinned host memory, runs, and reads w, u, v, psi back, all inside the
timed region. roofline = the persistent Poisson kernel, algorithmic bytes (24 B per interior
cell per sweep: read psi and f, write psi) over its CUDA-event duration, against the measured
HBM copy bandwidth; roofline.fp64_pipe = the same kernel's FP64 rate (7 add/multiply operations
per cell-sweep), against the device's rate for that mix measured by a probe kernel in the same
run -- the ceiling that binds, since the solve runs from L2. cpu_baseline = the CPU oracle (a
restatement of the reference's own algorithm) on this host's cores for the same steps as value,
started from the GPU's fields after the warm-up steps. config is the workload only; both arms
print the same dict (the reference arm runs the same steps); how this arm runs it is in path.

forms = the other ways the library takes the step, each timed the same way and compared field by
field (max and RMS relative difference) after the same steps with the plain FP64 SOR path and
with the converged FP64 answer (the direct sine-transform solve): fp64_fma, mixed (FP32 sweeps
in FP64 defect correction) and direct on the 1024^2 workload; mixed_2048, a 2048^2 cavity with
a smoothed-noise initial vorticity; batched_256, 256 cavities of uneven size, Re and lid speed
in one persistent launch per call against the FP64 path run cavity by cavity; adjoint_256, the
gradient of the final enstrophy of a 256^2 cavity after 2000 steps with respect to the initial
vorticity and the lid speed, checked against central differences on 16 random directions.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun each rank runs an independent replica (the step does not shard: one cavity per
GPU); value is the sum over ranks of cells x steps divided by the slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "fluid-dynamics1_gb300")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "Mcell-steps/s at residual 1e-6, mixed/batched vs plain FP64; %HBM peak"
UNIT = "Mcell-steps/s"
BYTES_PER_CELL_SWEEP = 24  # FP64: read psi (8) and f (8), write psi (8)


def workload(n=1024, re=1000.0, lid=1.0):
    h = 1.0 / n
    dt = 0.2 * min(h * h * re / 4.0, h / abs(lid))
    return dict(n=n, re=re, lid=lid, dt=dt, tol=1e-6, itmax=1000000)


def workload_name(w):
    return (f"lid-driven cavity {w['n']}x{w['n']}, Re {w['re']:g}, lid u={w['lid']:g}, dt={w['dt']:.6g}, "
            f"red-black SOR (reference beta) to sum|dpsi| < {w['tol']:g} from zero every step")


# ------------------------------------------------------------------------------ utilities
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Dist:
    """Barrier and max-reduction across torchrun ranks (no-ops for one process)."""

    def __init__(self, ws, device):
        self.ws = ws
        self.pg = None
        if ws > 1:
            import torch
            import torch.distributed as td

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            td.init_process_group(backend)
            self.td, self.torch = td, torch
            self.device = f"cuda:{device}" if backend == "nccl" else "cpu"

    def barrier(self):
        if self.ws > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.ws == 1:
            return x
        t = self.torch.tensor([x], dtype=self.torch.float64, device=self.device)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.ws > 1:
            self.td.destroy_process_group()


class L2Flusher:
    """Writes 256 MB (about twice the 129 MB L2) on the device before each timed step."""

    def __init__(self, device):
        self.buf = None
        try:
            import torch

            if torch.cuda.is_available():
                self.torch = torch
                self.buf = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{device}")
        except Exception:
            self.buf = None

    def __call__(self):
        if self.buf is not None:
            self.buf.fill_(1)
            self.torch.cuda.synchronize()

    @property
    def active(self):
        return self.buf is not None


class ClockSampler:
    """nvidia-smi samples (200 ms) while the timed region runs."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one k_poisson launch on the headline
# workload, from an ncu capture of the kernel as built at the commit named below. The solve runs
# from L2, so this is the compulsory first touch of psi and f, not a per-sweep figure.
POISSON_TRAFFIC = {"bytes_per_launch": 17982464.0,
                   "source": "ncu capture of k_poisson, 1024^2 workload, one launch (step 0), build of commit f9d9c8a"}

L2_NOTE = "flushed before every timed step on the GPU (256 MB device write)"


def bench_config(w, first_step, sweeps_per_step):
    """The workload description both arms print (the reference arm runs the same steps)."""
    return {"workload": workload_name(w), "grid": w["n"], "first_step": first_step,
            "sweeps_per_step": round(sweeps_per_step, 1), "l2": L2_NOTE}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# The two passes around the Poisson solve, per cell: algorithmic bytes (each field read or written
# once; halo re-reads not counted) and FP64 add/multiply operations on interior cells.
PRE_BYTES, PRE_OPS = 40, 66    # read w, u, v; write w_out and the right-hand side; 4 x 14 + 8 + 2
POST_BYTES, POST_OPS = 32, 57  # read psi; write u, v, psi; 2 x 14 (velocity) + 2 x 14 + 1 (continuity)


def step_passes(cnvpy, local, n, add_mul_rate, peak_gbs, reps=50):
    """k_pre and k_post timed alone (cnv_time_passes) on an n^2 cavity with a developed field (a
    smoothed-noise vorticity, one step), against the HBM peak and the device's FP64 add/multiply
    rate (fp64_frac counts all 66 / 57 operations, including the multiplications the kernels do on
    the integer pipes, so it can exceed 1)."""
    w = workload(n)
    init = dict(init_field=1, seed=2024, init_sigma=0.1, init_smooth_passes=8)
    with cnvpy.Cavity(make_config(cnvpy, w, local, poisson_type=4, **init)) as cav:
        cav.step(1)
        pre_ms, post_ms = cav.time_passes(reps)
    cells = n * n
    out = {}
    for name, ms, nb, ops in (("k_pre", pre_ms, PRE_BYTES, PRE_OPS), ("k_post", post_ms, POST_BYTES, POST_OPS)):
        gbs = cells * nb / (ms * 1e-3) / 1e9
        gops = cells * ops / (ms * 1e-3) / 1e9
        out[name] = {"ms": round(ms, 4), "bytes_per_cell": nb, "achieved_gbs": round(gbs, 1),
                     "hbm_frac": round(gbs / peak_gbs, 4), "fp64_ops_per_cell": ops, "fp64_gops": round(gops, 1),
                     "fp64_frac": round(gops * 1e9 / add_mul_rate, 4) if add_mul_rate else None}
    return out


def form_adjoint(cnvpy, local, ndirs=16, n=256, steps=2000, every=100, eps=1e-6):
    """256^2 cavity, Re 400, 2000 steps, initial vorticity = seeded smooth Gaussian field: gradient
    of J = 1/2 sum w(T)^2 h^2 with respect to w0 and the lid speed by the adjoint kernels
    (checkpoints every 100 steps), checked against central differences on seeded random
    directions; cost of forward and gradient."""
    import numpy as np

    h = 1.0 / n
    dt = 0.2 * min(h * h * 400.0 / 4, h)
    cfg = cnvpy.default_config(nx=n, ny=n, Re=400.0, dt=dt, device=local)
    w0 = cnvpy.noise_field(n, seed=2025, sigma=1.0, passes=16)
    rng = np.random.default_rng(2026)
    with cnvpy.Adjoint(cfg, every) as adj:
        adj.enstrophy_gradient(w0, 1.0, steps)  # warm-up
        J, gw, glid = adj.enstrophy_gradient(w0, 1.0, steps)
        fwd_ms, bwd_ms, state_bytes = adj.stats()

        def objective(w, l):
            wT = adj.forward(w, l, steps)
            return 0.5 * adj.h2 * float(np.sum(wT * wT))

        errs = []
        for _ in range(ndirs):
            d = np.zeros((n, n))
            d[1:-1, 1:-1] = rng.standard_normal((n - 2, n - 2))
            dl = float(rng.standard_normal())
            fd = (objective(w0 + eps * d, 1.0 + eps * dl) - objective(w0 - eps * d, 1.0 - eps * dl)) / (2 * eps)
            ad = float(np.sum(gw * d)) + glid * dl
            errs.append(abs(fd - ad) / abs(ad))
        fwd_only_ms = adj.stats()[0]
    return {"workload": f"{n}x{n} cavity, Re 400, lid 1, dt={dt:.6g}, {steps} steps, initial vorticity = seeded "
                        f"Gaussian noise (sigma 1, seed 2025) smoothed by 16 Jacobi passes; J = 1/2 sum w(T)^2 h^2",
            "J": J, "dJ_dlid": glid, "grad_w0_norm": float(np.linalg.norm(gw)),
            "forward_ms": round(fwd_only_ms, 2), "gradient_ms": round(fwd_ms + bwd_ms, 2),
            "gradient_cost_over_forward": round((fwd_ms + bwd_ms) / fwd_only_ms, 3),
            "forward_value": mcells(n * n, steps, fwd_only_ms), "unit": UNIT,
            "checkpoint_every": every, "state_bytes": state_bytes,
            "fd_check": {"directions": ndirs, "eps": eps, "max_rel_err": max(errs),
                         "median_rel_err": float(np.median(errs))},
            "poisson": "direct (exact sine-transform solve; self-adjoint)"}


# ------------------------------------------------------------------------------- our arm
FORMS = {
    # name: (precision, poisson_type, description)
    "fp64": (0, 2, "fp64 red-black SOR, reference rounding"),
    "fp64_fma": (1, 2, "fp64 red-black SOR, FMA form of the update"),
    "mixed": (2, 2, "FP32 red-black SOR sweeps inside FP64 defect correction to relative residual 1e-10"),
    "direct": (0, 4, "exact FP64 sine-transform solve of the same discrete equation (converged answer)"),
}


def make_config(cnvpy, w, device, precision=0, poisson_type=2, **extra):
    return cnvpy.default_config(nx=w["n"], ny=w["n"], Re=w["re"], u4=w["lid"], dt=w["dt"],
                                poisson_tol=w["tol"], poisson_max_it=w["itmax"], device=device,
                                precision=precision, poisson_type=poisson_type, mixed_rtol=1e-10, **extra)


def run_device(cnvpy, w, device, steps, warmup, flush, precision=0, poisson_type=2, clocks=None, fields=False,
               **extra):
    """Device-resident run: per-step records with CUDA-event times (and the final fields)."""
    cfg = make_config(cnvpy, w, device, precision, poisson_type, **extra)
    recs = []
    with cnvpy.Cavity(cfg) as cav:
        for t in range(warmup + steps):
            flush()
            if t == warmup and clocks is not None:
                clocks.start()
            rc, info = cav.step(1)
            sweeps, ms, pms = cav.stats()
            if t >= warmup:
                recs.append(dict(ms=ms, poisson_ms=pms, sweeps=sweeps, iters=info[0]["iters"],
                                 solver=cav.solver_info()))
        out = cav.get_fields() if fields else None
    return (recs, out) if fields else recs


def field_error(test, ref):
    """Per field (w, u, v, psi): max |test - ref| / max |ref| and RMS(test - ref) / RMS(ref)."""
    import numpy as np

    out = {}
    for name, a, b in zip(("w", "u", "v", "psi"), test, ref):
        d = a - b
        out[name] = {"max_rel": float(np.max(np.abs(d)) / max(np.max(np.abs(b)), 1e-300)),
                     "rms_rel": float(np.sqrt(np.mean(d * d)) / max(np.sqrt(np.mean(b * b)), 1e-300))}
    return out


def mcells(cells, steps, ms):
    return round(cells * steps / (ms * 1e-3) / 1e6, 4)


def form_1024(cnvpy, w, local, args, flush, name, ref_fields, conv_fields):
    """Another solver of the headline workload, with its field errors against the FP64 SOR path
    and against the converged FP64 answer (the direct solve)."""
    fprec, ptype, fdesc = FORMS[name]
    fr, fields = run_device(cnvpy, w, local, args.steps, args.warmup, flush, precision=fprec, poisson_type=ptype,
                            fields=True)
    f_ms = sum(r["ms"] for r in fr)
    out = {"value": mcells(w["n"] ** 2, len(fr), f_ms), "unit": UNIT, "steps": len(fr),
           "sweeps_per_step": sum(r["sweeps"] for r in fr) / len(fr), "solver": fdesc,
           "compared_after_steps": args.warmup + args.steps}
    if ref_fields is not None:
        out["error_vs_fp64_sor"] = field_error(fields, ref_fields)
    if conv_fields is not None and name != "direct":
        out["error_vs_converged_fp64"] = field_error(fields, conv_fields)
    return out, fields


def form_mixed_2048(cnvpy, local, flush, steps=3, warmup=3):
    """2048^2 cavity, Re 1000, initial vorticity = seeded Gaussian noise (sigma 0.1) smoothed by 8
    Jacobi passes: FP32 sweeps in FP64 defect correction (relative residual 1e-10) against the
    plain FP64 path (sum|dpsi| < 1e-6) and the direct solve, all timed; fields compared with the
    converged FP64 answer (the direct solve) after the same steps."""
    w = workload(2048)
    init = dict(init_field=1, seed=2024, init_sigma=0.1, init_smooth_passes=8)
    out = {"workload": f"2048x2048 cavity, Re 1000, lid 1, dt={w['dt']:.6g}, noise initial vorticity "
                       f"(sigma 0.1, 8 smoothing passes, seed 2024)"}
    res = {}
    for name, prec, ptype in (("fp64", 0, 2), ("mixed", 2, 2), ("direct", 0, 4)):
        fr, fields = run_device(cnvpy, w, local, steps, warmup, flush, precision=prec, poisson_type=ptype, fields=True,
                                **init)
        res[name] = fields
        out[name] = {"value": mcells(w["n"] ** 2, len(fr), sum(r["ms"] for r in fr)), "unit": UNIT,
                     "steps": len(fr), "sweeps_per_step": sum(r["sweeps"] for r in fr) / len(fr)}
    for name in ("fp64", "mixed"):
        out[name]["error_vs_converged_fp64"] = field_error(res[name], res["direct"])
    out["mixed"]["error_vs_fp64_sor"] = field_error(res["mixed"], res["fp64"])
    out["compared_after_steps"] = steps + warmup
    out["speedup_mixed_over_fp64"] = round(out["mixed"]["value"] / out["fp64"]["value"], 3)
    out["speedup_direct_over_fp64"] = round(out["direct"]["value"] / out["fp64"]["value"], 3)
    return out


def form_batched(cnvpy, local, steps, count=256, seed=0):
    """256 cavities (n from {64,...,384}, Re in [100,2000], lid in [0.5,1.5], stable dt) in one
    persistent launch per call, shape autotuned; against the plain FP64 path run cavity by
    cavity on one cavity of each size, fields compared after the same steps."""
    specs = cnvpy.batch_specs(count, seed=seed)
    base = cnvpy.default_config(mixed_rtol=1e-10, device=local)
    out = {"workload": f"{count} cavities, seed {seed}: n uniform over {{64,96,128,192,256,384}}, Re uniform in "
                       f"[100,2000], lid uniform in [0.5,1.5], dt = 0.2 min(h^2 Re/4, h/lid)"}
    sample = []
    for n in sorted({s["n"] for s in specs}):
        sample.append(next(k for k, s in enumerate(specs) if s["n"] == n))
    with cnvpy.Batch(base, specs) as bt:
        threads, per_sm = bt.tune()
        groups = bt.groups()
        bt.step(1)
        rc, last = bt.step(steps)
        cells, sweeps, ms = bt.stats()
        fields = {k: bt.get_fields(k) for k in sample}
    out["batched"] = {"value": mcells(cells, steps, ms), "unit": UNIT, "steps": steps, "cells": cells,
                      "ms_per_step": round(ms / steps, 3), "tuned_shape": {"threads": threads,
                                                                           "blocks_per_sm": per_sm},
                      "blocks_per_cavity": {str(n): groups[sample[i]] for i, n in
                                            enumerate(sorted({s["n"] for s in specs}))},
                      "cost_model_ms_per_step": round(cnvpy.batch_plan(specs)[1] / 1e3, 3),
                      "max_relative_residual": max(x["err"] for x in last)}
    f_cells, f_ms, m_ms, errs = 0, 0.0, 0.0, {}
    for k in sample:
        sp = specs[k]
        h = 1.0 / sp["n"]
        dt = sp["dt"] or 0.2 * min(h * h * sp["Re"] / 4.0, h / abs(sp["lid"]))  # the batch's stable dt
        cfg = cnvpy.default_config(nx=sp["n"], ny=sp["n"], Re=sp["Re"], u4=sp["lid"], dt=dt,
                                   poisson_tol=1e-6, poisson_max_it=1000000, mixed_rtol=1e-10, device=local)
        with cnvpy.Cavity(cfg) as cav:
            cav.step(1)
            cav.step(steps)
            _, c_ms, _ = cav.stats()
            sor_fields = cav.get_fields()
        cfg.precision = 2  # the mixed form alone: same solver as the batch, one cavity at a time
        with cnvpy.Cavity(cfg) as cav:
            cav.step(1)
            cav.step(steps)
            _, mc_ms, _ = cav.stats()
        cfg.precision = 0
        cfg.poisson_type = 4
        with cnvpy.Cavity(cfg) as cav:
            cav.step(1 + steps)
            conv = cav.get_fields()
        errs[f"n{sp['n']}"] = {"batched_vs_converged_fp64": field_error(fields[k], conv),
                               "fp64_sor_vs_converged_fp64": field_error(sor_fields, conv)}
        f_cells += sp["n"] ** 2
        f_ms += c_ms
        m_ms += mc_ms
    sample_note = f"one cavity of each size, each its own cnv_state, one call of {steps} steps"
    out["fp64_cavity_by_cavity"] = {"value": mcells(f_cells, steps, f_ms), "unit": UNIT, "sample": sample_note}
    out["mixed_cavity_by_cavity"] = {"value": mcells(f_cells, steps, m_ms), "unit": UNIT, "sample": sample_note}
    out["errors"] = errs
    out["compared_after_steps"] = steps + 1
    b, f, m = out["batched"]["value"], out["fp64_cavity_by_cavity"]["value"], out["mixed_cavity_by_cavity"]["value"]
    out["speedup_batched_over_fp64"] = round(b / f, 3)
    out["speedup_mixed_over_fp64_cavity_by_cavity"] = round(m / f, 3)   # what the FP32 sweeps buy
    out["speedup_batched_over_mixed_cavity_by_cavity"] = round(b / m, 3)  # what batching buys
    out["cost_model_check"] = batch_model_check(cnvpy, local)
    return out


def batch_model_check(cnvpy, local, steps=20):
    """The batch cost model's estimated step time against the measured one, on two small batches
    where the model splits cavities that fit one block: ten 192^2 cavities, and five of 33^2..128^2."""
    out = {}
    for name, specs in (("ten_192", [dict(n=192, Re=1000.0, lid=1.0)] * 10),
                        ("five_33_to_128", [dict(n=n, Re=1000.0, lid=1.0) for n in (33, 64, 96, 112, 128)])):
        groups, est_us = cnvpy.batch_plan(specs)
        with cnvpy.Batch(cnvpy.default_config(mixed_rtol=1e-10, device=local), specs) as bt:
            bt.step(1)
            bt.step(steps)
            ms = bt.stats()[2] / steps
            used = bt.groups()
        out[name] = {"strips": used, "model_ms": round(est_us / 1e3, 3), "measured_ms": round(ms, 3),
                     "model_error": round(est_us / 1e3 / ms - 1, 3), "planned_strips": groups}
    return out


def run_e2e(cnvpy, w, device, steps, warmup):
    """Host-buffer run through the C ABI: upload w,u,v, step, read w,u,v,psi, every step."""
    import numpy as np

    n = w["n"]
    pinned = False
    try:
        import torch

        bufs = [torch.empty((n, n), dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
        pinned = True
    except Exception:
        bufs = [np.empty((n, n)) for _ in range(4)]
    hw, hu, hv, hpsi = bufs
    cfg = make_config(cnvpy, w, device)
    with cnvpy.Cavity(cfg) as cav:
        cw, cu, cv, cpsi = cav.get_fields()
        hw[...], hu[...], hv[...] = cw, cu, cv
        lib, h = cav._lib, cav._h
        ptr = cnvpy._ptr
        elapsed = 0.0
        for t in range(warmup + steps):
            t0 = time.perf_counter()
            cnvpy.check(lib.cnv_set_fields(h, ptr(hw), ptr(hu), ptr(hv)), "cnv_set_fields")
            cnvpy.check(lib.cnv_step(h, 1, None), "cnv_step")
            cnvpy.check(lib.cnv_get_fields(h, ptr(hw), ptr(hu), ptr(hv), ptr(hpsi)), "cnv_get_fields")
            t1 = time.perf_counter()
            if t >= warmup:
                elapsed += t1 - t0
    return elapsed, pinned


def cpu_baseline(w, ncores, start_fields, first_step, steps, gpu_sweeps):
    """The CPU oracle on this host for the same steps as the GPU's timed region: it starts from
    the GPU's fields after the warm-up steps (bit for bit the oracle's own state there) and runs
    steps first_step .. first_step + steps - 1."""
    import orc

    orc.build()
    n = w["n"]
    p = orc.make_params(n, re=w["re"], dt=w["dt"], u_bc=(0.0, 0.0, 0.0, w["lid"]), tol=w["tol"],
                        itmax=w["itmax"], threads=ncores, exact_norm=0)
    W, U, V, PSI = (a.copy() for a in start_fields)
    t0 = time.perf_counter()
    rc, info = orc.run(p, steps, W, U, V, PSI)
    t1 = time.perf_counter()
    sweeps = [s["iters"] + 1 for s in info]
    return {"value": n * n * steps / (t1 - t0) / 1e6, "unit": UNIT, "cores": ncores, "kind": "port",
            "sample": f"steps {first_step}..{first_step + steps - 1} of the {n}^2 workload (the GPU's timed "
                      f"steps, {sum(sweeps) / len(sweeps):.1f} red-black SOR sweeps per step), "
                      f"oracle/cnv_oracle.c with OpenMP on {ncores} threads, {t1 - t0:.2f} s",
            "sweeps_match_gpu": sweeps == gpu_sweeps}


def ours(args):
    ws, rank, local = dist_env()
    dist = Dist(ws, local)
    import cnvpy

    cnvpy.load()
    w = workload(args.n)
    flush = L2Flusher(local)
    clocks = ClockSampler(local) if rank == 0 else None
    dist.barrier()
    prec, ptype, prec_name = FORMS[args.form]
    recs, head_fields = run_device(cnvpy, w, local, args.steps, args.warmup, flush, precision=prec,
                                   poisson_type=ptype, clocks=clocks, fields=True)
    clk = clocks.stop() if clocks else None
    dist.barrier()
    total_ms = sum(r["ms"] for r in recs)
    total_ms_max = dist.max(total_ms)
    cells = w["n"] * w["n"]
    value = ws * cells * args.steps / (total_ms_max * 1e-3) / 1e6

    interior = (w["n"] - 2) ** 2
    sweeps = sum(r["sweeps"] for r in recs)
    pms = sum(r["poisson_ms"] for r in recs)
    if args.form == "mixed":
        # FP32 sweep: read e and R/den, write e (12 B); per correction: FP64 residual (read psi,
        # g, write R/den: 20 B) and update (read + write psi: 16 B)
        outer = sum(r["iters"] for r in recs)
        alg_bytes = interior * (12 * sweeps + 36 * outer)
        kernel = "k_mixed (persistent FP32 red-black SOR in FP64 defect correction, one launch per step)"
    else:
        alg_bytes = interior * BYTES_PER_CELL_SWEEP * sweeps
        kernel = "k_poisson (persistent red-black SOR, one launch per step)"
    achieved = alg_bytes / (pms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = POISSON_TRAFFIC["bytes_per_launch"] if args.form == "fp64" else None
    fp64 = None
    add_mul, fma_rate = cnvpy.probe_fp64(local)
    if args.form == "fp64":
        # the binding ceiling: the update's 7 FP64 add/multiply operations per interior cell-sweep
        # (5 on the FP64 pipe, the 2 multiplications by constants in exact integer arithmetic),
        # against the device's own FP64 rate for that mix (probe kernels, same process)
        ops = 7.0 * interior * sweeps / (pms * 1e-3)
        fp64 = {"achieved_gops": round(ops / 1e9, 1), "peak_gops": round(add_mul / 1e9, 1),
                "frac": round(ops / add_mul, 4), "fma_peak_gops": round(fma_rate / 1e9, 1),
                "ops_per_cell_sweep": 7, "on_fp64_pipe_per_cell_sweep": 5,
                "peak_source": "probe kernel: independent round-to-nearest multiply-then-add chains"}

    e2e_s, pinned = run_e2e(cnvpy, w, local, args.steps, args.warmup)
    e2e_s = dist.max(e2e_s)
    e2e = {"value": ws * cells * args.steps / e2e_s / 1e6, "unit": UNIT,
           "h2d_bytes_per_step": 3 * cells * 8, "d2h_bytes_per_step": 4 * cells * 8,
           "host_buffers": "pinned" if pinned else "pageable"}

    passes = {str(n): step_passes(cnvpy, local, n, add_mul, peak) for n in (w["n"], 2 * w["n"])}

    forms = {}
    conv_err = None
    if not args.skip_forms:
        # converged FP64 answer of the same steps (direct solve), and the FP64 SOR path's fields
        direct_form, conv_fields = form_1024(cnvpy, w, local, args, flush, "direct",
                                             head_fields if args.form == "fp64" else None, None)
        sor_fields = head_fields
        if args.form != "fp64":
            _, sor_fields = run_device(cnvpy, w, local, args.steps, args.warmup, flush, fields=True)
            direct_form["error_vs_fp64_sor"] = field_error(conv_fields, sor_fields)
        conv_err = field_error(head_fields, conv_fields)
        for name in FORMS:
            if name not in (args.form, "fp64", "direct"):
                forms[name], _ = form_1024(cnvpy, w, local, args, flush, name, sor_fields, conv_fields)
        forms["direct"] = direct_form
        forms["mixed_2048"] = form_mixed_2048(cnvpy, local, flush)
        forms["batched_256"] = form_batched(cnvpy, local, max(5, args.steps // 2))
        forms["adjoint_256"] = form_adjoint(cnvpy, local)

    cpu = None
    if rank == 0 and ws == 1 and not args.skip_cpu and args.form == "fp64":
        start = run_device(cnvpy, w, local, args.warmup, 0, lambda: None, fields=True)[1]
        cpu = cpu_baseline(w, os.cpu_count() or 1, start, args.warmup, args.steps,
                           [r["iters"] + 1 for r in recs])

    line = {
        "metric": METRIC, "value": round(value, 4), "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms_max / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(w, args.warmup, sweeps / len(recs)),
        "path": {"precision": prec_name, "solver": recs[0]["solver"] if recs else None,
                 "parallelism": f"replicas x{ws}", "l2_flushed": flush.active},
        "Mcell_sweeps_per_s": round(interior * sweeps / (pms * 1e-3) / 1e6, 2),
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4), "traffic": traffic,
                     "traffic_source": POISSON_TRAFFIC["source"] if traffic else None, "peak_source": peak_kind,
                     "kernel": kernel, "fp64_pipe": fp64},
        "e2e": e2e,
        "gpu_launches": 3 * args.steps,  # k_pre, k_poisson, k_post per step
        "step_passes": passes,
        "clocks": clk,
        "forms": forms,
    }
    if conv_err is not None:
        line["error_vs_converged_fp64"] = conv_err
    if cpu:
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist.close()


# ------------------------------------------------------------------------- reference arm
def reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return  # the reference is CPU code: rank 0 alone runs it
    import numpy as np
    import orc

    orc.build()
    w = workload(args.n)
    n = w["n"]
    cores = os.cpu_count() or 1
    p = orc.make_params(n, re=w["re"], dt=w["dt"], u_bc=(0.0, 0.0, 0.0, w["lid"]), tol=w["tol"],
                        itmax=w["itmax"], threads=cores, exact_norm=0)
    W, U, V, PSI = orc.initial_state(n)
    for _ in range(args.warmup):
        orc.run(p, 1, W, U, V, PSI)
    t0 = time.perf_counter()
    rc, info = orc.run(p, args.steps, W, U, V, PSI)
    t1 = time.perf_counter()
    value = n * n * args.steps / (t1 - t0) / 1e6
    # The reference's own dense operators need 4*(n^2)^2*8 bytes (35 TB at 1024^2), so its CPU path
    # at this size is the banded restatement (bitwise-equal to it where both run).
    kind = "port"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 6), "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round((t1 - t0) * 1e3 / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(w, args.warmup, sum(s["iters"] + 1 for s in info) / len(info)),
        "cpu_baseline": {"value": round(value, 6), "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"steps {args.warmup}..{args.warmup + args.steps - 1} of the {n}^2 workload, "
                                   f"oracle/cnv_oracle.c (restatement of the reference's CPU path, red-black "
                                   f"SOR) with OpenMP on {cores} threads"},
        "e2e": {"value": round(value, 6), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def full_config(args):
    """One of the workloads run to its stated length (not part of the default run): a JSON line
    with throughput sampled over windows of steps, sweeps per step, and the per-field error at the
    end against the converged FP64 answer (the direct sine-transform solve of the same steps).
        1: 64^2, Re 100, dt 1e-3, SOR factor 1.5, tol 1e-6, 1000 steps, against the CPU oracle
        2: the 1024^2 headline workload, 10,000 steps: FP64 SOR, mixed and direct
        3: 2048^2, Re 1000, smoothed-noise start, 5,000 steps: mixed and direct (FP64 SOR too
           with --with-sor)
        4: 256 uneven cavities, 2,000 steps: batched, against each size's direct run"""
    import numpy as np

    import cnvpy

    cnvpy.load()
    which = args.full_config
    out = {"full_config": which, "unit": UNIT}

    def windows(w, steps, window, **kw):
        """Run steps in windows; per window: Mcell-steps/s from CUDA-event times and sweeps/step."""
        cfg = make_config(cnvpy, w, 0, **kw)
        rows, total_ms, sweeps_all = [], 0.0, 0
        with cnvpy.Cavity(cfg) as cav:
            done = 0
            while done < steps:
                k = min(window, steps - done)
                rc, info = cav.step(k)
                sw, ms, _ = cav.stats()
                total_ms += ms
                sweeps_all += sw
                rows.append({"steps": [done, done + k - 1], "value": mcells(w["n"] ** 2, k, ms),
                             "sweeps_per_step": round(sw / k, 1), "iters_last": info[-1]["iters"],
                             "cont_max_last": info[-1]["cont_max"]})
                done += k
            fields = cav.get_fields()
        return {"value": mcells(w["n"] ** 2, steps, total_ms), "steps": steps, "seconds": round(total_ms / 1e3, 2),
                "sweeps_per_step": round(sweeps_all / steps, 1), "windows": rows}, fields

    if which == 1:
        import orc

        n, steps = 64, 1000
        w = dict(n=n, re=100.0, lid=1.0, dt=1e-3, tol=1e-6, itmax=1000000)
        res, g = windows(w, steps, 100, sor_omega=1.5)
        p = orc.make_params(n, re=100.0, dt=1e-3, tol=1e-6, beta=1.5, itmax=1000000, threads=1)
        W, U, V, PSI = orc.initial_state(n)
        t0 = time.perf_counter()
        rc, info = orc.run(p, steps, W, U, V, PSI)
        t1 = time.perf_counter()
        res["bitwise_equal_to_oracle"] = all(np.array_equal(a.view(np.uint64), b.view(np.uint64))
                                             for a, b in zip(g, (W, U, V, PSI)))
        res["oracle_1_core"] = mcells(n * n, steps, (t1 - t0) * 1e3)
        out["fp64"] = res
    elif which == 2:
        w = workload(1024)
        out["workload"] = workload_name(w) + ", 10,000 steps"
        fields = {}
        for name, prec, ptype in (("fp64", 0, 2), ("mixed", 2, 2), ("direct", 0, 4)):
            out[name], fields[name] = windows(w, 10000, 500, precision=prec, poisson_type=ptype)
        for name in ("fp64", "mixed"):
            out[name]["error_vs_converged_fp64"] = field_error(fields[name], fields["direct"])
        out["mixed"]["error_vs_fp64_sor"] = field_error(fields["mixed"], fields["fp64"])
    elif which == 3:
        w = workload(2048)
        init = dict(init_field=1, seed=2024, init_sigma=0.1, init_smooth_passes=8)
        out["workload"] = f"2048x2048 cavity, Re 1000, lid 1, dt={w['dt']:.6g}, noise start, 5,000 steps"
        fields = {}
        forms = (("fp64", 0, 2),) if args.with_sor else ()
        for name, prec, ptype in forms + (("mixed", 2, 2), ("direct", 0, 4)):
            out[name], fields[name] = windows(w, 5000, 500, precision=prec, poisson_type=ptype, **init)
        for name in fields:
            if name != "direct":
                out[name]["error_vs_converged_fp64"] = field_error(fields[name], fields["direct"])
    elif which == 4:
        steps = 2000
        specs = cnvpy.batch_specs(256, seed=0)
        base = cnvpy.default_config(mixed_rtol=1e-10)
        sample = [next(k for k, x in enumerate(specs) if x["n"] == n) for n in sorted({x["n"] for x in specs})]
        with cnvpy.Batch(base, specs) as bt:
            bt.tune()
            rows, total_ms = [], 0.0
            for k in range(steps // 250):
                rc, last = bt.step(250)
                cells, _, ms = bt.stats()
                total_ms += ms
                rows.append({"steps": [250 * k, 250 * k + 249], "value": mcells(cells, 250, ms),
                             "max_relative_residual": max(x["err"] for x in last)})
            fields = {k: bt.get_fields(k) for k in sample}
        errs = {}
        for k in sample:
            sp = specs[k]
            h = 1.0 / sp["n"]
            dt = sp["dt"] or 0.2 * min(h * h * sp["Re"] / 4.0, h / abs(sp["lid"]))
            cfg = cnvpy.default_config(nx=sp["n"], ny=sp["n"], Re=sp["Re"], u4=sp["lid"], dt=dt, poisson_type=4)
            with cnvpy.Cavity(cfg) as cav:
                cav.step(steps)
                errs[f"n{sp['n']}"] = field_error(fields[k], cav.get_fields())
        out["batched"] = {"value": mcells(cells, steps, total_ms), "steps": steps, "cells": cells,
                          "seconds": round(total_ms / 1e3, 2), "windows": rows, "error_vs_converged_fp64": errs}
    print(json.dumps(out), flush=True)


def only(args):
    """One small invocation of each named form, in order, for profilers: the kernels run as in the
    forms above; prints one JSON line of wall times (not a benchmark result)."""
    import cnvpy

    cnvpy.load()
    out = {}
    for item in args.only.split(","):
        name, _, size = item.partition("@")  # e.g. fp64@512: that form on a 512^2 cavity
        size, _, start = size.partition("+")  # direct@2048+noise: from a smoothed-noise vorticity
        init = dict(init_field=1, seed=2024, init_sigma=0.1, init_smooth_passes=8) if start == "noise" else {}
        t0 = time.perf_counter()
        if name in ("fp64", "fp64_fma", "mixed", "direct"):
            prec, ptype, _ = FORMS[name]
            run_device(cnvpy, workload(int(size) if size else 1024), 0, 1, 0, lambda: None, precision=prec,
                       poisson_type=ptype, **init)
        elif name == "batched":
            with cnvpy.Batch(cnvpy.default_config(mixed_rtol=1e-10), cnvpy.batch_specs(256, seed=0)) as bt:
                bt.tune()  # one launch per candidate decomposition (5), then the step on the kept one
                bt.step(1)
        elif name == "adjoint":
            n = 256
            h = 1.0 / n
            cfg = cnvpy.default_config(nx=n, ny=n, Re=400.0, dt=0.2 * min(h * h * 100.0, h))
            with cnvpy.Adjoint(cfg, 10) as adj:
                adj.enstrophy_gradient(cnvpy.noise_field(n, seed=2025, sigma=1.0, passes=16), 1.0, 20)
        else:
            raise SystemExit(f"unknown form {name}")
        out[item] = round(time.perf_counter() - t0, 3)
    print(json.dumps({"only": out, "unit": "s (wall, first call)"}), flush=True)


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--grid", dest="n", type=int, default=1024, help=argparse.SUPPRESS)
    ap.add_argument("--skip-cpu", action="store_true", help="omit the cpu_baseline leg")
    ap.add_argument("--skip-forms", action="store_true", help="omit the extra precision/batch forms")
    ap.add_argument("--form", choices=["fp64", "fp64_fma", "mixed"], default="fp64",
                    help="form measured for the headline value")
    ap.add_argument("--only", default=None,
                    help="comma list of fp64,fp64_fma,mixed,direct,batched,adjoint (fp64@512: on a 512^2 "
                         "cavity; direct@2048+noise: from a smoothed-noise vorticity): run one small case of "
                         "each (for profilers) and exit")
    ap.add_argument("--full-config", type=int, choices=[1, 2, 3, 4], default=None,
                    help="run that workload to its stated step count and print its JSON line (minutes)")
    ap.add_argument("--with-sor", action="store_true", help="--full-config 3: also the FP64 SOR path (~25 min)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)  # at least 3 untimed warm-up steps
    if args.full_config:
        full_config(args)
    elif args.only:
        only(args)
    elif args.impl == "reference":
        reference(args)
    else:
        ours(args)


if __name__ == "__main__":
    main()
