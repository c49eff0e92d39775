"""Generate the committed golden fixtures from the reference's own recorded runs.

Reads the four run logs shipped with SorinBetisor/fluid-dynamics1 (output/logs/*.txt) and
writes ``logs_kat.json``: per logged time step, the Poisson iteration count and stop norm
(src/poisson.c:275) and the continuity max/min (src/main.c:407-408), as the printed strings.
These are the reference's known-answer values for the step; the tests replay the oracle (and
the CUDA path) on the same configuration and compare the printed digits.

With ``--verify`` it also rebuilds the unmodified reference (``make -C oracle ref``), runs it
on the same configurations truncated to a few steps, and checks that its fresh log repeats
the shipped lines, so the fixtures are pinned to the code, not only to the files.

Run from the repository root:  python tests/golden/make_golden.py [--verify]
This script needs the reference tree ($CNV_REFERENCE_TREE, or a checkout named "reference" beside
this repository); the fixtures it writes do not.
"""
from __future__ import annotations

import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
# the reference tree: $CNV_REFERENCE_TREE, else a checkout named "reference" beside this repository
REF = os.path.abspath(os.environ.get("CNV_REFERENCE_TREE") or os.path.join(ROOT, "..", "reference"))

# Run configurations: config_default.txt (64^2, Re 1000, dt 0.005, tol 1e-3, itmax 10000) and
# config_high_re.txt (128^2, Re 5000, dt 1e-3, tol 5e-4, itmax 15000); openmp_enabled selects
# the red-black SOR of the OPENMP_ENABLED build, 0 the lexicographic sweep.
RUNS = {
    "testRunNOOMP": dict(config="config_default.txt", n=64, re=1000.0, dt=0.005, tol=1e-3,
                         itmax=10000, ordering="lex"),
    "testRunOMP": dict(config="config_default.txt", n=64, re=1000.0, dt=0.005, tol=1e-3,
                       itmax=10000, ordering="redblack"),
    "testRunNOOMPHIGHRES": dict(config="config_high_re.txt", n=128, re=5000.0, dt=0.001,
                                tol=5e-4, itmax=15000, ordering="lex"),
    "testRunOMPHIGHRES": dict(config="config_high_re.txt", n=128, re=5000.0, dt=0.001,
                              tol=5e-4, itmax=15000, ordering="redblack"),
}

PAT_P = re.compile(r"Poisson equation solved with (\d+) iterations - root-sum-of-squares error: (\S+)")
PAT_C = re.compile(r"Continuity max: (\S+) \| Continuity min: (\S+) \|")


def parse_log(text: str):
    steps, cur = [], None
    for line in text.splitlines():
        m = PAT_P.search(line)
        if m:
            cur = dict(iters=int(m.group(1)), err=m.group(2))
            continue
        m = PAT_C.search(line)
        if m and cur is not None:
            cur["cont_max"], cur["cont_min"] = m.group(1), m.group(2)
            steps.append(cur)
            cur = None
    return steps


def verify(name: str, spec: dict, shipped: list, nsteps: int = 4) -> None:
    """Run the freshly built reference binary for nsteps and compare with the shipped log."""
    binary = os.path.join(ROOT, "oracle", "_ref",
                          "cnavier_omp" if spec["ordering"] == "redblack" else "cnavier_seq")
    with tempfile.TemporaryDirectory() as tmp:
        cfg = open(os.path.join(REF, spec["config"])).read()
        # tf = (nsteps + 1) * dt gives it_max + 1 = nsteps steps (src/main.c:162)
        cfg = re.sub(r"^tf\s*=.*$", f"tf = {(nsteps + 1) * spec['dt']}", cfg, flags=re.M)
        cfg = re.sub(r"^output_interval\s*=.*$", "output_interval = 100000", cfg, flags=re.M)
        if spec["ordering"] == "lex":
            cfg = re.sub(r"^openmp_enabled\s*=.*$", "openmp_enabled = 0", cfg, flags=re.M)
        open(os.path.join(tmp, "cfg.txt"), "w").write(cfg)
        subprocess.run([binary, "cfg.txt", "kat"], cwd=tmp, check=True,
                       stdout=subprocess.DEVNULL, env=dict(os.environ, OMP_NUM_THREADS="1"))
        fresh = parse_log(open(os.path.join(tmp, "output", "logs", "kat.txt")).read())
    got = fresh[:nsteps]
    want = shipped[:nsteps]
    status = "OK" if got == want else "MISMATCH"
    print(f"  verify {name}: {status} over {len(got)} steps")
    if got != want:
        for a, b in zip(got, want):
            print("    fresh", a, "\n    shipped", b)


def main() -> int:
    out = {}
    for name, spec in RUNS.items():
        text = open(os.path.join(REF, "output", "logs", name + ".txt")).read()
        steps = parse_log(text)
        out[name] = dict(spec, source=f"output/logs/{name}.txt", steps=steps)
        print(f"{name}: {len(steps)} logged steps")
        if "--verify" in sys.argv:
            subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"],
                           check=True)
            verify(name, spec, steps)
    with open(os.path.join(HERE, "logs_kat.json"), "w") as f:
        json.dump(out, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
