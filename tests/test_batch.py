"""Batched form: many cavities of uneven size, Re and lid speed in one persistent launch.

Each cavity must equal a single-cavity run of the same mixed-precision step (same operators,
same FP32 red-black sweeps, same defect-correction stop rule) to 1e-12 normwise relative per
field, and match the FP64 oracle run to a tight tolerance within the mixed form's 1e-7.
"""
from __future__ import annotations

import numpy as np
import pytest

SAME_SCHEME_TOL = 1e-12   # batch vs single-cavity mixed run, normwise relative
ORACLE_TOL = 1e-7         # batch vs FP64 oracle converged tightly, normwise relative


def test_specs_generator_is_deterministic_and_in_range(cnv):
    a = cnv.batch_specs(256, seed=0)
    b = cnv.batch_specs(256, seed=0)
    c = cnv.batch_specs(256, seed=1)
    assert a == b and a != c
    assert {x["n"] for x in a} == {64, 96, 128, 192, 256, 384}
    assert all(100 <= x["Re"] <= 2000 and 0.5 <= x["lid"] <= 1.5 for x in a)
    counts = np.bincount([[64, 96, 128, 192, 256, 384].index(x["n"]) for x in a], minlength=6)
    assert counts.min() > 20  # roughly uniform over the six sizes


def test_plan_of_the_256_cavity_workload(cnv):
    """The decomposition the batch picks, planned on the host for a GB300 (152 blocks of 231424
    bytes of shared memory): 384^2 and 256^2 cavities as 3-strip groups (the cost model's choice;
    3 and 2 strips are the smallest that fit), the rest one block each, and an estimated step time
    close to the balanced load."""
    specs = cnv.batch_specs(256, seed=0)
    groups, us = cnv.batch_plan(specs)
    by_n = {}
    for sp, g in zip(specs, groups):
        by_n.setdefault(sp["n"], set()).add(g)
    assert by_n == {64: {1}, 96: {1}, 128: {1}, 192: {1}, 256: {3}, 384: {3}}
    assert 30e3 < us < 36e3, us  # measured on a GB300: 33.5 ms per step


def test_plan_of_ten_192_cavities_counts_the_group_barriers(cnv):
    """Ten 192^2 cavities: the plan splits each into row strips, and its estimate includes the
    groups' barriers (one per 4 FP32 sweeps plus about 20 per step). Measured on a GB300: 3.9 ms
    per step on 4-strip groups (9.8 ms on one block each); without the barrier term the estimate
    was 3.0 ms. It must be within 10% now."""
    groups, us = cnv.batch_plan([dict(n=192, Re=1000.0, lid=1.0)] * 10)
    assert len(set(groups)) == 1 and groups[0] >= 2, groups
    assert abs(us - 3.9e3) <= 0.1 * 3.9e3, us


def test_plan_balances_a_few_large_cavities_and_rejects_bad_input(cnv):
    # three cavities on 152 blocks: more strips than needed shorten the step
    groups, us = cnv.batch_plan([dict(n=384, Re=1500.0, lid=1.2), dict(n=256, Re=300.0, lid=0.7),
                                 dict(n=192, Re=900.0, lid=1.0)])
    assert groups[0] > 3 and groups[1] >= 2 and groups[2] == 1, groups
    one, us1 = cnv.batch_plan([dict(n=384, Re=1500.0, lid=1.2)], blocks=3)
    assert one == [3] and us1 > us  # three blocks: the smallest count that fits, and slower
    for bad in (dict(blocks=0), dict(smem_bytes=0)):
        with pytest.raises(cnv.CnvError):
            cnv.batch_plan(SPECS, **bad)
    with pytest.raises(cnv.CnvError):
        cnv.batch_plan([dict(n=384, Re=1.0, lid=1.0)], blocks=2)  # needs 3 blocks


def _stable_dt(n, re, lid):
    h = 1.0 / n
    return 0.2 * min(h * h * re / 4, h / abs(lid))


SPECS = [dict(n=64, Re=400.0, lid=1.0), dict(n=40, Re=1500.0, lid=0.7), dict(n=96, Re=120.0, lid=1.3),
         dict(n=33, Re=900.0, lid=0.5), dict(n=128, Re=2000.0, lid=1.1)]


@pytest.mark.gpu
def test_batch_equals_single_cavity_runs(cnv):
    base = cnv.default_config(mixed_rtol=1e-10)
    nsteps = 3
    with cnv.Batch(base, SPECS) as bt:
        rc, last = bt.step(nsteps)
        fields = [bt.get_fields(k) for k in range(len(SPECS))]
    assert rc == 0
    for k, sp in enumerate(SPECS):
        cfg = cnv.default_config(nx=sp["n"], ny=sp["n"], Re=sp["Re"], u4=sp["lid"],
                                 dt=_stable_dt(sp["n"], sp["Re"], sp["lid"]), precision=cnv.PREC_MIXED,
                                 mixed_rtol=1e-10)
        with cnv.Cavity(cfg) as cav:
            _, steps = cav.step(nsteps)
            single = cav.get_fields()
        assert last[k]["iters"] == steps[-1]["iters"]
        for name, a, b in zip("w u v psi".split(), fields[k], single):
            assert np.max(np.abs(a - b)) <= SAME_SCHEME_TOL * np.max(np.abs(b)), (k, name)


@pytest.mark.gpu
def test_batch_matches_fp64_oracle(cnv, orc):
    base = cnv.default_config(mixed_rtol=1e-10)
    specs = SPECS[:3]
    with cnv.Batch(base, specs) as bt:
        bt.step(3)
        fields = [bt.get_fields(k) for k in range(len(specs))]
    for k, sp in enumerate(specs):
        n = sp["n"]
        p = orc.make_params(n, re=sp["Re"], dt=_stable_dt(n, sp["Re"], sp["lid"]), u_bc=(0, 0, 0, sp["lid"]),
                            tol=1e-13 * n * n, itmax=10_000_000, threads=0, exact_norm=0)
        w, u, v, psi = orc.initial_state(n)
        orc.run(p, 3, w, u, v, psi)
        for name, a, b in zip("w u v psi".split(), fields[k], (w, u, v, psi)):
            assert np.max(np.abs(a - b)) <= ORACLE_TOL * np.max(np.abs(b)), (k, name)


@pytest.mark.gpu
def test_batch_tuned_shape_gives_the_same_fields(cnv):
    base = cnv.default_config(mixed_rtol=1e-10)
    specs = cnv.batch_specs(12, seed=3)
    specs = [dict(x, n=min(x["n"], 128)) for x in specs]  # keep the test quick
    with cnv.Batch(base, specs) as bt:
        bt.step(2)
        ref = [bt.get_fields(k) for k in range(len(specs))]
        threads, per_sm = bt.tune()
        assert threads in (256, 512, 1024) and per_sm in (1, 2)
        bt.step(2)
        tuned = [bt.get_fields(k) for k in range(len(specs))]
    for a4, b4 in zip(ref, tuned):
        for a, b in zip(a4, b4):
            assert np.max(np.abs(a - b)) <= SAME_SCHEME_TOL * max(np.max(np.abs(b)), 1e-300)


@pytest.mark.gpu
def test_warm_batch_equals_warm_single_cavity_runs(cnv):
    base = cnv.default_config(mixed_rtol=1e-10, mixed_warm_start=1)
    nsteps = 4
    specs = SPECS[:3]
    with cnv.Batch(base, specs) as bt:
        rc, last = bt.step(nsteps)
        fields = [bt.get_fields(k) for k in range(len(specs))]
    assert rc == 0
    for k, sp in enumerate(specs):
        cfg = cnv.default_config(nx=sp["n"], ny=sp["n"], Re=sp["Re"], u4=sp["lid"],
                                 dt=_stable_dt(sp["n"], sp["Re"], sp["lid"]), precision=cnv.PREC_MIXED,
                                 mixed_rtol=1e-10, mixed_warm_start=1)
        with cnv.Cavity(cfg) as cav:
            _, steps = cav.step(nsteps)
            single = cav.get_fields()
        assert last[k]["iters"] == steps[-1]["iters"]
        for name, a, b in zip("w u v psi".split(), fields[k], single):
            assert np.max(np.abs(a - b)) <= SAME_SCHEME_TOL * np.max(np.abs(b)), (k, name)


def _single_mixed(cnv, sp, nsteps, **kw):
    cfg = cnv.default_config(nx=sp["n"], ny=sp["n"], Re=sp["Re"], u4=sp["lid"],
                             dt=_stable_dt(sp["n"], sp["Re"], sp["lid"]), precision=cnv.PREC_MIXED,
                             mixed_rtol=1e-10, **kw)
    with cnv.Cavity(cfg) as cav:
        _, steps = cav.step(nsteps)
        return steps, cav.get_fields()


@pytest.mark.gpu
def test_row_strip_groups_equal_single_cavity_runs(cnv):
    """Cavities split into 2 or 4 row strips (forced on small grids) give the single-cavity
    mixed run's fields: the strips' halo exchange reproduces global red-black sweeps."""
    base = cnv.default_config(mixed_rtol=1e-10)
    nsteps = 3
    with cnv.Batch(base, SPECS) as bt:
        bt.split(4, 1)
        groups = bt.groups()
        rc, last = bt.step(nsteps)
        fields = [bt.get_fields(k) for k in range(len(SPECS))]
    assert rc == 0
    assert groups == [4, 2, 4, 2, 4]
    for k, sp in enumerate(SPECS):
        steps, single = _single_mixed(cnv, sp, nsteps)
        assert last[k]["iters"] == steps[-1]["iters"], k
        for name, a, b in zip("w u v psi".split(), fields[k], single):
            assert np.max(np.abs(a - b)) <= SAME_SCHEME_TOL * np.max(np.abs(b)), (k, name)


@pytest.mark.gpu
def test_tuned_groups_on_large_cavities_equal_single_runs(cnv):
    """The tuner's candidates include group sizes picked by the cost model (any strip count, not
    only powers of two); whichever it keeps, every cavity equals its single-cavity run."""
    specs = [dict(n=384, Re=1500.0, lid=1.2), dict(n=384, Re=200.0, lid=0.6), dict(n=256, Re=300.0, lid=0.7),
             dict(n=256, Re=1900.0, lid=1.4), dict(n=96, Re=900.0, lid=1.0)]
    base = cnv.default_config(mixed_rtol=1e-10)
    nsteps = 2
    with cnv.Batch(base, specs) as bt:
        bt.tune()
        groups = bt.groups()
        rc, last = bt.step(nsteps)
        fields = [bt.get_fields(k) for k in range(len(specs))]
    assert rc == 0 and min(groups[:2]) >= 3 and min(groups[2:4]) >= 2, groups
    for k, sp in enumerate(specs):
        steps, single = _single_mixed(cnv, sp, nsteps)
        assert last[k]["iters"] == steps[-1]["iters"], k
        for name, a, b in zip("w u v psi".split(), fields[k], single):
            assert np.max(np.abs(a - b)) <= SAME_SCHEME_TOL * np.max(np.abs(b)), (k, name)


@pytest.mark.gpu
def test_default_strip_counts_equal_single_cavity_runs(cnv):
    """The cost model's default decomposition of a few large cavities uses more strips than
    shared memory needs (6 for 384^2 on a GB300, not a power of two); every cavity still equals
    its single-cavity run."""
    specs = [dict(n=384, Re=1500.0, lid=1.2), dict(n=256, Re=300.0, lid=0.7), dict(n=192, Re=900.0, lid=1.0)]
    base = cnv.default_config(mixed_rtol=1e-10)
    nsteps = 2
    with cnv.Batch(base, specs) as bt:
        groups = bt.groups()
        rc, last = bt.step(nsteps)
        fields = [bt.get_fields(k) for k in range(len(specs))]
    assert rc == 0 and groups == cnv.batch_plan(specs)[0] and groups[0] == 6, groups
    for k, sp in enumerate(specs):
        steps, single = _single_mixed(cnv, sp, nsteps)
        assert last[k]["iters"] == steps[-1]["iters"], k
        for name, a, b in zip("w u v psi".split(), fields[k], single):
            assert np.max(np.abs(a - b)) <= SAME_SCHEME_TOL * np.max(np.abs(b)), (k, name)


@pytest.mark.gpu
def test_large_cavities_on_their_smallest_strips(cnv):
    specs = [dict(n=384, Re=1500.0, lid=1.2), dict(n=256, Re=300.0, lid=0.7), dict(n=192, Re=900.0, lid=1.0)]
    base = cnv.default_config(mixed_rtol=1e-10)
    nsteps = 2
    with cnv.Batch(base, specs) as bt:
        model = bt.groups()  # the cost model's counts: at least the smallest that fit
        bt.split(1, 256)     # strips only where shared memory needs them
        groups = bt.groups()
        rc, last = bt.step(nsteps)
        fields = [bt.get_fields(k) for k in range(len(specs))]
    # a 384^2 correction needs 3 strips of a GB300 block's shared memory, 256^2 needs 2
    assert rc == 0 and groups == [3, 2, 1]
    assert all(m >= g for m, g in zip(model, groups)) and model[0] > 3, model
    for k, sp in enumerate(specs):
        steps, single = _single_mixed(cnv, sp, nsteps)
        assert last[k]["iters"] == steps[-1]["iters"], k
        for name, a, b in zip("w u v psi".split(), fields[k], single):
            assert np.max(np.abs(a - b)) <= SAME_SCHEME_TOL * np.max(np.abs(b)), (k, name)
