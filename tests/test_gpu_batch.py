"""Batches (ft_batch_*, ft_integrate_batch): many integrals of several topologies in
one CUDA graph launch, against ft_integrate of each integral on the same samples.

Each integral of a batch walks the same sample stream as ft_integrate with the same
seed and first sample, so the counts of kept, dropped and FP64-re-evaluated samples
agree exactly and the averages agree to the rounding of the sums (their order
differs): to 1e-6 of a standard error in FP64, 1e-3 in mixed precision (the FP32
partial sums of 256 samples round differently when the samples are grouped
differently).
"""
import json
import os

import numpy as np
import pytest

import feyntrop_gb300 as ft
from feyntrop_gb300 import workloads

pytestmark = pytest.mark.gpu

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))
NAMES = ["C1_K4", "C2_double_box", "2L_5pt_box_pent", "C3_box_pentagon_0", "1L_3pt_eucl", "2L_3pt_tutorial",
         "wheel4_vacuum", "ladder3_4pt_mink"]
TOL = {ft.FP64: 1e-6, ft.MIXED: 1e-3}


def assert_same(b, r, precision, what):
    assert b["kept"] == r["kept"] and b["dropped"] == r["dropped"], what
    assert b["fp64_fallback"] == r["fp64_fallback"] and b["exact_steps"] == r["exact_steps"], what
    for j, ((re, dre), (im, dim)) in enumerate(r["integral"]):
        (bre, bdre), (bim, bdim) = b["integral"][j]
        assert abs(bre - re) <= TOL[precision] * dre, (what, j, bre, re, dre)
        assert abs(bdre - dre) <= 1e-3 * dre, (what, j, bdre, dre)
        if dim == 0:
            assert bim == 0 and bdim == 0, what
        else:
            assert abs(bim - im) <= TOL[precision] * dim, (what, j, bim, im, dim)


@pytest.fixture(scope="module")
def plans():
    ps = [ft.Plan(PINS["cases"][n]["input"]) for n in NAMES]
    yield ps
    for p in ps:
        p.close()


@pytest.mark.parametrize("precision", [ft.FP64, ft.MIXED])
def test_batch_equals_single_integrals(plans, precision):
    Ns = [1_500_000, 700_001, 1_000_003, 333_333, 2_000_000, 123_457, 999_999, 800_001]
    seeds = [0, 1, 2, 3, 4, 5, 6, 7]
    b = ft.Batch(plans, precision)
    out = b.run(Ns, seeds)
    info = b.info()
    assert info["num_integrals"] == len(plans)
    assert info["num_classes"] == len(set(NAMES))   # all topologies differ here
    for i, p in enumerate(plans):
        r = p.integrate(Ns[i], seed=seeds[i], precision=precision)
        assert_same(out[i], r, precision, NAMES[i])
    b.close()


def test_batch_is_reusable_with_new_seeds_and_offsets(plans):
    b = ft.Batch(plans, ft.MIXED)
    b.run(200_000, seeds=1)
    captures = b.info()["graph_captures"]
    out = b.run(150_000, seeds=9, first_samples=[0, 10, 20, 30, 40, 50, 60, 70])
    assert b.info()["graph_captures"] == captures   # fewer items than before: graph replayed
    for i, p in enumerate(plans):
        r = p.integrate(150_000, seed=9, precision=ft.MIXED, first_sample=10 * i)
        assert_same(out[i], r, ft.MIXED, NAMES[i])
    out = b.run(2_500_000, seeds=2)           # more items: buffers grow, graph recaptured
    assert b.info()["graph_captures"] == captures + 1
    r = plans[1].integrate(2_500_000, seed=2, precision=ft.MIXED)
    assert_same(out[1], r, ft.MIXED, NAMES[1])
    b.close()


def test_integrate_batch_splits_precisions(plans):
    ps = plans[:4]
    N = [300_000] * 4
    precs = [ft.FP64, ft.MIXED, ft.MIXED, ft.FP64]
    n = len(ps)
    import ctypes
    arr = (ctypes.c_void_p * n)(*[p.h.value for p in ps])
    opts = (ft.RunOptions * n)(*[ft.RunOptions(N[i], 3, 0, precs[i], None) for i in range(n)])
    ras = [ft._ResultArrays(p.K) for p in ps]
    res = (ft.Result * n)(*[r.res for r in ras])
    rc = ft.lib().ft_integrate_batch(ctypes.cast(arr, ctypes.c_void_p), n, ctypes.cast(opts, ctypes.c_void_p),
                                     ctypes.cast(res, ctypes.c_void_p))
    assert rc == ft.FT_OK, ft.lib().ft_last_error()
    for i, p in enumerate(ps):
        ras[i].res = res[i]
        b = ras[i].as_dict(p.info["IGtr"])
        r = p.integrate(N[i], seed=3, precision=precs[i])
        assert_same(b, r, precs[i], NAMES[i])


def test_sharded_batch_blocks_merge_to_one_run(plans):
    """The GPU side of a sharded batch (feyntrop_gb300.shard.batch_sharded, mode
    "samples"): the two ranks' sample blocks of every integral, run as batches and
    merged, equal one run of the whole batch (the same samples; sums to rounding)."""
    from feyntrop_gb300 import shard
    b = ft.Batch(plans, ft.FP64)
    Ns = [300_001, 200_000, 250_003, 100_000, 400_000, 50_001, 300_000, 120_001]
    full = b.run(Ns, seeds=5)
    blocks = []
    for r in range(2):
        fc = [shard.split_samples(N, r, 2) for N in Ns]
        blocks.append(b.run([c for _, c in fc], seeds=5, first_samples=[f for f, _ in fc]))
    for i, p in enumerate(plans):
        m = shard.merge_moments([blocks[0][i]["moments"], blocks[1][i]["moments"]])
        assert [x[0] for x in m] == [x[0] for x in full[i]["moments"]], NAMES[i]
        merged = ft.finalize_moments(m, p.K, real_only=not p.info["deformed"])
        for j, ((re, dre), (im, dim)) in enumerate(full[i]["integral"]):
            (mre, mdre), (mim, mdim) = merged[j]
            assert abs(mre - re) <= 1e-6 * dre and abs(mdre - dre) <= 1e-6 * dre, (NAMES[i], j)
            assert abs(mim - im) <= 1e-6 * max(dim, 1e-300) or (dim == 0 and mim == 0), (NAMES[i], j)
    b.close()


@pytest.mark.parametrize("mode", ["samples", "integrals"])
def test_run_sharded_on_one_rank_equals_run(plans, mode):
    """Batch.run_sharded with a single rank (no process group needed) takes the sharded
    path end to end and returns the whole batch's results: the same counts and, to
    rounding, the same integrals as Batch.run."""
    b = ft.Batch(plans, ft.FP64)
    Ns = [200_000 + 1000 * i for i in range(len(plans))]
    full = b.run(Ns, seeds=4)
    sh = b.run_sharded(Ns, rank=0, world=1, seeds=4, mode=mode)
    for i, p in enumerate(plans):
        assert sh[i]["samples"] == Ns[i]
        assert [m[0] for m in sh[i]["moments"]] == [m[0] for m in full[i]["moments"]], NAMES[i]
        for j, ((re, dre), (im, dim)) in enumerate(full[i]["integral"]):
            (sre, sdre), (sim, sdim) = sh[i]["integral"][j]
            assert abs(sre - re) <= 1e-9 * max(dre, 1e-300) and abs(sdre - dre) <= 1e-9 * dre, (NAMES[i], j)
            assert abs(sim - im) <= 1e-9 * max(dim, 1e-300) or (dim == 0 and sim == 0), (NAMES[i], j)
    b.close()


def test_batch_runs_are_bit_identical():
    """The FP64 pass of a mixed batch adds its samples into exact fixed-point
    accumulators, so the order in which the queue's entries are handled does not
    matter: the same batch run twice gives bit-identical sums.  The double box at its
    Minkowski point without the deformation (lambda = 0, one eps order; the reference
    accepts it) has V changing sign inside the domain, and the FP32 evaluation hands
    every sample with V near or below zero to the FP64 pass; deformed integrals beside it."""
    undeformed = dict(workloads.double_box(N=1000, lam=0.0), num_eps_terms=1)
    names = ["double box, lambda 0", "2L_3pt_tutorial", "C3_box_pentagon_1", "1L_3pt_mink"]
    ps = [ft.Plan(undeformed)] + [ft.Plan(PINS["cases"][n]["input"]) for n in names[1:]]
    assert not ps[0].info["deformed"]
    b = ft.Batch(ps, ft.MIXED)
    Ns = [2_000_000, 2_000_000, 1_000_000, 500_000]
    first = b.run(Ns, seeds=[1, 2, 3, 4])
    second = b.run(Ns, seeds=[1, 2, 3, 4])
    assert first[0]["fp64_fallback"] > 10_000
    for a, c, n in zip(first, second, names):
        assert a["kept"] == c["kept"] and a["dropped"] == c["dropped"], n
        assert a["moments"] == c["moments"], n
        assert a["integral"] == c["integral"], n
    b.close()
    for p in ps:
        p.close()


def test_kinematic_scan_batch():
    """64 random box-pentagon points (their own masses, invariants, lambda and N) in one
    persistent launch, each against its own ft_integrate."""
    def accept(inp):
        try:
            ft.subgraph_table(inp)
            return True
        except ft.FeyntropError:
            return False

    inputs, _ = workloads.box_pentagon_scan(64, seed=11, accept=accept)
    ps = [ft.Plan(x) for x in inputs]
    Ns = [min(x["N"], 400_000) for x in inputs]
    b = ft.Batch(ps, ft.MIXED)
    out = b.run(Ns, seeds=list(range(64)))
    classes = b.info()["num_classes"]
    assert classes <= 2    # deformed, and possibly a pseudo-Euclidean point
    for i, p in enumerate(ps):
        r = p.integrate(Ns[i], seed=i, precision=ft.MIXED)
        assert_same(out[i], r, ft.MIXED, "scan %d" % i)
    b.close()
    for p in ps:
        p.close()


def test_batch_matches_reference_aggregates():
    """The reference's own N = 2e5 aggregates (same samples, seed 0) through a batch."""
    names = ["1L_2pt", "1L_3pt_mink", "2L_4pt_ladder", "C4_cube", "K4_masses_1to6"]
    ps = [ft.Plan(PINS["cases"][n]["input"]) for n in names]
    N = PINS["N_aggregate"]
    out = ft.Batch(ps, ft.FP64).run(N, seeds=0)
    for i, n in enumerate(names):
        for j, ((re, dre), (im, dim)) in enumerate(PINS["cases"][n]["aggregate"]["integral"]):
            g_re, g_dre = out[i]["integral"][j][0]
            assert abs(g_re - re) <= 1e-6 * dre, (n, j, g_re, re)
            assert abs(g_dre - dre) <= 1e-6 * dre
    for p in ps:
        p.close()


def test_plans_create_matches_single_creation_and_reports_failures():
    inputs = [PINS["cases"][n]["input"] for n in NAMES]
    bad = dict(inputs[0], graph=[[[0, 0], 1]] + inputs[0]["graph"][1:])   # a tadpole: invalid argument
    ps = ft.create_plans(inputs + [bad], skip_failed=True)
    assert ps[-1] is None
    for p, x in zip(ps[:-1], inputs):
        q = ft.Plan(x)
        assert p.info["IGtr"] == q.info["IGtr"] and p.info["deformed"] == q.info["deformed"]
        a = p.integrate(100_000, seed=4, precision=ft.MIXED)
        b = q.integrate(100_000, seed=4, precision=ft.MIXED)
        assert_same(a, b, ft.MIXED, "create_plans")
        q.close()
    with pytest.raises(ft.FeyntropError) as e:
        ft.create_plans([bad])
    assert "problem 0" in str(e.value) and "tadpole" in str(e.value)
    assert e.value.code == ft.FT_ERR_INVALID_ARGUMENT


def test_autotune_records_a_shape_and_keeps_the_samples():
    """The autotuner only changes launch shapes: the same samples give the same counts
    and the same integral after it recorded its choice."""
    p = ft.Plan(PINS["cases"]["C1_K4"]["input"])
    before = p.integrate(300_000, seed=8, precision=ft.MIXED)
    t = p.autotune(ft.MIXED, samples=1_000_000)
    assert t["candidates"] >= 4 and t["samples_per_second"] > 0
    assert t["block"] in (64, 128, 256, 384, 512) and t["variant"] in range(32)
    assert t["samples_per_second"] >= t["default_samples_per_second"]
    assert t["batch_chunk"] in (32, 64, 128, 256) and t["batch_samples_per_second"] > 0
    after = p.integrate(300_000, seed=8, precision=ft.MIXED)
    assert_same(after, before, ft.MIXED, "after autotune")
    p.close()


def test_run_to_accuracy_reaches_the_target_on_the_same_samples(plans):
    """Variance-adaptive N: every integral ends at (about) the requested relative error,
    and the merged pilot + continuation equals one run over the same samples."""
    b = ft.Batch(plans, ft.MIXED)
    out = b.run_to_accuracy(0.02, pilot=20_000, max_samples=5_000_000, seeds=3)
    for i, r in enumerate(out):
        (re, dre), (im, dim) = r["integral"][0]
        scale = max(abs(re), abs(im))
        if r["samples"] < 5_000_000:
            assert max(dre, dim) <= 0.03 * scale, (NAMES[i], r["samples"], re, dre, im, dim)
        single = plans[i].integrate(r["samples"], seed=3, precision=ft.MIXED)
        assert_same(r, single, ft.MIXED, NAMES[i])
    b.close()


def test_choose_lambda_finds_the_low_variance_contour():
    """The double box at lambda = 0.5 (the benchmark's value) has a per-sample spread
    that swamps the integral; pilot runs pick a lambda whose estimate is precise, and
    the integral at it agrees with the estimates at neighbouring lambdas."""
    inp = workloads.double_box(N=1000)
    (lam, rel, table), = ft.choose_lambda([inp], candidates=(0.1, 0.2, 0.3, 0.5), pilot=300_000)
    assert lam in (0.1, 0.2, 0.3) and rel < 0.05 < table[0.5], table
    vals = []
    for l in (0.1, 0.2, 0.3):
        p = ft.Plan(dict(inp, **{"lambda": l}))
        r = p.integrate(2_000_000, seed=1, precision=ft.MIXED)
        vals.append(r["integral"][0])
        p.close()
    (re0, d0), (im0, e0) = vals[1]
    for (re, d), (im, e) in vals:
        assert abs(re - re0) <= 5 * (d + d0) and abs(im - im0) <= 5 * (e + e0), vals
