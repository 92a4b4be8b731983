"""Per-sample accuracy of the mixed form at scale, against the plain-FP64 form on the
same samples (the FP64 form itself is checked against the oracle in test_gpu_parity).
The FP32 evaluation has a tail: on the benchmark's double box about one sample in
250 000 ends above 1e-5 (the largest seen 1.4e-5), on random box-pentagon kinematics
(deformation angles of tens of radians) a few in 100 000; both are bounded here."""
import numpy as np
import pytest

import feyntrop_gb300 as ft
from feyntrop_gb300 import workloads

pytestmark = pytest.mark.gpu


def errors(plan, n, seed=0):
    rm = plan.records(n, seed=seed, precision=ft.MIXED)
    r6 = plan.records(n, seed=seed, precision=ft.FP64)
    assert (rm["order"] == r6["order"]).all()
    ok = (r6["flags"] & 1) == 0
    assert ((rm["flags"][ok] & 1) == 0).all(), "mixed form dropped a sample the FP64 form kept"
    scale = np.abs(r6["R"][ok]).max(axis=1)
    e = np.abs(rm["R"][ok] - r6["R"][ok]).max(axis=1) / np.where(scale > 0, scale, 1.0)
    return e, (rm["flags"] & 2) != 0


def test_double_box_tail():
    p = ft.Plan(workloads.double_box())
    e, queued = errors(p, 1 << 18)
    assert (e > 1e-5).sum() <= 3, np.sort(e)[-5:]
    assert e.max() <= 2.5e-5, e.max()
    assert np.quantile(e, 0.9999) <= 1e-5
    assert np.median(e) < 1e-6
    assert queued.mean() < 0.005
    p.close()


def test_random_box_pentagon_tail():
    def accept(inp):
        try:
            ft.subgraph_table(inp)
            return True
        except ft.FeyntropError:
            return False

    inputs, _ = workloads.box_pentagon_scan(16, seed=11, accept=accept)
    es, qs = [], []
    for inp in inputs:
        p = ft.Plan(inp)
        e, q = errors(p, 8192, seed=2)
        es.append(e)
        qs.append(q)
        p.close()
    e = np.concatenate(es)
    q = np.concatenate(qs)
    assert np.quantile(e, 0.999) <= 1e-5, np.quantile(e, 0.999)
    assert (e > 1e-5).mean() <= 5e-4, (e > 1e-5).mean()
    assert e.max() <= 2.5e-5, e.max()
    assert q.mean() < 0.03


def test_v_pass_variant_keeps_the_accuracy_with_fewer_fp64_hand_offs():
    """Code variant bit 3 (an autotuner candidate for deformed classes): samples rejected
    only for V's FP32 rounding are re-evaluated with V in two-float instead of going to
    the FP64 pass.  Same accuracy tail, fewer FP64 hand-offs, the same integral."""
    import os

    def accept(inp):
        try:
            ft.subgraph_table(inp)
            return True
        except ft.FeyntropError:
            return False

    inp = workloads.box_pentagon_scan(4, seed=11, accept=accept)[0][1]
    os.environ["FEYNTROP_GB300_VARIANT"] = "13"
    try:
        p = ft.Plan(inp)
        e13, _ = errors(p, 1 << 15, seed=4)
        rec = p.records(1 << 15, seed=4, precision=ft.MIXED)
        r13 = p.integrate(2_000_000, seed=6, precision=ft.MIXED)
        p.close()
    finally:
        del os.environ["FEYNTROP_GB300_VARIANT"]
    p = ft.Plan(inp)
    e5, _ = errors(p, 1 << 15, seed=4)
    r5 = p.integrate(2_000_000, seed=6, precision=ft.MIXED)
    p.close()
    assert ((rec["flags"] & 16) != 0).any(), "no sample took the V pass"
    assert np.quantile(e13, 0.999) <= max(1e-5, 1.5 * np.quantile(e5, 0.999))
    assert e13.max() <= 2.5e-5
    assert r13["fp64_fallback"] < r5["fp64_fallback"]
    assert r13["kept"] + r13["dropped"] == 2_000_000
    for j in range(len(r5["integral"])):
        for part in range(2):
            x, dx = r5["integral"][j][part]
            y = r13["integral"][j][part][0]
            assert abs(x - y) <= 0.02 * dx + 1e-300, (j, part, x, y, dx)
