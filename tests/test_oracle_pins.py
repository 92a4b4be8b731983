"""The CPU oracle against the reference's own outputs (tests/golden/reference_pins.json,
generated from the reference build by tests/golden/make_golden.py).

Bit-exact: the J(gamma) table, the regime flags, the sector draws (removal order,
X, psi_tr, xi_tr) over 20000 consecutive draws.  Within tolerance: per-sample
integrand values (the reference's FP64 path differs only by its library's
operation order and fast-math contraction) and the single-thread integral.
"""
import hashlib
import json
import os

import numpy as np
import pytest

import oracle_lib as ol

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))
CASES = sorted(PINS["cases"])
PER_SAMPLE_RTOL = 1e-10   # relative to |R| of the sample, per eps order


def hx(x):
    return "%016x" % np.float64(x).view(np.uint64)


@pytest.fixture(scope="module", params=CASES)
def case(request):
    c = PINS["cases"][request.param]
    return request.param, c, ol.Prepared(c["input"])


def test_table_bit_exact(case):
    name, c, p = case
    Jr, r, mm, L = p.table()
    blob = "".join(hx(x) for x in Jr) + "".join(hx(x) for x in r) + "".join(str(int(x)) for x in mm) + "".join(
        str(int(x)) for x in L)
    assert hashlib.sha256(blob.encode()).hexdigest() == c["table"]["sha256"]
    t = c["table"]
    assert (p.gp, p.pseudo_euclidean, p.generic, p.euclidean) == (t["gp"], t["pseudo_euclidean"], t["generic"],
                                                                    t["euclidean"])
    assert hx(p.W) == t["W"] and hx(p.IGtr) == t["IGtr"]


def test_sectors_bit_exact(case):
    name, c, p = case
    n = c["orders_count"]
    s = p.samples(0, 0, n)
    orders = ",".join("".join("%x" % e for e in o) for o in s["order"])
    assert hashlib.sha256(orders.encode()).hexdigest() == c["orders_sha256"]
    for i, sec in enumerate(c["sectors"]):
        assert [hx(x) for x in s["X"][i]] == sec["X"]
        assert hx(s["psi_tr"][i]) == sec["psi_tr"] and hx(s["xi_tr"][i]) == sec["xi_tr"]
        assert list(s["order"][i]) == sec["order"]


def test_per_sample_values(case):
    name, c, p = case
    for seed, vals in enumerate(c["per_sample_seed0"]):
        o = p.samples(seed, 0, 1)
        for j, (re, im) in enumerate(vals):
            if re is None:
                assert o["dropped"][0]
                continue
            R = o["R"][0, j]
            scale = abs(R)
            assert abs(R.real - re) <= PER_SAMPLE_RTOL * scale, (seed, j, R, re)
            assert abs(R.imag - im) <= PER_SAMPLE_RTOL * scale, (seed, j, R, im)


def test_single_thread_integral(case):
    name, c, p = case
    out, kept, dropped = p.integrate(PINS["N_aggregate"], 0, 4)
    for j, ((re, dre), (im, dim)) in enumerate(c["aggregate"]["integral"]):
        # same samples, so the averages agree far inside the statistical error
        assert abs(out[j, 0] - re) <= 1e-6 * dre, (j, out[j], re)
        assert abs(out[j, 2] - im) <= 1e-6 * max(dim, 1e-300) or (im == 0 and out[j, 2] == 0)
        assert abs(out[j, 1] - dre) <= 1e-6 * dre
        assert abs(out[j, 3] - dim) <= 1e-6 * max(dim, 1e-300) or (dim == 0 and out[j, 3] == 0)


def test_thread_count_does_not_change_the_samples():
    c = PINS["cases"]["C1_K4"]
    p = ol.Prepared(c["input"])
    a, _, _ = p.integrate(20000, 7, 1)
    b, _, _ = p.integrate(20000, 7, 5)
    assert np.allclose(a, b, rtol=1e-13, atol=0)


def test_skip_matches_stepping():
    p = ol.Prepared(PINS["cases"]["C1_K4"]["input"])
    s = p.samples(11, 0, 40)
    t = p.samples(11, 37, 3)
    assert (s["order"][37:] == t["order"]).all()
    assert (s["X"][37:] == t["X"]).all()
