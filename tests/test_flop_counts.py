"""The operation counts behind the benchmark's roofline: the counting scalar runs the
same restatement (its values equal the oracle's), and the committed table
profiles/flop_counts.txt is what tests/golden/make_flop_counts.py produces."""
import importlib.util
import os

import numpy as np

import oracle_lib as ol
from feyntrop_gb300 import workloads

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _generator():
    spec = importlib.util.spec_from_file_location("make_flop_counts",
                                                  os.path.join(REPO, "tests", "golden", "make_flop_counts.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m


def test_counted_run_is_the_oracle_run():
    for inp in (workloads.k4_euclidean(), workloads.double_box(), workloads.cube_propagator()):
        p = ol.Prepared(inp)
        c = p.count_ops(5, 100, 500, values=True)
        ref = p.samples(5, 100, 500)
        ok = ~ref["dropped"]
        assert c["dropped"] == (~ok).sum()
        scale = np.abs(ref["R"][ok]).max(axis=1, keepdims=True)
        assert (np.abs(c["R"][ok] - ref["R"][ok]) / scale).max() < 1e-12


def test_counts_are_additive_and_stable():
    p = ol.Prepared(workloads.double_box())
    a = p.count_ops(0, 0, 300)
    b = p.count_ops(0, 300, 300)
    ab = p.count_ops(0, 0, 600)
    for k in ("add", "mul", "div", "sqrt", "trans"):
        assert a[k] + b[k] == ab[k]
        assert a[k] > 0 or k == "sqrt"


def test_committed_table_matches_a_fresh_count():
    gen = _generator()
    rows = {}
    for line in open(os.path.join(REPO, "profiles", "flop_counts.txt")):
        if line.startswith("#") or not line.strip():
            continue
        f = line.split()
        rows[f[0]] = [float(x) for x in f[1:]]
    names = [n for n, _ in gen.cases()]
    assert sorted(rows) == sorted(names)
    for name, inputs in gen.cases():
        if name not in ("k4", "double_box", "triangle"):
            continue
        per, n = gen.count(inputs)
        r = rows[name]
        assert int(r[-1]) == n
        assert abs(r[9] - per["flops"]) <= 0.051, (name, r[9], per["flops"])
