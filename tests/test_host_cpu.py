"""Host-side checks that need no GPU: the C ABI library loads and exports every
declared entry point, the host J(gamma) table equals the oracle's bit for bit,
input validation matches the reference's, and the library refuses to run
without a device instead of falling back to anything."""
import ctypes
import json
import os
import re

import numpy as np
import pytest

import feyntrop_gb300 as ft
import oracle_lib as ol
from feyntrop_gb300 import workloads

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))
HEADER = os.path.join(os.path.dirname(os.path.dirname(__file__)), "include", "feyntrop_gb300.h")


def header_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(ft_\w+)\s*\(", text, re.M)))


def test_every_declared_function_is_exported():
    names = header_functions()
    assert len(names) >= 12
    L = ft.lib()
    for n in names:
        assert hasattr(L, n), n
    assert set(names) <= set(ft.EXPORTED)


@pytest.mark.parametrize("name", sorted(PINS["cases"]))
def test_host_table_equals_oracle(name):
    inp = PINS["cases"][name]["input"]
    Jr, r, mm, L, info = ft.subgraph_table(inp)
    o = ol.Prepared(inp)
    oJr, orr, omm, oL = o.table()
    assert (Jr.view(np.uint64) == oJr.view(np.uint64)).all()
    assert (r.view(np.uint64) == orr.view(np.uint64)).all()
    assert (mm == omm).all() and (L == oL).all()
    assert info["IGtr"] == o.IGtr and info["W"] == o.W
    assert (info["euclidean"], info["pseudo_euclidean"], info["generic"], info["gp_property"]) == (
        o.euclidean, o.pseudo_euclidean, o.generic, o.gp)
    assert bool(info["deformed"]) == (o.def_ref != 0)


def test_probe_generator_is_the_c_library_rand():
    # the product reproduces std::rand() with its default seed for the probe points
    libc = ctypes.CDLL(None)
    libc.srand(1)
    ref = [libc.rand() for _ in range(50)]
    inp = workloads.k4_euclidean()
    # compare through the table: identical mm flags on a case where they matter
    Jr, r, mm, L, info = ft.subgraph_table(PINS["cases"]["C2_double_box"]["input"])
    o = ol.Prepared(PINS["cases"]["C2_double_box"]["input"])
    assert (mm == o.table()[2]).all()
    assert len(ref) == 50 and inp


def bad(inp, **kw):
    x = json.loads(json.dumps(inp))
    x.update(kw)
    return x


@pytest.mark.parametrize("mutate,code,text", [
    (lambda i: bad(i, graph=[[[0, 0], 1], [[0, 1], 1]]), ft.FT_ERR_INVALID_ARGUMENT, "tadpole"),
    (lambda i: bad(i, graph=[[[0, 1], 0], [[0, 2], 1], [[0, 3], 1], [[1, 2], 1], [[2, 3], 1], [[3, 1], 1]]),
     ft.FT_ERR_INVALID_ARGUMENT, "edge weights"),
    (lambda i: bad(i, scalarproducts=[[1, 0, 0, 0], [0, 0, 0, 0], [0, 0, 0, 0], [0, 0, 0, 0]]),
     ft.FT_ERR_DOMAIN, "momentum conservation"),
    (lambda i: bad(i, scalarproducts=[[0, 1, 0, -1], [0, 0, 0, 0], [0, 0, 0, 0], [0, -1, 0, 1]]),
     ft.FT_ERR_DOMAIN, "not symmetric"),
])
def test_invalid_inputs_are_rejected_like_the_reference(mutate, code, text):
    inp = mutate(workloads.k4_euclidean())
    with pytest.raises(ft.FeyntropError) as e:
        ft.subgraph_table(inp)
    assert e.value.code == code and text in str(e.value)
    with pytest.raises(ol.OracleError):
        ol.Prepared(inp)


def test_disconnected_graph_and_subdivergence():
    inp = workloads.k4_euclidean()
    inp["graph"] = inp["graph"] + [[[4, 5], 1]]
    inp["scalarproducts"] = [[0.0] * 6 for _ in range(6)]
    inp["masses_sqr"] = list(inp["masses_sqr"]) + [1.0]
    with pytest.raises(ft.FeyntropError) as e:
        ft.subgraph_table(inp)
    assert "not connected" in str(e.value)
    # massless bubble in D=4 with an eps expansion: UV subdivergence of the full graph is allowed,
    # a D=2 massless 2-loop sunrise subgraph is IR divergent
    sun = {"graph": [[[0, 1], 1], [[0, 1], 1], [[0, 1], 1]], "dimension": 2,
           "scalarproducts": [[1, -1], [-1, 1]], "masses_sqr": [0, 0, 0], "num_eps_terms": 1, "lambda": 0,
           "N": 10, "seed": 0}
    with pytest.raises(ft.FeyntropError) as e:
        ft.subgraph_table(sun)
    with pytest.raises(ol.OracleError):
        ol.Prepared(sun)


def test_json_contract_rejects_missing_keys_without_a_device():
    inp = workloads.k4_euclidean()
    del inp["seed"]
    with pytest.raises(ft.FeyntropError) as e:
        ft.run_json(inp)
    assert "must contain the data fields" in str(e.value)


def test_no_cpu_fallback_without_a_device():
    from conftest import gpu_available
    if gpu_available():
        pytest.skip("a GPU is present")
    with pytest.raises(ft.FeyntropError) as e:
        ft.Plan(workloads.k4_euclidean())
    assert e.value.code == ft.FT_ERR_NO_DEVICE


def test_batch_api_rejects_bad_arguments_without_a_device():
    import ctypes
    L = ft.lib()
    h = ctypes.c_void_p()
    assert L.ft_batch_create(None, 0, ft.MIXED, ctypes.byref(h)) == ft.FT_ERR_INVALID_ARGUMENT
    assert "no plans" in L.ft_last_error().decode()
    arr = (ctypes.c_void_p * 1)(None)
    assert L.ft_batch_create(ctypes.cast(arr, ctypes.c_void_p), 1, 7, ctypes.byref(h)) == ft.FT_ERR_INVALID_ARGUMENT
    assert h.value is None


def test_batch_workloads_are_seeded_and_redraw_rejected_points():
    from feyntrop_gb300 import workloads as w
    a, _ = w.box_pentagon_scan(16, seed=3)
    b, _ = w.box_pentagon_scan(16, seed=3)
    assert a == b
    assert all(1e5 <= x["N"] <= 1e7 for x in a)
    calls = []

    def reject_every_other(inp):
        calls.append(1)
        return len(calls) % 2 == 0

    c, redrawn = w.box_pentagon_scan(8, seed=3, accept=reject_every_other)
    assert redrawn == 8 and len(c) == 8
    m, _ = w.mixed_batch(seed=5, counts=(4, 4, 2, 2))
    assert [len(x["graph"]) for x in m] == [3] * 4 + [10] * 4 + [8] * 2 + [8] * 2
    assert [x["lambda"] for x in m[4:8]] == [0, 0.5, 0, 0.5]


def test_plans_create_without_a_device_reports_no_device():
    import ctypes
    inp = PINS["cases"]["C1_K4"]["input"]
    a = ft._ProblemArrays(inp)
    probs = (ft.Problem * 2)(a.struct, a.struct)
    hs = (ctypes.c_void_p * 2)()
    st = (ctypes.c_int32 * 2)()
    rc = ft.lib().ft_plans_create(ctypes.cast(probs, ctypes.c_void_p), 2, ctypes.cast(hs, ctypes.c_void_p),
                                  ctypes.cast(st, ctypes.c_void_p))
    assert rc == ft.FT_ERR_NO_DEVICE and list(st) == [ft.FT_ERR_NO_DEVICE] * 2
    assert hs[0] is None and hs[1] is None
