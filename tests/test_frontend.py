"""The drop-in surfaces: the py_feyntrop call surface (feyntrop_gb300.py_feyntrop) and
the `feyntrop` command with the reference's JSON contract."""
import json
import os
import subprocess

import pytest

import feyntrop_gb300 as ft

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))


def symbolic(name):
    sym = PINS["suite_symbolic"][name]
    pf = pytest.importorskip("feyntrop_gb300.py_feyntrop")
    edges = [(tuple(e[0]), e[1], e[2]) for e in sym["edges"]]
    rules = [(pf.sp[i, j], expr) for i, j, expr in sym["rules"]]
    point = [tuple(p) for p in sym["point"]]
    return pf, edges, rules, point, sym


@pytest.mark.parametrize("name", sorted(PINS["suite_symbolic"]))
def test_kinematic_data_equals_the_reference_front_end(name):
    pytest.importorskip("sympy")
    pf, edges, rules, point, sym = symbolic(name)
    P, m2 = pf.prepare_kinematic_data(edges, rules, point)
    ref = PINS["cases"][name]["input"]
    assert [[float(x) for x in row] for row in P] == ref["scalarproducts"]
    assert [float(x) for x in m2] == ref["masses_sqr"]


def test_prefactor_and_expansion():
    pytest.importorskip("sympy")
    pf, edges, rules, point, sym = symbolic("1L_2pt")
    graph = [e[:-1] for e in edges]
    # one loop, nu = 1, 2, D0 = 4: omega = 3 - (4 - 2 eps)/2 = 1 + eps; Gamma(1+eps)/(Gamma(1)Gamma(2))
    assert abs(float(pf.prefactor(graph, 4, 1).subs(pf.eps, 0)) - 1.0) < 1e-15
    res = [[[1.0, 0.1], [0.0, 0.0]], [[2.0, 0.1], [0.5, 0.1]]]
    series = pf.eps_expansion(res, graph, 4)
    assert abs(complex(series.coeff(pf.eps, 0)) - 1.0) < 1e-9


def test_print_res_format(capsys):
    pytest.importorskip("sympy")
    import feyntrop_gb300.py_feyntrop as pf
    pf.print_res([[[1.2345678, 0.0012], [0.0, 0.0]]])
    out = capsys.readouterr().out
    assert "-- eps^0:" in out and "1.2346" in out and "0.0012" in out and "+/-" in out


def test_cli_reports_bad_input_like_the_reference():
    inp = dict(PINS["cases"]["C1_K4"]["input"])
    del inp["N"]
    p = subprocess.run([ft.CLI_PATH], input=json.dumps(inp), capture_output=True, text=True)
    assert p.returncode != 0 and p.stdout == ""
    assert "must contain the data fields" in p.stderr
    p = subprocess.run([ft.CLI_PATH], input="{not json", capture_output=True, text=True)
    assert p.returncode != 0


@pytest.mark.gpu
def test_cli_and_in_process_agree():
    inp = dict(PINS["cases"]["K4_masses_1to6"]["input"], N=100000)
    p = subprocess.run([ft.CLI_PATH], input=json.dumps(inp), capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    cli = json.loads(p.stdout)
    mem = ft.run_json(inp)
    assert cli["integral"] == mem["integral"] and cli["IGtr"] == mem["IGtr"] == 84.0
    assert "Euclidean" in p.stderr


@pytest.mark.gpu
def test_tropical_integration_surface():
    pytest.importorskip("sympy")
    pf, edges, rules, point, sym = symbolic("1L_3pt_eucl")
    res, Itr = pf.tropical_integration(200000, sym["D0"], sym["Lambda"], sym["eps_order"], edges, rules, point)
    agg = PINS["cases"]["1L_3pt_eucl"]["aggregate"]
    assert Itr == agg["IGtr"]
    for j, ((re, dre), (im, dim)) in enumerate(agg["integral"]):
        assert abs(res[j][0][0] - re) <= 1e-6 * dre
    with pytest.raises(RuntimeError):
        pf.tropical_integration(1000, sym["D0"], sym["Lambda"], sym["eps_order"],
                                [((0, 0), 1, "mm0")] + edges[1:], rules, point)
