"""The py_feyntrop call surface (py_feyntrop.py of the reference) on the GB300 path.

Same names, arguments, return values and error behaviour as the reference's
front end:

    tropical_integration(N, D0, Lambda, eps_order, edges, replacement_rules,
                         phase_space_point) -> (trop_res, Itr)       py_feyntrop.py:250
    prepare_kinematic_data(edges, replacement_rules, phase_space_point)   :241
    eps_expansion(res, edges, D0)                                         :115
    prefactor(edges, D0, eps_order)                                       :100
    print_res(res)                                                        :68
    sp, eps                                                               :15-16

The reference writes the low-level JSON input (seed 0) and runs ./feyntrop as a
subprocess (py_feyntrop.py:260-291); here the same JSON document goes through the
library in process (feyntrop_gb300.run_json), or through the `feyntrop` command of
this package when use_cli=True.  A failed integration raises RuntimeError, as the
reference does on a non-zero exit status.  Optional keyword arguments beyond the
reference's: precision ("fp64" or "mixed"), seed, use_cli.

Symbolic kinematics use sympy, as in the reference.
"""
import json
import subprocess
from math import log10

from sympy import IndexedBase, gamma, prod, series, symbols, zeros

import feyntrop_gb300 as _ft

sp = IndexedBase("sp")
eps = symbols("eps")

__all__ = ["sp", "eps", "flatten", "vertices", "get_V_ext", "round_res", "print_res", "prefactor", "eps_expansion",
           "to_dict", "replace_all", "replace_sp", "get_m_sqr", "get_P_uv", "prepare_kinematic_data",
           "tropical_integration"]


def flatten(lst):
    """One level of nesting removed."""
    return [x for sub in lst for x in sub]


def vertices(edges):
    """Distinct vertex numbers of an edge list [((v, w), nu, ...), ...]."""
    return list(set(flatten([e[0] for e in edges])))


def get_V_ext(momentum_vars):
    """Number of external vertices: the largest sp index + 2 (the last external
    vertex's momentum follows from conservation)."""
    idx = flatten([list(m[0].indices) for m in momentum_vars])
    return max(idx) + 2


def round_res(res_err):
    """Value and error as strings, rounded two digits past the error's leading zeros."""
    res, err = res_err[0], res_err[1]
    if err == 0:
        return [str(res), str(err)]
    digits = abs(int(log10(err))) + 2
    return ["%.*f" % (digits, round(res, digits)), "%.*f" % (digits, round(err, digits))]


def print_res(res):
    """One line per eps order: [Re +/- dRe] + i * [Im +/- dIm]."""
    re_s = [round_res(r[0]) for r in res]
    im_s = [round_res(r[1]) for r in res]
    w_re = max(len(r[0]) for r in re_s)
    w_ree = max(len(r[1]) for r in re_s)
    w_im = max(len(r[0]) for r in im_s)
    w_ime = max(len(r[1]) for r in im_s)
    print("")
    for i, (r, m) in enumerate(zip(re_s, im_s)):
        print("%-5s[%s +/- %s]  +  i * [%s +/- %s]" % ("-- eps^%d: " % i, r[0].center(w_re), r[1].center(w_ree),
                                                       m[0].center(w_im), m[1].center(w_ime)))


def prefactor(edges, D0, eps_order):
    """Gamma(omega) / prod Gamma(nu_e) with omega = sum nu - L (D0 - 2 eps) / 2."""
    V = len(vertices(edges))
    E = len(edges)
    nu = [e[1] for e in edges]
    L = E - V + 1
    w = sum(nu) - L * (D0 - 2 * eps) / 2
    return gamma(w) / prod([gamma(n) for n in nu])


def eps_expansion(res, edges, D0):
    """prefactor * sum_j (Re_j + i Im_j) eps^j, expanded to the computed order."""
    order = len(res)
    terms = sum(complex(r[0][0], r[1][0]) * eps ** j for j, r in enumerate(res))
    return series(prefactor(edges, D0, order) * terms, eps, 0, order).evalf(10)


def to_dict(phase_space_point):
    """[(name, value), ...] -> {name: str(value)} (later entries win)."""
    return {var: str(val) for var, val in phase_space_point}


def replace_all(expr, dic):
    """Plain string substitution of every key of dic in expr, in the dict's order
    (as the reference does it: names that are prefixes of other names collide)."""
    for k, v in dic.items():
        expr = expr.replace(k, v)
    return expr


def replace_sp(replacement_rules, phase_space_point):
    """[(sp[i,j], expr), ...] with the phase-space values substituted and evaluated."""
    d = to_dict(phase_space_point)
    return [(var, eval(replace_all(str(val), d))) for var, val in replacement_rules]


def get_m_sqr(edges, phase_space_point):
    """Squared mass of every edge: the edge's third entry with the values substituted."""
    d = to_dict(phase_space_point)
    return [eval(replace_all(str(e[2]), d)) for e in edges]


def get_P_uv(edges, phase_space_point, replacement_rules):
    """V x V scalar products: sp[i,j] for the first V_ext-1 external vertices, the last
    external row and column by momentum conservation, zero rows for internal vertices."""
    V = len(vertices(edges))
    P = zeros(V)
    if not replacement_rules:
        return P.tolist()
    n = get_V_ext(replacement_rules) - 1
    for i in range(n):
        for j in range(i, n):
            P[i, j] = sp[i, j]
            P[j, i] = sp[i, j]
    for j in range(n):
        P[n, j] = -sum(P[i, j] for i in range(n))
    for i in range(n + 1):
        P[i, n] = -sum(P[i, j] for j in range(n))
    return P.subs(replace_sp(replacement_rules, phase_space_point)).tolist()


def prepare_kinematic_data(edges, replacement_rules, phase_space_point):
    """(scalar-product matrix, squared masses) of a phase-space point."""
    return get_P_uv(edges, phase_space_point, replacement_rules), get_m_sqr(edges, phase_space_point)


def tropical_integration(N, D0, Lambda, eps_order, edges, replacement_rules, phase_space_point, precision="fp64",
                         seed=0, use_cli=False):
    """The Feynman integral without its Gamma prefactor, as [[[Re, dRe], [Im, dIm]], ...]
    per eps order, and the tropical normalisation I_G^tr."""
    P_uv, m_sqr = prepare_kinematic_data(edges, replacement_rules, phase_space_point)
    graph = [e[:-1] for e in edges]
    P_uv = [[float(x) for x in row] for row in P_uv]
    inp = {"graph": graph, "dimension": D0, "scalarproducts": P_uv, "masses_sqr": m_sqr,
           "num_eps_terms": eps_order, "lambda": Lambda, "N": N, "seed": seed}
    if precision != "fp64":
        inp["precision"] = precision
    print("Starting integration using feyntrop_gb300 with input:")
    print("Graph with edge weights:", graph)
    print("Dimension:", D0)
    print("Scalarproducts (matrix element (u,v) is the scalar product of ext. momentum flowing into vertices u "
          "and v):\n", P_uv)
    print("Squared masses:", m_sqr)
    print("Epsilon order:", eps_order)
    print("Deformation parameter Lambda:", Lambda)
    print("Sample points:", N)
    if use_cli:
        p = subprocess.run([_ft.CLI_PATH], input=json.dumps(inp), capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("An error occurred in the feyntrop core-code. No output was generated.\n" + p.stderr)
        out = json.loads(p.stdout.replace("NaN", "null"))
    else:
        try:
            out = _ft.run_json(inp)
        except _ft.FeyntropError as e:
            raise RuntimeError("An error occurred in the feyntrop core-code. No output was generated.\n" + str(e))
    trop_res, Itr = out["integral"], out["IGtr"]
    print("Prefactor: " + str(prefactor(graph, D0, eps_order)) + ".")
    print_res(trop_res)
    return trop_res, Itr
