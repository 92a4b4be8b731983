"""Regenerates tests/golden/reference_pins.json from the reference itself.

Run with FEYNTROP_REFERENCE naming a checkout of the reference's sources, after
`make -C oracle ref REF=$FEYNTROP_REFERENCE`:

    python tests/golden/make_golden.py                # every case
    python tests/golden/make_golden.py --only NAME..  # these cases, merged into the pins

For every case below it records, from the reference build (oracle/_ref):
  * the J(gamma) table of generate_subgraph_table (full table as IEEE bit patterns
    for E <= 8, a SHA-256 of it otherwise) with W, IGtr and the regime flags;
  * the first sector draws of stream 0 (removal order, X, psi_tr, xi_tr) and a
    SHA-256 of the removal orders of the first 20000 draws;
  * per-sample integrand values: the stock binary run with N=1 and
    OMP_NUM_THREADS=1 for seeds 0..31 (its printed average is that sample);
  * the single-thread integral (N=200000, seed 0) printed by the stock binary.
It also carries the reference's own test-suite expectations (tests/*.txt with
the inputs of tests/test_suite.py), converted with the reference's
py_feyntrop.prepare_kinematic_data.
"""
import ast
import hashlib
import json
import math
import os
import random
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = os.environ.get("FEYNTROP_REFERENCE")
if not REF or not os.path.isdir(os.path.join(REF, "srcs")):
    sys.exit("make_golden.py: set FEYNTROP_REFERENCE to a checkout of the reference (its srcs/ and "
             "py_feyntrop.py), and build oracle/_ref with `make -C oracle ref REF=$FEYNTROP_REFERENCE`")
REF_BIN = os.path.join(REPO, "oracle", "_ref", "feyntrop")
HARNESS = os.path.join(REPO, "oracle", "_ref", "ref_harness")

sys.path.insert(0, REF)
import py_feyntrop as ref_py  # noqa: E402  (the reference's own front end)
from py_feyntrop import sp  # noqa: E402

N_AGG = 200000
N_SECTOR_HASH = 20000
N_SECTOR_DUMP = 32
SEEDS = list(range(32))


SYMBOLIC = {}


def kin_input(edges, rules, point, D, K, lam, N=1000, seed=0, name=None):
    if name:
        # the front end's own arguments, for checking a re-implementation of it
        SYMBOLIC[name] = {"edges": [[list(e[0]), e[1], str(e[2])] for e in edges],
                          "rules": [[int(r[0].indices[0]), int(r[0].indices[1]), str(r[1])] for r in rules],
                          "point": [[k, v] for k, v in point], "D0": D, "eps_order": K, "Lambda": lam}
    P, m2 = ref_py.prepare_kinematic_data(edges, rules, point)
    return {
        "graph": [[list(e[0]), e[1]] for e in edges],
        "dimension": D,
        "scalarproducts": [[float(x) for x in row] for row in P],
        "masses_sqr": [float(x) for x in m2],
        "num_eps_terms": K,
        "lambda": lam,
        "N": N,
        "seed": seed,
    }


def suite_cases():
    """The seven inputs of the reference's tests/test_suite.py:47-117."""
    c = {}
    c["1L_2pt"] = (kin_input([((0, 1), 1, "mm0"), ((0, 1), 2, "mm1")], [(sp[0, 0], "pp")],
                             [("mm0", 0.2), ("mm1", 1.2), ("pp", 3)], 4, 5, 1, name="1L_2pt"))
    tri = [((0, 1), 1, "mm0"), ((1, 2), 1, "mm1"), ((2, 0), 1, "mm2")]
    tri_rules = [(sp[0, 0], "pp0"), (sp[1, 1], "pp1"), (sp[0, 1], "(s01-pp0-pp1)/2")]
    c["1L_3pt_eucl"] = kin_input(tri, tri_rules, [("mm0", 0.2), ("mm1", 1.2), ("mm2", 2.2), ("pp0", -4),
                                                  ("pp1", -5), ("s01", -13)], 4, 5, 1, name="1L_3pt_eucl")
    c["1L_3pt_mink"] = kin_input(tri, tri_rules, [("mm0", 0.01), ("mm1", 0.5), ("mm2", 1), ("pp0", 1),
                                                  ("pp1", 4), ("s01", 3)], 4, 5, 1, name="1L_3pt_mink")
    c["2L_2pt_ladder"] = kin_input(
        [((0, 2), 1, "mm0"), ((0, 3), 1, "mm1"), ((1, 2), 1, "mm2"), ((1, 3), 1, "mm3"), ((2, 3), 1, "mm4")],
        [(sp[0, 0], "pp")], [("mm0", 0.1), ("mm1", 0.2), ("mm2", 0.3), ("mm3", 0.4), ("mm4", 0.5), ("pp", 3)],
        4, 4, 0.5, name="2L_2pt_ladder")
    c["2L_4pt_ladder"] = kin_input(
        [((0, 1), 1, "0"), ((0, 4), 1, "0"), ((1, 5), 1, "0"), ((5, 4), 1, "0"), ((5, 2), 1, "0"),
         ((4, 3), 1, "0"), ((3, 2), 1, "0")],
        [(sp[0, 0], "pp0"), (sp[1, 1], "pp1"), (sp[2, 2], "pp2"), (sp[0, 1], "(s01-pp0-pp1)/2"),
         (sp[0, 2], "(s02-pp0-pp2)/2"), (sp[1, 2], "(s12-pp1-pp2)/2")],
        [("pp0", 1.2), ("pp1", 1.3), ("pp2", 1.4), ("s01", 2.1), ("s02", 2.2), ("s12", 2.3)], 4, 5, 1, name="2L_4pt_ladder")
    c["2L_3pt_tutorial"] = kin_input(
        [((0, 1), 1, "mm"), ((1, 3), 1, "mm"), ((3, 2), 1, "mm"), ((2, 0), 1, "mm"), ((0, 3), 1, "mm")],
        [(sp[0, 0], "0"), (sp[1, 1], "0"), (sp[0, 1], "s01/2")], [("mm", 0.2), ("s01", 1)], 2, 5, 7.6, name="2L_3pt_tutorial")
    c["2L_5pt_box_pent"] = kin_input(
        [((0, 1), 1, "0"), ((1, 2), 1, "mm"), ((2, 6), 1, "0"), ((6, 3), 1, "mm"), ((3, 4), 1, "0"),
         ((4, 5), 1, "mm"), ((5, 0), 1, "0"), ((5, 6), 1, "mm")],
        [(sp[0, 0], "0"), (sp[1, 1], "mm"), (sp[2, 2], "mm"), (sp[3, 3], "mm"), (sp[0, 1], "(s01-mm)/2"),
         (sp[0, 2], "(s02-mm)/2"), (sp[0, 3], "(s03-mm)/2"), (sp[1, 2], "(s12-2*mm)/2"),
         (sp[1, 3], "(s13-2*mm)/2"), (sp[2, 3], "(s23-2*mm)/2")],
        [("mm", 1 / 2), ("s01", 2.2), ("s02", 2.3), ("s02", 2.3), ("s03", 2.4), ("s12", 2.5), ("s13", 2.6),
         ("s23", 2.7)], 6, 5, 0.28, name="2L_5pt_box_pent")
    return c


def suite_expectations():
    out = {}
    for name in ["1L_2pt", "1L_3pt_eucl", "1L_3pt_mink", "2L_2pt_ladder", "2L_4pt_ladder", "2L_3pt_tutorial",
                 "2L_5pt_box_pent"]:
        with open(os.path.join(REF, "tests", name + ".txt")) as f:
            out[name] = [[list(re), list(im)] for re, im in ast.literal_eval(f.read())]
    return out


def extra_cases():
    """Inputs shaped like the benchmark configurations (seeded)."""
    c = {}
    k4 = [[[0, 1], 1], [[0, 2], 1], [[0, 3], 1], [[1, 2], 1], [[2, 3], 1], [[3, 1], 1]]
    k4P = [[-3, 1, 1, 1], [1, -3, 1, 1], [1, 1, -3, 1], [1, 1, 1, -3]]
    c["K4_masses_1to6"] = {"graph": k4, "dimension": 4, "scalarproducts": k4P, "masses_sqr": [1, 2, 3, 4, 5, 6],
                           "num_eps_terms": 3, "lambda": 0, "N": 1000, "seed": 0}
    c["C1_K4"] = dict(c["K4_masses_1to6"], masses_sqr=[0, 1, 2, 3, 4, 5])

    # double box, externals 0-3 (p_i^2 = 1), internals 4, 5; masses, s, t from Random(1)
    rng = random.Random(1)
    m2 = [rng.uniform(0.5, 2.0) for _ in range(7)]
    s, t = rng.uniform(8, 20), rng.uniform(-6, -1)
    db = [((0, 1), 1, "m0"), ((0, 4), 1, "m1"), ((1, 5), 1, "m2"), ((5, 4), 1, "m3"), ((5, 2), 1, "m4"),
          ((4, 3), 1, "m5"), ((3, 2), 1, "m6")]
    c["C2_double_box"] = kin_input(
        db, [(sp[0, 0], "1"), (sp[1, 1], "1"), (sp[2, 2], "1"), (sp[0, 1], "(S-2)/2"), (sp[1, 2], "(T-2)/2"),
             (sp[0, 2], "(2-S-T)/2")],
        [("m%d" % i, m2[i]) for i in range(7)] + [("S", s), ("T", t)], 4, 2, 0.5)

    # box-pentagon topology with random masses and invariants (first two accepted draws)
    bp = [((0, 1), 1, "m0"), ((1, 2), 1, "m1"), ((2, 6), 1, "m2"), ((6, 3), 1, "m3"), ((3, 4), 1, "m4"),
          ((4, 5), 1, "m5"), ((5, 0), 1, "m6"), ((5, 6), 1, "m7")]
    rng = random.Random(3)
    found = 0
    attempt = 0
    while found < 2 and attempt < 50:
        attempt += 1
        m2 = [rng.uniform(0, 2) for _ in range(8)]
        inv = [rng.uniform(-10, 10) for _ in range(10)]
        lam = rng.uniform(0.2, 1.0)
        pairs = [(i, j) for i in range(4) for j in range(i, 4)]
        rules = [(sp[i, j], "q%d" % n) for n, (i, j) in enumerate(pairs)]
        point = [("m%d" % i, m2[i]) for i in range(8)] + [("q%d" % n, inv[n]) for n in range(10)]
        inp = kin_input(bp, rules, point, 6, 3, lam)
        r = run_ref(inp, 1, 0, check=False)
        if r is not None:
            c["C3_box_pentagon_%d" % found] = inp
            found += 1

    # cube Q3 (5 loops), externals at the antipodal pair 0 and 7 relabelled to 0 and 1
    label = {0: 0, 7: 1}
    for v in range(1, 7):
        label[v] = v + 1
    cube = []
    for a in range(8):
        for b in range(3):
            w = a ^ (1 << b)
            if a < w:
                cube.append([[label[a], label[w]], 1])
    P = [[0.0] * 8 for _ in range(8)]
    P[0][0] = P[1][1] = -1.0
    P[0][1] = P[1][0] = 1.0
    c["C4_cube"] = {"graph": cube, "dimension": 4, "scalarproducts": P, "masses_sqr": [1] * 12,
                    "num_eps_terms": 4, "lambda": 0, "N": 1000, "seed": 0}

    # 3-loop 4-point ladder, Euclidean point: P = -Gram of four momenta summing to 0
    rng = random.Random(5)
    ladder = [[[0, 1], 1], [[4, 5], 1], [[6, 7], 1], [[3, 2], 1], [[0, 4], 1], [[4, 6], 1], [[6, 3], 1],
              [[1, 5], 1], [[5, 7], 1], [[7, 2], 1]]
    q = [[rng.uniform(-1, 1) for _ in range(4)] for _ in range(3)]
    q.append([-(q[0][d] + q[1][d] + q[2][d]) for d in range(4)])
    P = [[0.0] * 8 for _ in range(8)]
    for i in range(4):
        for j in range(4):
            P[i][j] = -sum(q[i][d] * q[j][d] for d in range(4))
    c["ladder3_4pt"] = {"graph": ladder, "dimension": 4, "scalarproducts": P,
                        "masses_sqr": [rng.uniform(0, 3) for _ in range(10)], "num_eps_terms": 3, "lambda": 0,
                        "N": 1000, "seed": 0}

    # the same ladder at a Minkowski point (the deformed class of the mixed batch):
    # on-shell externals p_i^2 = 1, s U[8, 20], t U[-6, -1], masses U[0, 3] from
    # Random(7), lambda = 0.5, through the reference's front end
    rng = random.Random(7)
    m2 = [rng.uniform(0, 3) for _ in range(10)]
    s, t = rng.uniform(8, 20), rng.uniform(-6, -1)
    c["ladder3_4pt_mink"] = kin_input(
        [(tuple(e), nu, "m%d" % i) for i, (e, nu) in enumerate(ladder)],
        [(sp[0, 0], "1"), (sp[1, 1], "1"), (sp[2, 2], "1"), (sp[0, 1], "(S-2)/2"), (sp[1, 2], "(T-2)/2"),
         (sp[0, 2], "(2-S-T)/2")],
        [("m%d" % i, m2[i]) for i in range(10)] + [("S", s), ("T", t)], 4, 3, 0.5)

    # 4-loop wheel vacuum graph, all masses 1, P = 0
    wheel = [[[0, 1], 1], [[1, 2], 1], [[2, 3], 1], [[3, 0], 1], [[0, 4], 1], [[1, 4], 1], [[2, 4], 1],
             [[3, 4], 1]]
    c["wheel4_vacuum"] = {"graph": wheel, "dimension": 4, "scalarproducts": [[0.0] * 5 for _ in range(5)],
                          "masses_sqr": [1.0] * 8, "num_eps_terms": 2, "lambda": 0, "N": 1000, "seed": 0}

    # non-unit, non-integer edge weights: the double box (Minkowski, deformed) and a
    # Euclidean triangle
    nus = [1, 1.5, 1, 2, 1, 0.5, 1]
    c["nu_double_box"] = dict(c["C2_double_box"],
                              graph=[[e[0], nu] for e, nu in zip(c["C2_double_box"]["graph"], nus)])
    c["nu_triangle_eucl"] = {"graph": [[[0, 1], 0.7], [[1, 2], 1.3], [[2, 0], 2]], "dimension": 4,
                             "scalarproducts": [[-1.0, 0.25, 0.75], [0.25, -2.0, 1.75], [0.75, 1.75, -2.5]],
                             "masses_sqr": [0.5, 1.0, 1.5], "num_eps_terms": 3, "lambda": 0, "N": 1000, "seed": 0}

    # odd dimension (half-integer degree of divergence), and a massless box in D = 6
    # with off-shell external legs (Minkowski, deformed)
    c["D3_triangle_eucl"] = dict(c["nu_triangle_eucl"], dimension=3,
                                 graph=[[[0, 1], 1], [[1, 2], 1], [[2, 0], 1]])
    box_sp = {(0, 0): 1.0, (1, 1): 2.0, (2, 2): 1.5, (0, 1): 3.0, (1, 2): -2.0, (0, 2): 0.5}
    n = 3
    P = [[0.0] * 4 for _ in range(4)]
    for (i, j), v in box_sp.items():
        P[i][j] = P[j][i] = v
    for j in range(n):
        P[n][j] = -sum(P[i][j] for i in range(n))
    for i in range(n + 1):
        P[i][n] = -sum(P[i][j] for j in range(n))
    c["massless_box_D6"] = {"graph": [[[0, 1], 1], [[1, 2], 1], [[2, 3], 1], [[3, 0], 1]], "dimension": 6,
                            "scalarproducts": P, "masses_sqr": [0.0] * 4, "num_eps_terms": 2, "lambda": 0.5,
                            "N": 1000, "seed": 0}
    return c


def run_ref(inp, N, seed, threads=1, check=True):
    inp = dict(inp, N=N, seed=seed)
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    p = subprocess.run([REF_BIN], input=json.dumps(inp), capture_output=True, text=True, env=env)
    if p.returncode != 0:
        if check:
            raise RuntimeError(p.stderr)
        return None
    return json.loads(p.stdout.replace("NaN", "null"))


def run_harness(inp, args):
    p = subprocess.run([HARNESS] + args, input=json.dumps(inp), capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS="1"), check=True)
    return json.loads(p.stdout)


def main():
    """All cases, or with `--only name ...` just those, merged into the existing pins."""
    cases = suite_cases()
    cases.update(extra_cases())
    pins = {"generator": "tests/golden/make_golden.py", "N_aggregate": N_AGG, "seeds": SEEDS, "cases": {},
            "suite_expectations": suite_expectations(), "suite_symbolic": SYMBOLIC}
    if "--only" in sys.argv:
        only = sys.argv[sys.argv.index("--only") + 1:]
        with open(os.path.join(HERE, "reference_pins.json")) as f:
            pins = json.load(f)
        cases = {k: v for k, v in cases.items() if k in only}
    for name, inp in cases.items():
        print("case", name, flush=True)
        table = run_harness(inp, ["table"])
        E = table["E"]
        blob = "".join(table["Jr"]) + "".join(table["r"]) + "".join(map(str, table["mm"])) + "".join(
            map(str, table["L"]))
        tab = {k: table[k] for k in ["E", "V", "W", "IGtr", "gp", "pseudo_euclidean", "generic", "euclidean"]}
        tab["sha256"] = hashlib.sha256(blob.encode()).hexdigest()
        if E <= 8:
            tab.update({k: table[k] for k in ["Jr", "r", "mm", "L"]})
        sectors = run_harness(inp, ["sectors", str(N_SECTOR_HASH)])
        orders = ",".join("".join("%x" % e for e in s["order"]) for s in sectors)
        per_sample = []
        for seed in SEEDS:
            r = run_ref(inp, 1, seed)
            per_sample.append([[t[0][0], t[1][0]] for t in r["integral"]])
        agg = run_ref(inp, N_AGG, 0)
        pins["cases"][name] = {
            "input": dict(inp, N=N_AGG, seed=0),
            "table": tab,
            "sectors": sectors[:N_SECTOR_DUMP],
            "orders_sha256": hashlib.sha256(orders.encode()).hexdigest(),
            "orders_count": N_SECTOR_HASH,
            "per_sample_seed0": per_sample,
            "aggregate": {"integral": agg["integral"], "IGtr": agg["IGtr"]},
        }
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(pins, f, indent=None, separators=(",", ":"))
    print("wrote", os.path.join(HERE, "reference_pins.json"))


if __name__ == "__main__":
    main()
