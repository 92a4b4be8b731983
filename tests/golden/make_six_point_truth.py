"""Regenerates tests/golden/six_point_truth.json: 50-digit values of the samples where
the oracle's FP64 evaluation is not exact, for the deformed six-point graphs of
tests/test_gpu_edge.py.

    python tests/golden/make_six_point_truth.py [processes]

For each graph it evaluates the first 4096 samples of stream 0 with the oracle (the
FP64 restatement of the reference's loop) and with tests/hp_truth.py (the reference's
formulas at 50 significant digits, mpmath), and records every sample whose oracle
value is more than 1e-11 (relative to its largest component) from the 50-digit one:
its index, both values and that error.  In these ill-conditioned sectors the
reference's own FP64 arithmetic is the inaccurate side, so the GPU test referees its
disagreements with the oracle there against the 50-digit values.  Runs on the CPU
(mpmath, the oracle library built by `make -C oracle oracle`); about a minute on 8
processes.
"""
import json
import multiprocessing
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
REPO = os.path.dirname(TESTS)
N_SAMPLES = 4096
LAMBDA = 0.5
GRAPHS = {
    "hexagon": [[[i, (i + 1) % 6], 1] for i in range(6)],
    "six_point_double_box": [[[0, 1], 1], [[1, 2], 1], [[2, 3], 1], [[3, 4], 1], [[4, 5], 1], [[5, 0], 1],
                             [[1, 4], 1]],
}


def six_point_input(graph, seed):
    """The input of tests/test_gpu_edge.py::six_point (kept identical)."""
    import random
    sys.path.insert(0, REPO)
    from feyntrop_gb300.workloads import kinematic_matrix
    rng = random.Random(seed)
    sp = {(i, j): (rng.uniform(0.5, 3) if i == j else rng.uniform(-5, 5)) for i in range(5) for j in range(i, 5)}
    return {"graph": graph, "dimension": 6, "scalarproducts": kinematic_matrix(6, sp),
            "masses_sqr": [rng.uniform(0.5, 2) for _ in graph], "num_eps_terms": 2, "lambda": LAMBDA, "N": 1000,
            "seed": 0}


def referee(args):
    name, indices = args
    sys.path.insert(0, TESTS)
    import hp_truth
    import oracle_lib as ol
    inp = six_point_input(GRAPHS[name], 11)
    prep = ol.Prepared(inp)
    s = prep.samples(0, 0, N_SAMPLES)
    info = {"W": prep.W, "IGtr": prep.IGtr, "loops": prep.loops, "lambda_used": LAMBDA, "deformed": True}
    out = []
    for i in indices:
        if s["dropped"][i]:
            continue
        t = np.array(hp_truth.truth(inp, info, s["X"][i], s["psi_tr"][i], s["xi_tr"][i]))
        scale = np.abs(t).max()
        err = float(np.abs(s["R"][i] - t).max() / scale)
        if err > 1e-11:
            out.append({"index": int(i), "oracle_error": err,
                        "truth": [[float(z.real), float(z.imag)] for z in t],
                        "oracle": [[float(z.real), float(z.imag)] for z in s["R"][i]]})
    return out


def main():
    procs = int(sys.argv[1]) if len(sys.argv) > 1 else 8
    ctx = multiprocessing.get_context("spawn")
    result = {"n_samples": N_SAMPLES, "seed": 0, "cases": {}}
    for name in GRAPHS:
        parts = [(name, list(range(k, N_SAMPLES, 32))) for k in range(32)]
        with ctx.Pool(procs) as pool:
            rows = [r for part in pool.map(referee, parts) for r in part]
        rows.sort(key=lambda r: r["index"])
        result["cases"][name] = rows
        print(name, [(r["index"], "%.1e" % r["oracle_error"]) for r in rows])
    with open(os.path.join(HERE, "six_point_truth.json"), "w") as f:
        json.dump(result, f, indent=1)


if __name__ == "__main__":
    main()
