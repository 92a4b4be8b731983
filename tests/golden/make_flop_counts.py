"""Writes profiles/flop_counts.txt: floating-point operations per sample of the
reference's sampling loop (sector draw srcs/tropical_sampling.hpp:468-564 and
integrand srcs/feynman_integral.hpp:162-362) for every benchmarked workload, counted
by running the oracle's restatement with its operation-counting scalar
(oracle/opcount.hpp).  The benchmark divides these counts by the sampling kernels'
time for its roofline.

Run from the repository root:  python tests/golden/make_flop_counts.py
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.dirname(HERE))

import oracle_lib as ol  # noqa: E402
from feyntrop_gb300 import workloads  # noqa: E402

SAMPLES = 4000
OUT = os.path.join(REPO, "profiles", "flop_counts.txt")


def cases():
    """(name, list of inputs): one topology class per line; where the workload draws
    kinematics, the counts are averaged over the first few accepted draws."""
    def accept(inp):
        try:
            ol.Prepared(inp)
            return True
        except ol.OracleError:
            return False

    scan, _ = workloads.box_pentagon_scan(8, seed=3, accept=accept)
    mixed, _ = workloads.mixed_batch(seed=5, counts=(4, 4, 4, 4), accept=accept)
    return [
        ("k4", [workloads.k4_euclidean()]),
        ("double_box", [workloads.double_box()]),
        ("cube", [workloads.cube_propagator()]),
        ("box_pentagon", scan),
        ("box_pentagon_undeformed", [dict(x, **{"lambda": 0.0}) for x in scan]),
        ("triangle", mixed[0:4]),
        ("ladder3_euclidean", mixed[4:8:2]),
        ("ladder3_minkowski", mixed[5:8:2]),
        ("wheel4", mixed[8:12]),
    ]


def count(inputs, samples=SAMPLES):
    tot = dict(add=0.0, mul=0.0, div=0.0, sqrt=0.0, trans=0.0, cmp=0.0)
    n = 0
    for inp in inputs:
        c = ol.Prepared(inp).count_ops(0, 0, samples)
        for k in tot:
            tot[k] += c[k]
        n += samples
    per = {k: v / n for k, v in tot.items()}
    per["flops"] = per["add"] + per["mul"] + per["div"] + per["sqrt"] + per["trans"]
    return per, n


def main():
    lines = [
        "# Floating-point operations per sample of the reference's loop (sector draw and integrand),",
        "# counted by running the oracle's restatement with an operation-counting scalar",
        "# (oracle/opcount.hpp: complex operations written out in real ones; each transcendental,",
        "# pow, exp, log, sin, cos, atan2, counts one in 'trans'; comparisons are not flops).",
        "# Command: python tests/golden/make_flop_counts.py",
        "# workload E V K deformed add mul div sqrt trans flops cmp samples",
    ]
    for name, inputs in cases():
        p = ol.Prepared(inputs[0])
        per, n = count(inputs)
        lines.append("%s %d %d %d %d %.1f %.1f %.1f %.1f %.1f %.1f %.1f %d" % (
            name, p.E, p.V, p.K, int(p.def_ref != 0.0), per["add"], per["mul"], per["div"], per["sqrt"],
            per["trans"], per["flops"], per["cmp"], n))
    open(OUT, "w").write("\n".join(lines) + "\n")
    print("\n".join(lines))


if __name__ == "__main__":
    main()
