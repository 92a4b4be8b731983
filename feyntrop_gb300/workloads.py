"""Seeded synthetic inputs for the benchmark configurations, in the reference's
low-level JSON schema (srcs/feyntrop.cpp:25-96).

The kinematics follow py_feyntrop.get_P_uv (py_feyntrop.py:186-234): the first
V_ext-1 external vertices carry the given scalar products, the last external row
and column follow from momentum conservation, internal vertices have zero rows.
All inputs are synthetic (no external data set exists for this path).
"""
import math
import random

__all__ = ["k4_euclidean", "double_box", "box_pentagon", "cube_propagator", "ladder3", "wheel4_vacuum",
           "triangle", "kinematic_matrix", "log_uniform_n", "box_pentagon_scan", "mixed_batch"]


def kinematic_matrix(V, sp):
    """V x V scalar products from sp[(i, j)] (i <= j < n_ext - 1) with momentum conservation."""
    n = max(max(i, j) for i, j in sp) + 1 if sp else 0
    P = [[0.0] * V for _ in range(V)]
    for (i, j), v in sp.items():
        P[i][j] = P[j][i] = float(v)
    for j in range(n):
        P[n][j] = -sum(P[i][j] for i in range(n))
    for i in range(n + 1):
        P[i][n] = -sum(P[i][j] for j in range(n))
    return P


def _inp(graph, D, P, m2, K, lam, N, seed=0):
    return {"graph": graph, "dimension": D, "scalarproducts": P, "masses_sqr": list(m2), "num_eps_terms": K,
            "lambda": lam, "N": int(N), "seed": seed}


def k4_euclidean(N=10**7, masses=(0, 1, 2, 3, 4, 5)):
    """Complete graph K4 (6 edges, 3 loops), D=4, P = -3 on the diagonal and +1 off it,
    3 eps orders, lambda=0 (the reference's low-level example with masses 0..5)."""
    g = [[[0, 1], 1], [[0, 2], 1], [[0, 3], 1], [[1, 2], 1], [[2, 3], 1], [[3, 1], 1]]
    P = [[-3, 1, 1, 1], [1, -3, 1, 1], [1, 1, -3, 1], [1, 1, 1, -3]]
    return _inp(g, 4, P, masses, 3, 0, N)


DOUBLE_BOX_EDGES = [[[0, 1], 1], [[0, 4], 1], [[1, 5], 1], [[5, 4], 1], [[5, 2], 1], [[4, 3], 1], [[3, 2], 1]]


def double_box(N=10**8, seed=1, lam=0.5):
    """Planar double box (6 vertices, 7 edges), externals 0-3 on shell (p^2 = 1),
    internal masses U[0.5, 2], s U[8, 20], t U[-6, -1] from random.Random(seed)
    (masses first, then s, then t), D=4, 2 eps orders."""
    rng = random.Random(seed)
    m2 = [rng.uniform(0.5, 2.0) for _ in range(7)]
    s, t = rng.uniform(8, 20), rng.uniform(-6, -1)
    sp = {(0, 0): 1.0, (1, 1): 1.0, (2, 2): 1.0, (0, 1): (s - 2) / 2, (1, 2): (t - 2) / 2, (0, 2): (2 - s - t) / 2}
    return _inp(DOUBLE_BOX_EDGES, 4, kinematic_matrix(6, sp), m2, 2, lam, N)


BOX_PENTAGON_EDGES = [[[0, 1], 1], [[1, 2], 1], [[2, 6], 1], [[6, 3], 1], [[3, 4], 1], [[4, 5], 1], [[5, 0], 1],
                      [[5, 6], 1]]


def log_uniform_n(rng, nmin, nmax):
    return int(math.exp(rng.uniform(math.log(nmin), math.log(nmax))))


def box_pentagon(rng, D=6, K=3, nmin=1e5, nmax=1e7, mmax=2.0):
    """Box-pentagon topology of the reference's test suite (7 vertices, 8 edges,
    externals 0-4) with masses U[0, mmax], the 10 independent invariants U[-10, 10],
    lambda U[0.2, 1.0] and N log-uniform in [nmin, nmax]."""
    m2 = [rng.uniform(0, mmax) for _ in range(8)]
    inv = [rng.uniform(-10, 10) for _ in range(10)]
    lam = rng.uniform(0.2, 1.0)
    N = int(math.exp(rng.uniform(math.log(nmin), math.log(nmax))))
    pairs = [(i, j) for i in range(4) for j in range(i, 4)]
    sp = {p: inv[k] for k, p in enumerate(pairs)}
    return _inp(BOX_PENTAGON_EDGES, D, kinematic_matrix(7, sp), m2, K, lam, N)


def cube_propagator(N=10**9):
    """5-loop 2-point cube graph Q3 (8 vertices, 12 edges), externals at the antipodal
    pair relabelled 0 and 1, p^2 = -1, all masses 1, D=4, 4 eps orders, lambda=0."""
    label = {0: 0, 7: 1}
    for v in range(1, 7):
        label[v] = v + 1
    g = []
    for a in range(8):
        for b in range(3):
            w = a ^ (1 << b)
            if a < w:
                g.append([[label[a], label[w]], 1])
    P = [[0.0] * 8 for _ in range(8)]
    P[0][0] = P[1][1] = -1.0
    P[0][1] = P[1][0] = 1.0
    return _inp(g, 4, P, [1.0] * 12, 4, 0, N)


LADDER3_EDGES = [[[0, 1], 1], [[4, 5], 1], [[6, 7], 1], [[3, 2], 1], [[0, 4], 1], [[4, 6], 1], [[6, 3], 1],
                 [[1, 5], 1], [[5, 7], 1], [[7, 2], 1]]


def ladder3(rng, euclidean=True, nmin=1e5, nmax=1e8, K=3):
    """3-loop 4-point ladder (8 vertices, 10 edges), externals 0-3, masses U[0, 3].
    Euclidean point: P = -Gram of four random momenta summing to zero; otherwise
    on-shell externals with s U[8, 20], t U[-6, -1]."""
    m2 = [rng.uniform(0, 3) for _ in range(10)]
    if euclidean:
        q = [[rng.uniform(-1, 1) for _ in range(4)] for _ in range(3)]
        q.append([-(q[0][d] + q[1][d] + q[2][d]) for d in range(4)])
        P = [[0.0] * 8 for _ in range(8)]
        for i in range(4):
            for j in range(4):
                P[i][j] = -sum(q[i][d] * q[j][d] for d in range(4))
        lam = 0
    else:
        s, t = rng.uniform(8, 20), rng.uniform(-6, -1)
        sp = {(0, 0): 1.0, (1, 1): 1.0, (2, 2): 1.0, (0, 1): (s - 2) / 2, (1, 2): (t - 2) / 2,
              (0, 2): (2 - s - t) / 2}
        P = kinematic_matrix(8, sp)
        lam = 0.5
    N = int(math.exp(rng.uniform(math.log(nmin), math.log(nmax))))
    return _inp(LADDER3_EDGES, 4, P, m2, K, lam, N)


WHEEL4_EDGES = [[[0, 1], 1], [[1, 2], 1], [[2, 3], 1], [[3, 0], 1], [[0, 4], 1], [[1, 4], 1], [[2, 4], 1],
                [[3, 4], 1]]


def wheel4_vacuum(N=10**6, K=2):
    """4-loop wheel vacuum graph (5 vertices, 8 edges), all masses 1, P = 0, D=4."""
    return _inp(WHEEL4_EDGES, 4, [[0.0] * 5 for _ in range(5)], [1.0] * 8, K, 0, N)


def triangle(rng, nmin=1e5, nmax=1e8, K=3):
    """1-loop triangle (3 edges), masses U[0, 3], Euclidean invariants."""
    m2 = [rng.uniform(0, 3) for _ in range(3)]
    pp0, pp1, s01 = -rng.uniform(0.5, 5), -rng.uniform(0.5, 5), -rng.uniform(1, 15)
    sp = {(0, 0): pp0, (1, 1): pp1, (0, 1): (s01 - pp0 - pp1) / 2}
    N = int(math.exp(rng.uniform(math.log(nmin), math.log(nmax))))
    return _inp([[[0, 1], 1], [[1, 2], 1], [[2, 0], 1]], 4, kinematic_matrix(3, sp), m2, K, 0, N)


def _accepted(make, accept):
    """make() until accept(inp) holds; returns (inp, number of rejected draws)."""
    rejected = 0
    while True:
        inp = make()
        if accept is None or accept(inp):
            return inp, rejected
        rejected += 1


def box_pentagon_scan(count=4096, seed=3, accept=None):
    """Batched kinematic scan: `count` box-pentagon instances drawn from
    random.Random(seed) (masses U[0, 2], invariants U[-10, 10], lambda U[0.2, 1],
    N log-uniform in [1e5, 1e7]).  An instance that accept() rejects (the plan's own
    input checks: non-generic or divergent points) is redrawn from the same generator.
    Returns (inputs, number of redrawn instances)."""
    rng = random.Random(seed)
    out, redrawn = [], 0
    for _ in range(count):
        inp, r = _accepted(lambda: box_pentagon(rng), accept)
        out.append(inp)
        redrawn += r
    return out, redrawn


def mixed_batch(seed=5, counts=(512, 512, 256, 256), nmin=1e5, nmax=1e8, accept=None):
    """Mixed uneven batch: counts[0] 1-loop triangles (Euclidean), counts[1] 3-loop
    4-point ladders (alternately Euclidean and Minkowski), counts[2] 4-loop wheel vacuum
    graphs (all masses 1) and counts[3] box-pentagons (Minkowski), masses U[0, 3], every
    instance with N log-uniform in [nmin, nmax], all from random.Random(seed).  Returns
    (inputs, number of redrawn instances)."""
    rng = random.Random(seed)
    out, redrawn = [], 0
    makers = [
        lambda k: triangle(rng, nmin, nmax),
        lambda k: ladder3(rng, euclidean=(k % 2 == 0), nmin=nmin, nmax=nmax),
        lambda k: wheel4_vacuum(N=log_uniform_n(rng, nmin, nmax)),
        lambda k: box_pentagon(rng, nmin=nmin, nmax=nmax, mmax=3.0),
    ]
    for kind, n in enumerate(counts):
        for k in range(n):
            inp, r = _accepted(lambda: makers[kind](k), accept)
            out.append(inp)
            redrawn += r
    return out, redrawn
