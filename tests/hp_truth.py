"""Integrand of one sample at 50 significant digits (mpmath): the reference's formulas
(srcs/feynman_integral.hpp:198-362, srcs/laplacian.hpp:14-215) evaluated without
rounding concerns, to referee per-sample disagreements between two FP64
implementations in ill-conditioned sectors.  Test infrastructure only."""
import mpmath as mp
mp.mp.dps = 50

def truth(inp, info, X, psi_tr, xi_tr, detail=False):
    E = len(inp['graph']); V = max(max(e[0]) for e in inp['graph']) + 1; n = V - 1
    D = mp.mpf(inp['dimension']); W = mp.mpf(info['W']); L = info['loops']; K = int(inp['num_eps_terms'])
    IG = mp.mpf(info['IGtr']); kappa = -mp.mpf(info['lambda_used']) if info['deformed'] else mp.mpf(0)
    m2 = [mp.mpf(x) for x in inp['masses_sqr']]; nu = [mp.mpf(e[1]) for e in inp['graph']]
    P = [[mp.mpf(x) for x in row] for row in inp['scalarproducts']]
    ek = [max(e[0]) for e in inp['graph']]; el = [min(e[0]) for e in inp['graph']]
    psi_tr = mp.mpf(psi_tr); xi_tr = mp.mpf(xi_tr)
    tgt = psi_tr ** (-D / 2) * (psi_tr / xi_tr) ** W
    scale = tgt ** (1 / (D / 2 * L + W))
    X = [mp.mpf(x) * scale for x in X]
    def lap(y):
        A = mp.matrix(n, n)
        for e in range(E):
            k, l = ek[e], el[e]
            A[l, l] += y[e]
            if k == V - 1: continue
            A[k, k] += y[e]; A[k, l] -= y[e]; A[l, k] -= y[e]
        return A
    La = lap([1 / x for x in X])
    Pt = mp.matrix(n, n)
    for i in range(n):
        for j in range(n): Pt[i, j] = P[i][j]
    det = mp.det(La); psi = det
    for x in X: psi *= x
    G = La ** -1
    pphi = -sum((G * Pt)[i, i] for i in range(n))
    if kappa == 0:
        R = IG * psi ** (-D / 2)
        pxi = pphi + sum(m2[e] * X[e] for e in range(E))
        R *= pxi ** (-W)
        out = [R]
        ef = mp.log(psi) - L * mp.log(pxi)
        for j in range(1, K): out.append(out[-1] * ef / j)
        return [complex(x) for x in out]
    M = G * Pt * G
    def gx(A, i, j): return mp.mpf(0) if (i == V - 1 or j == V - 1) else A[i, j]
    def bil(A, a, b): return gx(A, ek[a], ek[b]) + gx(A, el[a], el[b]) - gx(A, ek[a], el[b]) - gx(A, el[a], ek[b])
    d = [None] * E; H = mp.matrix(E, E)
    for a in range(E):
        xa = 1 / X[a] ** 2
        s = bil(M, a, a); t = bil(G, a, a)
        d[a] = -xa * s
        H[a, a] = 2 * xa * s * (1 / X[a] - xa * t)
        for b in range(a + 1, E):
            H[a, b] = H[b, a] = -2 * xa / X[b] ** 2 * bil(M, a, b) * bil(G, a, b)
    th = [(d[e] + m2[e]) * kappa for e in range(E)]
    cX = [X[e] * mp.expj(th[e]) for e in range(E)]
    cL = lap([1 / c for c in cX])
    cdet = mp.det(cL)
    cPsi = cdet
    for c in cX: cPsi *= c
    cR = IG * mp.exp(-D / 2 * mp.log(cPsi))
    J = mp.matrix(E, E)
    for a in range(E):
        for b in range(E): J[a, b] = (1 if a == b else 0) + 1j * kappa * H[a, b] * X[b]
    detJ = mp.det(J)
    xnu = sum(nu[e] * th[e] for e in range(E))
    cR *= detJ * mp.expj(xnu)
    cG = cL ** -1
    cpphi = -sum((cG * Pt)[i, i] for i in range(n))
    cV = cpphi + sum(m2[e] * cX[e] for e in range(E))
    cR *= mp.exp(-W * mp.log(cV))
    out = [cR]
    ef = mp.log(cPsi) - L * mp.log(cV)
    for j in range(1, K): out.append(out[-1] * ef / j)
    if detail:
        return [complex(x) for x in out], dict(th=[float(t) for t in th], detJ=complex(detJ), cV=complex(cV), cpphi=complex(cpphi), cPsi=complex(cPsi), H=H, G=G, X=X)
    return [complex(x) for x in out]
