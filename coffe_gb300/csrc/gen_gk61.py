"""Generate the 61-point Gauss-Kronrod rule (30-point Gauss + 31 Kronrod nodes).

The rule is the one QUADPACK's QAG uses with
key 6 (GSL_INTEG_GAUSS61, called at common.c:1024 of the reference).  The nodes are
computed here from their mathematical definition, not copied:

* Gauss nodes: roots of the Legendre polynomial P_30.
* Kronrod nodes: roots of the Stieltjes polynomial E_31, defined by
  int_{-1}^{1} P_30(x) E_31(x) P_m(x) dx = 0 for m = 0..30; E_31 is expanded in
  Legendre polynomials, the triple products int P_a P_b P_c = 2 (a b c; 0 0 0)^2
  give a linear system solved at 60 digits.
* Kronrod weights: the 61-point rule integrating P_0..P_60 exactly.
* Gauss weights: 2 / ((1 - x^2) P_30'(x)^2).

Writes a C header with the non-negative half of the nodes, ordered like QUADPACK
(largest node first; even index = Kronrod-only node, odd index = Gauss node, last =
centre).  Usage: python gen_gk61.py OUT.h [macro-prefix]
"""
import sys

import mpmath as mp
from sympy.physics.wigner import wigner_3j

mp.mp.dps = 60
N_GAUSS = 30


def triple(a, b, c):
    w = wigner_3j(a, b, c, 0, 0, 0)
    return 2 * mp.mpf(str(w.evalf(90))) ** 2 if w != 0 else mp.mpf(0)


def bisect(f, a, b, iters=230):
    fa = f(a)
    for _ in range(iters):
        m = (a + b) / 2
        fm = f(m)
        if fm == 0:
            return m
        if (fm < 0) == (fa < 0):
            a, fa = m, fm
        else:
            b = m
    return (a + b) / 2


def compute():
    n = N_GAUSS
    js = list(range(1, n + 1, 2))
    ms = list(range(1, n, 2))
    A = mp.matrix(len(ms), len(js))
    rhs = mp.matrix(len(ms), 1)
    for i, m in enumerate(ms):
        for j, jj in enumerate(js):
            A[i, j] = triple(n, m, jj)
        rhs[i] = -triple(n, m, n + 1)
    c = mp.lu_solve(A, rhs)
    coef = {jj: c[i] for i, jj in enumerate(js)}
    coef[n + 1] = mp.mpf(1)

    def stieltjes(x):
        return sum(cj * mp.legendre(j, x) for j, cj in coef.items())

    def legn(x):
        return mp.legendre(n, x)

    # Gauss nodes: P_n changes sign between consecutive Chebyshev-like guesses
    grid = [mp.cos(mp.pi * (n - i) / n) for i in range(n + 1)]
    gauss = []
    fine = [mp.mpf(-1) + 2 * mp.mpf(i) / 4000 for i in range(4001)]
    for i in range(len(fine) - 1):
        a, b = fine[i], fine[i + 1]
        if legn(a) == 0:
            gauss.append(a)
        elif (legn(a) < 0) != (legn(b) < 0):
            gauss.append(bisect(legn, a, b))
    assert len(gauss) == n, len(gauss)
    pts = [mp.mpf(-1)] + gauss + [mp.mpf(1)]
    kron = []
    for i in range(len(pts) - 1):
        a, b = pts[i], pts[i + 1]
        if i == n // 2:  # E_31 is odd: its middle root is exactly 0
            kron.append(mp.mpf(0))
            continue
        kron.append(bisect(stieltjes, a, b))
    assert len(kron) == n + 1
    nodes = sorted(gauss + kron)
    # Kronrod weights: exact for P_0..P_60
    M = mp.matrix(len(nodes), len(nodes))
    r = mp.matrix(len(nodes), 1)
    for k in range(len(nodes)):
        for i, x in enumerate(nodes):
            M[k, i] = mp.legendre(k, x)
        r[k] = 2 if k == 0 else 0
    wk = mp.lu_solve(M, r)
    wkron = {nodes[i]: wk[i] for i in range(len(nodes))}
    wgauss = {}
    for x in gauss:
        dp = mp.diff(legn, x)
        wgauss[x] = 2 / ((1 - x * x) * dp * dp)
    # checks: exactness of the Kronrod rule up to degree 91 on monomials
    for deg in range(0, 92, 7):
        s = sum(wkron[x] * x ** deg for x in nodes)
        exact = mp.mpf(2) / (deg + 1) if deg % 2 == 0 else 0
        assert abs(s - exact) < mp.mpf("1e-40"), (deg, s, exact)
    for deg in range(0, 60, 3):
        s = sum(wgauss[x] * x ** deg for x in gauss)
        exact = mp.mpf(2) / (deg + 1) if deg % 2 == 0 else 0
        assert abs(s - exact) < mp.mpf("1e-40"), (deg, s, exact)
    # non-negative half, largest first (QUADPACK ordering)
    half = sorted([x for x in nodes if x >= 0], reverse=True)
    xgk = half
    wgk = [wkron[x] for x in half]
    gauss_pos = sorted([x for x in gauss if x > 0], reverse=True)
    wg = [wgauss[x] for x in gauss_pos]
    # interleave check: odd entries of xgk are the Gauss nodes
    for j, x in enumerate(gauss_pos):
        assert abs(xgk[2 * j + 1] - x) < mp.mpf("1e-50")
    return xgk, wgk, wg


def main():
    out = sys.argv[1]
    prefix = sys.argv[2] if len(sys.argv) > 2 else "GK61"
    xgk, wgk, wg = compute()
    fmt = lambda v: mp.nstr(v, 36, min_fixed=-1, max_fixed=1) if v != 0 else "0.0"
    with open(out, "w") as fh:
        fh.write("/* Generated by gen_gk61.py: 61-point Gauss-Kronrod rule on [-1, 1].\n")
        fh.write("   XGK: non-negative Kronrod nodes, largest first; odd indices are the\n")
        fh.write("   30-point Gauss nodes, index 30 is the centre.  WGK: Kronrod weights.\n")
        fh.write("   WG: Gauss weights of the positive Gauss nodes (XGK[2j+1]).\n")
        fh.write("   The values are initialiser lists so host and device arrays can share them. */\n")
        fh.write(f"#pragma once\n#define {prefix}_NXGK 31\n#define {prefix}_NWG 15\n")
        for name, vals in (("XGK", xgk), ("WGK", wgk), ("WG", wg)):
            fh.write(f"#define {prefix}_{name}_INIT {{ \\\n")
            fh.write(", \\\n".join("    " + fmt(v) for v in vals) + " }\n")


if __name__ == "__main__":
    main()
