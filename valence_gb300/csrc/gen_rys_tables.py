"""Generate the Rys quadrature tables used by the ERI kernels.

The n-point Rys rule for parameter T integrates polynomials p of degree
< 2n in x = t^2 exactly against the Boys weight:
    int_0^1 p(t^2) exp(-T t^2) dt = sum_i w_i(T) p(x_i(T)),
whose moments are the Boys functions F_k(T) = int_0^1 t^{2k} e^{-T t^2} dt.
For every n = 1..NMAX and every interval [j*H, (j+1)*H) of T < TMAX we
compute the roots/weights at Chebyshev nodes in 80-digit arithmetic (monic
orthogonal polynomial from the Hankel moment system, mpmath.polyroots,
weights from the Vandermonde moment system) and store Chebyshev
coefficients of the smooth, O(1) functions
    x_i(T) * (1 + T)      and      w_i(T) * sqrt(1 + T).
For T >= TMAX the rule is the half-range Gauss-Hermite limit
    x_i = X_i / T,  w_i = W_i / sqrt(T)
with X_i, W_i the squared positive nodes and weights of the 2n-point
Gauss-Hermite rule (error ~ exp(-T), below 1e-17 relative at T = TMAX).

usage: python gen_rys_tables.py  -> writes rys_tables.inc next to this file
"""
import os
import sys

import mpmath as mp

NMAX = 5
TMAX = 64.0
H = 0.5
NCHEB = 12
mp.mp.dps = 80


def boys_moments(T, kmax):
    T = mp.mpf(T)
    out = []
    for k in range(kmax + 1):
        if T == 0:
            out.append(mp.mpf(1) / (2 * k + 1))
        else:
            a = mp.mpf(k) + mp.mpf(1) / 2
            out.append(mp.gammainc(a, 0, T) / (2 * mp.power(T, a)))
    return out


def rys_rule(n, T):
    mu = boys_moments(T, 2 * n)
    # monic p(x) = x^n + sum c_j x^j orthogonal to x^i, i < n
    A = mp.matrix(n, n)
    b = mp.matrix(n, 1)
    for i in range(n):
        for j in range(n):
            A[i, j] = mu[i + j]
        b[i] = -mu[i + n]
    c = mp.lu_solve(A, b)
    coeffs = [mp.mpf(1)] + [c[j] for j in range(n - 1, -1, -1)]  # highest first
    roots = mp.polyroots(coeffs, maxsteps=400, extraprec=400)
    roots = sorted([mp.re(r) for r in roots])
    V = mp.matrix(n, n)
    rhs = mp.matrix(n, 1)
    for k in range(n):
        for i in range(n):
            V[k, i] = roots[i] ** k
        rhs[k] = mu[k]
    w = mp.lu_solve(V, rhs)
    return roots, [w[i] for i in range(n)]


def hermite_limit(n):
    # 2n-point Gauss-Hermite: positive nodes s_i, weights h_i;
    # int_0^inf g(s^2) e^{-s^2} ds = sum_i h_i g(s_i^2)
    X, W = [], []
    nodes = mp.polyroots(hermite_coeffs(2 * n), maxsteps=400, extraprec=400)
    pos = sorted([mp.re(s) for s in nodes if mp.re(s) > 0])
    for s in pos:
        # Gauss-Hermite weight: 2^{m-1} m! sqrt(pi) / (m^2 H_{m-1}(s)^2), m = 2n
        m = 2 * n
        hm1 = mp.hermite(m - 1, s)
        w = mp.power(2, m - 1) * mp.factorial(m) * mp.sqrt(mp.pi) / (m * m * hm1 * hm1)
        X.append(s * s)
        W.append(w)
    return X, W


def hermite_coeffs(m):
    # physicists' Hermite polynomial coefficients, highest first
    from mpmath import mpf
    c = [[mpf(1)], [mpf(2), mpf(0)]]
    for k in range(2, m + 1):
        prev, prev2 = c[-1], c[-2]
        new = [2 * x for x in prev] + [mpf(0)]
        p2 = [mpf(0), mpf(0)] + [2 * (k - 1) * x for x in prev2]
        c.append([a - b for a, b in zip(new, p2)])
    return c[m]


def cheb_fit(vals):
    # vals at nodes x_k = cos(pi (k + 1/2) / N), k = 0..N-1
    N = len(vals)
    out = []
    for j in range(N):
        s = mp.mpf(0)
        for k in range(N):
            s += vals[k] * mp.cos(mp.pi * j * (k + mp.mpf(1) / 2) / N)
        out.append(s * (2 if j else 1) / N)
    return out


def main():
    here = os.path.dirname(os.path.abspath(__file__))
    nint = int(TMAX / H)
    nodes = [mp.cos(mp.pi * (k + mp.mpf(1) / 2) / NCHEB) for k in range(NCHEB)]
    lines = []
    lines.append("/* Generated by gen_rys_tables.py -- do not edit. */")
    lines.append(f"#define RYS_NMAX {NMAX}")
    lines.append(f"#define RYS_TMAX {TMAX!r}")
    lines.append(f"#define RYS_H {H!r}")
    lines.append(f"#define RYS_NINT {nint}")
    lines.append(f"#define RYS_NCHEB {NCHEB}")
    # layout: for n: for interval: for f in (x_0..x_{n-1}, w_0..w_{n-1}): NCHEB coeffs
    offs, data = [], []
    for n in range(1, NMAX + 1):
        offs.append(len(data))
        for j in range(nint):
            a = mp.mpf(j) * H
            funcs = [[None] * NCHEB for _ in range(2 * n)]
            for k, xk in enumerate(nodes):
                T = a + (xk + 1) * H / 2
                r, w = rys_rule(n, T)
                for i in range(n):
                    funcs[i][k] = r[i] * (1 + T)
                    funcs[n + i][k] = w[i] * mp.sqrt(1 + T)
            for f in funcs:
                data.extend(cheb_fit(f))
        print(f"n={n} done", file=sys.stderr, flush=True)
    lines.append("static const int rys_table_offset[RYS_NMAX] = {" + ", ".join(str(o) for o in offs) + "};")
    lines.append(f"static const double rys_table_data[{len(data)}] = {{")
    for i in range(0, len(data), 4):
        lines.append("  " + ", ".join(repr(float(v)) for v in data[i:i + 4]) + ",")
    lines.append("};")
    hx, hw = [], []
    for n in range(1, NMAX + 1):
        X, W = hermite_limit(n)
        hx.append(X + [mp.mpf(0)] * (NMAX - n))
        hw.append(W + [mp.mpf(0)] * (NMAX - n))
    lines.append("static const double rys_asym_x[RYS_NMAX][RYS_NMAX] = {")
    for row in hx:
        lines.append("  {" + ", ".join(repr(float(v)) for v in row) + "},")
    lines.append("};")
    lines.append("static const double rys_asym_w[RYS_NMAX][RYS_NMAX] = {")
    for row in hw:
        lines.append("  {" + ", ".join(repr(float(v)) for v in row) + "},")
    lines.append("};")
    with open(os.path.join(here, "rys_tables.inc"), "w") as f:
        f.write("\n".join(lines) + "\n")


if __name__ == "__main__":
    main()
