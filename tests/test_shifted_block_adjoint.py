"""The adjoint of a singular determinant-pair block, checked on the CPU.

The energy walk differentiates every struck determinant of an overlap block
A through det(A) and A^-1 (Jacobi's identity):
    det(A; r->e_c)                  = det A * T[c][r]
    det(A; r1->e_c1, r2->e_c2)      = det A * (T[c1][r1] T[c2][r2] - T[c1][r2] T[c2][r1])
    d/dA of det A * F(T)            = det A * (F T^T - T^T (dF/dT) T^T).
A block whose pivots fall below 1e-7 of its largest entry (exact rank
deficiency from molecular symmetry) has no inverse, so the GPU takes the
determinant and inverse of A + delta I together (delta = 1e-8 of the largest
entry) for these derivatives.  A sum of struck determinants is a polynomial
in A, so this is the exact derivative at A + delta I.

Here that construction is compared with the exact derivative at A itself.
The exact derivative of a struck determinant with respect to A[i][j] is the
determinant struck once more at (i, j), taken directly by LU.  The blocks are
the alpha blocks of n2.sc4val-b.p2 at its input weights, whose orbital
overlaps come from the oracle: one nonsingular block, one of rank deficiency
1 and one of rank deficiency 2.  The functional has random weights on every
one- and two-strike determinant, as the walk's coefficients are.  The
determinant of A itself, paired with the shifted inverse, loses the
deficient blocks' derivative entirely, which the last check shows.
"""
import itertools
import os

import numpy as np
import pytest

from tests import oracle_py

DELTA = 1e-8


def _struck_det(A, strikes):
    """det of A with each (r, c) in strikes: row r and column c zeroed, 1 at (r, c)"""
    M = A.copy()
    for r, c in strikes:
        M[r, :] = 0.0
        M[:, c] = 0.0
        M[r, c] = 1.0
    return np.linalg.det(M)


def _terms(n, rng):
    """the functional's terms: (weight, strikes) over all one- and two-strike sets"""
    out = [(rng.standard_normal(), ((r, c),)) for r in range(n) for c in range(n)]
    pairs = list(itertools.combinations(range(n), 2))
    for (r1, r2) in pairs:
        for (c1, c2) in pairs:
            out.append((rng.standard_normal(), ((r1, c1), (r2, c2))))
    return out


def _grad_exact(A, terms):
    n = A.shape[0]
    G = np.zeros((n, n))
    for w, st in terms:
        rows = {r for r, _ in st}
        cols = {c for _, c in st}
        for i in range(n):
            if i in rows:
                continue
            for j in range(n):
                if j in cols:
                    continue
                G[i, j] += w * _struck_det(A, st + ((i, j),))
    return G


def _grad_jacobi(B, terms, det=None):
    """the walk's construction: det and inverse of B (det may be overridden)"""
    T = np.linalg.inv(B)
    d = np.linalg.det(B) if det is None else det
    val = 0.0
    Gt = np.zeros_like(T)  # dF/dT
    for w, st in terms:
        if len(st) == 1:
            (r, c), = st
            val += w * T[c, r]
            Gt[c, r] += w
        else:
            (r1, c1), (r2, c2) = st
            val += w * (T[c1, r1] * T[c2, r2] - T[c1, r2] * T[c2, r1])
            Gt[c1, r1] += w * T[c2, r2]
            Gt[c2, r2] += w * T[c1, r1]
            Gt[c1, r2] -= w * T[c2, r1]
            Gt[c2, r1] -= w * T[c1, r2]
    return d * (val * T.T - T.T @ Gt @ T.T)


@pytest.fixture(scope="module")
def n2_blocks():
    path = os.path.join(oracle_py.GOLDEN, "cases", "testing", "n2.sc4val-b.p2")
    o = oracle_py.OptOracle(path)
    inp = o.inp
    o.guess_energy_sampled(1, 1 << 40)  # prepares the normalised weights only
    npair, nd, nsc = inp.npair, inp.ndocc, max(inp.nspinc, 1)
    nsp = 2 * npair + inp.nunpd + nd
    S = np.array([[o.ovint(i + 1, j + 1) for j in range(nsp)] for i in range(nsp)])
    ps = np.ctypeslib.as_array(inp.pair_sc, shape=(npair * 2 * nsc,))

    def alpha_orbs(isc, bits):
        out = [ps[k + npair * (((bits >> k) & 1) + 2 * isc)] - 1 for k in range(npair)]
        return out + [2 * npair + inp.nunpd + d for d in range(nd)]

    blocks = {}
    for isc, jsc, bb, kb in itertools.product(range(nsc), range(nsc), range(1 << npair), range(1 << npair)):
        A = S[np.ix_(alpha_orbs(isc, bb), alpha_orbs(jsc, kb))]
        sv = np.linalg.svd(A, compute_uv=False)
        blocks.setdefault(int(np.sum(sv < 1e-10 * sv[0])), A)
        if len(blocks) == 3:
            break
    assert sorted(blocks) == [0, 1, 2]
    return blocks


@pytest.mark.parametrize("deficiency", [0, 1, 2])
def test_shifted_pair_gives_the_exact_derivative(n2_blocks, deficiency):
    A = n2_blocks[deficiency]
    terms = _terms(A.shape[0], np.random.default_rng(deficiency))
    g = _grad_exact(A, terms)
    amax = np.abs(A).max()
    gs = _grad_jacobi(A + DELTA * amax * np.eye(A.shape[0]), terms)
    err = np.abs(gs - g).max() / np.abs(g).max()
    print(f"rank deficiency {deficiency}: shifted-pair derivative, relative error {err:.2e}")
    assert err < 2e-7, err


@pytest.mark.parametrize("deficiency", [1, 2])
def test_exact_determinant_with_the_shifted_inverse_loses_the_block(n2_blocks, deficiency):
    A = n2_blocks[deficiency]
    terms = _terms(A.shape[0], np.random.default_rng(deficiency))
    g = _grad_exact(A, terms)
    B = A + DELTA * np.abs(A).max() * np.eye(A.shape[0])
    gx = _grad_jacobi(B, terms, det=np.linalg.det(A))
    err = np.abs(gx - g).max() / np.abs(g).max()
    print(f"rank deficiency {deficiency}: exact det with the shifted inverse, relative error {err:.2e}")
    assert err > 0.5
