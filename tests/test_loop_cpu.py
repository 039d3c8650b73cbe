"""Host logic of the descent loop (valence_gb300.loop) on a quadratic
stand-in for a System: monotone decrease, the Armijo condition, the check
handle's records."""
import numpy as np

from valence_gb300 import loop


class Quadratic:
    def __init__(self, n=6, seed=0, shift=0.0):
        rng = np.random.default_rng(seed)
        q = rng.normal(size=(n, n))
        self.A = q @ q.T + n * np.eye(n)
        self.b = rng.normal(size=n)
        self.coeff0 = rng.normal(size=n)
        self.shift = shift
        self.calls = 0

    def energy(self, w):
        self.calls += 1
        return {"energy": 0.5 * w @ self.A @ w - self.b @ w + self.shift}

    def energy_grad(self, w):
        self.calls += 1
        return self.energy(w), self.A @ w - self.b


def test_descend_decreases_and_checks():
    s, c = Quadratic(), Quadratic(shift=1e-9)
    w, recs = loop.descend(s, steps=8, check=c)
    assert len(recs) == 8
    es = [r["energy"] for r in recs]
    assert all(b < a for a, b in zip(es, es[1:]))
    assert all(r["decrease"] > 0 for r in recs)
    assert all(abs(r["abs_dE_vs_check"] - 1e-9) < 1e-12 for r in recs)
    # the minimiser of the quadratic is A^-1 b: the loop approaches it
    w_star = np.linalg.solve(s.A, s.b)
    assert np.linalg.norm(w - w_star) < np.linalg.norm(s.coeff0 - w_star)


def test_descend_without_check():
    s = Quadratic(seed=3)
    _, recs = loop.descend(s, steps=3)
    assert "check_energy" not in recs[0]
    assert sum(r["evaluations"] for r in recs) >= 6
