"""Pin the CPU oracle against VALENCE's own golden energies.

Goldens: testing/testing.py:69-153 and examples/test_examples.py:63-153 of
the reference (copied with their inputs by tests/golden/make_goldens.py).
Tolerances are the reference's: 1e-10 Eh nuclear repulsion, 1e-8 Eh guess
energy (testing/testing.py:22-24).
"""
import math
import os

import numpy as np
import pytest

from tests import oracle_py

G = oracle_py.goldens()
CASES = G["cases"]
SLOW = {"f2-scval-p2", "n2.sc4val-b.p2", "ethane2"}


@pytest.mark.parametrize("case", CASES, ids=[f'{c["suite"]}/{c["name"]}' for c in CASES])
def test_oracle_matches_reference_golden(oracle, case):
    if case["name"] in SLOW and not os.environ.get("VSVB_SLOW"):
        pytest.skip("slow spin-coupled case; set VSVB_SLOW=1")
    o = oracle.Oracle(os.path.join(oracle.GOLDEN, case["input"]))
    r = o.guess_energy()
    assert abs(r.enucrep - case["nuclear_repulsion"]) < G["tolerances"]["nuclear_repulsion"]
    assert abs(r.energy - case["guess_energy"]) < G["tolerances"]["guess_energy"]


def test_boys_against_high_precision(oracle):
    # F_m(T) = gamma(m+1/2, T) / (2 T^(m+1/2)), evaluated in 40-digit arithmetic
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 40
    for T in (0.0, 1e-6, 0.3, 2.0, 9.5, 25.0, 29.999, 30.0, 31.0, 45.0, 90.0):
        f = oracle.boys(10, T)
        for m in range(11):
            if T == 0.0:
                ref = 1.0 / (2 * m + 1)
            else:
                a = mp.mpf(m) + mp.mpf(1) / 2
                ref = float(mp.gammainc(a, 0, T) / (2 * mp.power(T, a)))
            assert abs(f[m] - ref) <= 4e-15 * ref, (T, m, f[m], ref)


def test_hydrogen_atom_known_answer(oracle):
    o = oracle.Oracle(os.path.join(oracle.GOLDEN, "cases/testing/h"))
    r = o.guess_energy()
    assert abs(r.energy - (-0.4999455685829771)) < 1e-10
    assert r.e2 == 0.0


def test_translation_invariance(oracle):
    o = oracle.Oracle(os.path.join(oracle.GOLDEN, "cases/examples/h2o"))
    e0 = o.guess_energy().energy
    import re
    lines = open(os.path.join(oracle.GOLDEN, "cases/examples/h2o")).read().split("\n")
    # atoms are lines 3..5 of the data section: read them through the oracle-independent way
    xyz = []
    for ln in lines:
        p = ln.split()
        if len(p) == 4 and re.fullmatch(r"\d+", p[0]) and all(re.fullmatch(r"-?\d+\.\d+", q) for q in p[1:]):
            xyz.append([float(q) for q in p[1:]])
    xyz = np.array(xyz[:3])
    o.set_coords_angstrom((xyz + np.array([0.3, -1.1, 2.0])).ravel())
    e1 = o.guess_energy().energy
    assert abs(e1 - e0) < 1e-10


def test_timed_mode_at_stride_one_is_the_full_run():
    """vo_guess_energy_timed (the bench's bounded CPU samples) evaluates
    everything at stride 1: the same energy as vo_guess_energy, and phase
    times that are non-negative."""
    from tests import oracle_py
    p = os.path.join(oracle_py.GOLDEN, "cases", "testing", "be-sc")
    o = oracle_py.Oracle(p)
    full = o.guess_energy(2).energy
    r, ph = oracle_py.Oracle(p).guess_energy_timed(2, 1, 1, 1)
    assert abs(r.energy - full) < 1e-12 * max(1.0, abs(full))
    assert len(ph) == 4 and min(ph) >= 0.0
