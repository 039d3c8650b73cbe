"""Exactly singular determinant blocks above 32 electrons of one spin.

A coupled pair whose first orbital sits on an atom 25 A away from the rest
(valence_gb300.configs.singular_pair_large: 33 alpha electrons) makes every
transition determinant pair that moves that orbital between spin blocks
singular: its overlap block has a row of zeros.  The reference takes such
struck determinants with Givens rotations at any size (givdr,
valence.F90:2067-2144); the GPU takes them from three factorisations of the
block plus a fixed rank-2 term.  Bars: FP64 within 1e-8 Eh of the CPU oracle,
the mixed path within 1e-6 Eh, and the gradient against central differences
within 1e-6 Eh per unit weight.
"""
import json
import os

import numpy as np
import pytest

from tests.gpu_helpers import ROOT, built_lib, need_gpu

pytestmark = pytest.mark.gpu

GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def vg():
    need_gpu()
    built_lib()
    import valence_gb300
    return valence_gb300


@pytest.fixture(scope="module")
def case(tmp_path_factory):
    from valence_gb300 import configs
    fx = json.load(open(os.path.join(GOLD, "synthetic.json")))["singular_pair_large"]
    p = configs.singular_pair_large(str(tmp_path_factory.mktemp("sing") / "sing.inp"), seed=fx["seed"])
    return p, fx


def test_energy_matches_oracle(vg, case):
    p, fx = case
    s = vg.System(p)
    r = s.energy()
    assert r["n_singular_pairs"] > 0
    assert abs(r["energy"] - fx["energy"]) < 1e-8, (r["energy"], fx["energy"])  # Eh, absolute
    assert abs(r["wfnorm"] - fx["wfnorm"]) < 1e-10 * max(1.0, abs(fx["wfnorm"]))
    s.close()


def test_mixed_energy(vg, case):
    p, fx = case
    s = vg.System(p, precision=vg.MIXED_DF64)
    r = s.energy()
    assert abs(r["energy"] - fx["energy"]) < 1e-6
    s.close()


def test_gradient_matches_central_differences(vg, case):
    p, _ = case
    s = vg.System(p)
    c0 = s.coeff0.copy()
    r, g = s.energy_grad(c0)
    assert r["n_singular_pairs"] > 0
    h = 1e-5
    for j in np.random.default_rng(3).choice(len(c0), 12, replace=False):
        cp, cm = c0.copy(), c0.copy()
        cp[j] += h
        cm[j] -= h
        fd = (s.energy(cp)["energy"] - s.energy(cm)["energy"]) / (2 * h)
        assert abs(g[j] - fd) < 1e-6, (j, g[j], fd)
    s.close()


def test_core_mode_matches_oracle(vg, case):
    """The same configuration in core mode (forced; one coupled pair): the
    far orbital's 1 x 1 Schur blocks are about zero and take the exact path,
    whose first cofactor is det S_DD; energy against the oracle, gradient
    against the walk's (which shifts singular blocks by 1e-8 of their
    scale)."""
    p, fx = case
    s = vg.System(p, core_mode=1)
    assert s.core_stats()["on"]
    r, g = s.energy_grad()
    assert r["n_singular_pairs"] > 0
    assert abs(r["energy"] - fx["energy"]) < 1e-8, (r["energy"], fx["energy"])
    r0, g0 = vg.System(p, core_mode=-1).energy_grad()
    assert np.max(np.abs(g - g0)) < 1e-5 * max(1.0, np.max(np.abs(g0)))
    s.close()
