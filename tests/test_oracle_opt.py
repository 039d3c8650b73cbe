"""The oracle's restatement of the reference optimiser (minimize_energy with
first_order_opt, demgs_opt and spin_opt, valence.F90:350-936, 2744-2885)
against the optimised total energies the reference's own test suite pins
(testing/testing.py:69-151, examples/test_examples.py: 'True' entries,
1e-6 Eh).  The H/S builds are the oracle's literal transition energies over
the reference's dummy orbitals; rsg is scipy's generalised eigensolver."""
import os

import numpy as np
import pytest

from tests import oracle_py

# inputs the oracle optimises in seconds (c2-pt-vshf-p2, about 15 minutes
# here, is left out); h2o-vdz-dem and the testing li_opt run demgs_opt
FAST = ["be", "be+ndf", "cu+", "h", "h2-dz", "h2-sz", "he", "h+ndf", "h2o-vdz", "h2o-vdz-sc1", "h2o-vdz-dem", "lih-sv",
        "be-sc", "be-scv3s+2sc", "be3s2", "he1s2s", "he3s-1s3s", "li_opt"]


def _cases():
    out = []
    for c in oracle_py.goldens()["cases"]:
        if c["converged"] and c["name"] in FAST:
            out.append(pytest.param(c, id=f'{c["suite"]}-{c["name"]}'))
    return out


@pytest.mark.parametrize("case", _cases())
def test_oracle_optimiser_reproduces_optimised_goldens(case):
    o = oracle_py.OptOracle(os.path.join(oracle_py.GOLDEN, case["input"]))
    e, it = o.minimize_energy(0)
    tol = oracle_py.goldens()["tolerances"]["total_energy"]
    assert abs(e - case["total_energy"]) < tol, (e, case["total_energy"])
    assert it >= 1


def test_first_order_hs_is_the_energy_quadratic_form():
    """H/S of a singly occupied orbital: the guess energy of the wave
    function with that orbital's weights c is c^T H c / c^T S c (normalised
    c), so H/S reproduce the full energy evaluation."""
    o = oracle_py.OptOracle(os.path.join(oracle_py.GOLDEN, "cases", "testing", "lih-sv"))
    r = o.guess_energy(0)
    for iorb in (1, 3):
        ham, ovl = o.first_order_hs(iorb, 0)
        assert np.allclose(ham, ham.T) and np.allclose(ovl, ovl.T)
        c = o.coeff_raw()
        b0 = o.inp.map_orbs[iorb - 1] - 1
        v = c[b0:b0 + ham.shape[0]]
        e = v @ ham @ v / (v @ ovl @ v) + o.enucrep()
        assert abs(e - r.energy) < 1e-10, (iorb, e, r.energy)


def test_spin_hs_is_the_coupling_quadratic_form():
    o = oracle_py.OptOracle(os.path.join(oracle_py.GOLDEN, "cases", "testing", "be-sc"))
    r = o.guess_energy(0)
    ham, ovl = o.spin_hs(0)
    c = o.coeff_sc()
    e = c @ ham @ c / (c @ ovl @ c) + o.enucrep()
    assert abs(e - r.energy) < 1e-10, (e, r.energy)
