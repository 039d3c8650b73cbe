"""GPU parity: the sm_103a path against VALENCE's golden energies and the
CPU oracle (a literal restatement of valence.F90's guess energy).

Bar: 1e-8 Eh on the FP64 path (testing/testing.py:22-24), 1e-10 Eh on the
nuclear repulsion.  Orbital-level integrals (S_ij, h_ij and every
(i k|j l)) are compared element-wise against the oracle's ovint/int1e/int2e.
"""
import os

import numpy as np
import pytest

from tests.gpu_helpers import ROOT, built_lib, built_oracle, need_gpu

pytestmark = pytest.mark.gpu

GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def lib_built():
    need_gpu()
    built_lib()
    import valence_gb300
    return valence_gb300


@pytest.fixture(scope="module")
def oracle():
    return built_oracle()


def _cases():
    from tests import oracle_py
    return oracle_py.goldens()["cases"]


@pytest.mark.parametrize("case", _cases(), ids=[f'{c["suite"]}/{c["name"]}' for c in _cases()])
def test_golden_guess_energy(lib_built, case):
    s = lib_built.System(os.path.join(GOLD, case["input"]))
    r = s.energy()
    assert abs(r["enucrep"] - case["nuclear_repulsion"]) < 1e-10
    assert abs(r["energy"] - case["guess_energy"]) < 1e-8, (r["energy"], case["guess_energy"])
    s.close()


@pytest.mark.parametrize("case", _cases(), ids=[f'{c["suite"]}/{c["name"]}' for c in _cases()])
def test_golden_guess_energy_mixed(lib_built, case):
    """The mixed path (FP32 below a Schwarz bound of 1e-6, double-float
    above) against the reference goldens: within 1e-6 Eh, and within its own
    error estimate of the golden (plus the goldens' 1e-8 tolerance)."""
    s = lib_built.System(os.path.join(GOLD, case["input"]), precision=lib_built.MIXED_DF64)
    r = s.energy()
    d = abs(r["energy"] - case["guess_energy"])
    assert d < 1e-6, (r["energy"], case["guess_energy"])
    assert d <= r["err_est"] + 1e-8, (d, r["err_est"], r["n_quartets_fp32"])
    s.close()


def _orbital_checks(sysobj, o, nsp, tol_rel=1e-11):
    S, H = sysobj.orbital_1e()
    T = sysobj.orbital_eri()
    for i in range(nsp):
        for j in range(nsp):
            assert abs(S[i, j] - o.ovint(i + 1, j + 1)) < 1e-12 * max(1.0, abs(S[i, j]))
            assert abs(H[i, j] - o.int1e(i + 1, j + 1)) < 1e-11 * max(1.0, abs(H[i, j]))
    op = lambda a, b: a * (a + 1) // 2 + b if a >= b else b * (b + 1) // 2 + a
    rng = np.random.default_rng(0)
    quads = [tuple(rng.integers(0, nsp, 4)) for _ in range(60)] + [(i, i, i, i) for i in range(nsp)]
    for i, k, j, l in quads:
        ref = o.int2e(i + 1, k + 1, j + 1, l + 1)
        got = T[op(i, k), op(j, l)]
        assert abs(got - ref) <= tol_rel * max(1.0, abs(ref)), (i, k, j, l, got, ref)


@pytest.mark.parametrize("name", ["testing/h2o-vdz", "testing/cu+", "testing/be-sc", "examples/nme3"])
def test_orbital_integrals_match_oracle(lib_built, oracle, name):
    path = os.path.join(GOLD, "cases", name)
    o = oracle.Oracle(path)
    ro = o.guess_energy()
    s = lib_built.System(path)
    r = s.energy()
    nsp = s.orbital_1e()[0].shape[0]
    _orbital_checks(s, o, nsp)
    assert abs(r["energy"] - ro.energy) < 1e-8
    assert abs(r["wfnorm"] - ro.wfnorm) < 1e-10 * max(1.0, abs(ro.wfnorm))


def test_synthetic_water_matches_oracle(lib_built, oracle, tmp_path):
    from valence_gb300 import configs
    p = configs.water_vshf(str(tmp_path / "water.inp"))
    o = oracle.Oracle(p)
    ro = o.guess_energy()
    s = lib_built.System(p)
    r = s.energy()
    _orbital_checks(s, o, 5)
    assert abs(r["e1"] - ro.e1) < 1e-8 * max(1, abs(ro.e1))
    assert abs(r["e2"] - ro.e2) < 1e-8 * max(1, abs(ro.e2))
    assert abs(r["energy"] - ro.energy) < 1e-8  # Eh, absolute


def test_synthetic_chain_matches_fixture(lib_built, tmp_path):
    import json
    from valence_gb300 import configs
    fx = json.load(open(os.path.join(GOLD, "synthetic.json")))["ch_chain"]
    p = configs.ch_chain(str(tmp_path / "ch_chain.inp"), seed=fx["seed"])
    s = lib_built.System(p)
    r = s.energy()
    assert abs(r["energy"] - fx["energy"]) < 1e-8  # Eh, absolute
    assert abs(r["wfnorm"] - fx["wfnorm"]) < 1e-10 * max(1.0, abs(fx["wfnorm"]))


@pytest.mark.parametrize("precision", ["FP64", "MIXED", "MIXED_DF64"])
def test_synthetic_cluster_matches_fixture(lib_built, tmp_path, precision):
    """The Li/F cluster workload's geometry and basis family at 2x2x2 (72
    functions, 12 DOCC, wfnorm 0.16) against the oracle fixture: FP64 within
    1e-8 Eh, the mixed paths within 1e-6 Eh and their own estimate."""
    import json
    from valence_gb300 import configs
    fx = json.load(open(os.path.join(GOLD, "synthetic.json")))["lif_cluster_small"]
    p = configs.lif_cluster_small(str(tmp_path / "lif.inp"), seed=fx["seed"])
    s = lib_built.System(p, precision=getattr(lib_built, precision))
    r = s.energy()
    d = abs(r["energy"] - fx["energy"])
    if precision == "FP64":
        assert d < 1e-8  # Eh, absolute
        assert abs(r["wfnorm"] - fx["wfnorm"]) < 1e-10
    else:
        assert d < 1e-6, d
        assert d <= r["err_est"] + 1e-8 * abs(fx["energy"]), (d, r["err_est"])


def test_energy_is_repeatable(lib_built):
    s = lib_built.System(os.path.join(GOLD, "cases", "examples", "h2o"))
    a = s.energy()["energy"]
    b = s.energy()["energy"]
    assert abs(a - b) < 1e-12
