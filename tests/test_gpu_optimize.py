"""The optimiser path on the GPU (vsvb_opt_*, vsvb_rsg).

first_order_opt's H/S (valence.F90:527-758) are built on the GPU as
derivatives of the energy numerator and norm (one forward + adjoint pass per
column) and are compared with the oracle's literal build -- the reference's
nb(nb+1)/2 transition energies over its dummy orbitals -- on the same
weights: singly occupied orbitals, split DOCC orbitals, spin averaging with
unpaired electrons, derived basis functions, spin couplings.  spin_opt's
matrices likewise.  The GPU minimize_energy is checked against the
optimised total energies of the reference's own test suite
(testing/testing.py:69-151, 1e-6 Eh), including the direct-minimisation
inputs (demgs_opt).
"""
import os

import numpy as np
import pytest

from tests.gpu_helpers import built_lib, built_oracle, need_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    need_gpu()
    built_lib()
    oracle_py = built_oracle()
    from valence_gb300 import api
    return api, oracle_py


def _path(oracle_py, suite, name):
    return os.path.join(oracle_py.GOLDEN, "cases", suite, name)


HS_CASES = [("testing", "lih-sv", (1, 2, 3)),          # coupled pair orbitals, a DOCC orbital
            ("examples", "li_opt", (1, 2)),            # unpaired orbital; DOCC with spin averaging
            ("testing", "be+ndf", (1, 2)),             # an entry through a derived basis function
            ("testing", "h2o-vdz-sc1", (1, 3, 6)),
            ("testing", "he3s-1s3s", (1, 2)),          # two unpaired electrons
            ("testing", "be-sc", (1, 4))]              # two spin couplings


@pytest.mark.parametrize("suite,name,orbs", HS_CASES, ids=[c[1] for c in HS_CASES])
def test_first_order_hs_matches_oracle(env, suite, name, orbs):
    api, oracle_py = env
    path = _path(oracle_py, suite, name)
    o = oracle_py.OptOracle(path)
    opt = api.Optimizer(path)
    rng = np.random.default_rng(3)
    c = opt.coeff0 * (1.0 + 0.05 * rng.standard_normal(opt.totlen))  # off the optimum
    o.set_coeff(c)
    for iorb in orbs:
        h_ref, s_ref = o.first_order_hs(iorb, 0)
        h, s = opt.first_order_hs(iorb, c)
        scale_h, scale_s = np.max(np.abs(h_ref)), np.max(np.abs(s_ref))
        assert np.max(np.abs(h - h_ref)) <= 1e-9 * scale_h, (iorb, np.max(np.abs(h - h_ref)), scale_h)
        assert np.max(np.abs(s - s_ref)) <= 1e-9 * scale_s, (iorb, np.max(np.abs(s - s_ref)), scale_s)
    opt.close()


def test_first_order_hs_is_the_energy_quadratic_form(env):
    """v^T H v / v^T S v + E_nuc is the energy of the weights v."""
    api, oracle_py = env
    path = _path(oracle_py, "testing", "h2o-vdz")
    opt = api.Optimizer(path)
    sysm = api.System(path)
    e = sysm.energy(opt.coeff0)["energy"]
    enuc = sysm.energy(opt.coeff0)["enucrep"]
    for iorb in (1, 5):
        h, s = opt.first_order_hs(iorb)
        b0, b1 = opt.map_orbs[iorb - 1] - 1, opt.map_orbs[iorb] - 1
        v = opt.coeff0[b0:b1]
        assert abs(v @ h @ v / (v @ s @ v) + enuc - e) < 1e-10
    opt.close()
    sysm.close()


@pytest.mark.parametrize("name", ["be-sc", "be-scv3s+2sc"])
def test_spin_hs_matches_oracle(env, name):
    api, oracle_py = env
    path = _path(oracle_py, "testing", name)
    o = oracle_py.OptOracle(path)
    opt = api.Optimizer(path)
    h_ref, s_ref = o.spin_hs(0)
    h, s = opt.spin_hs()
    assert np.max(np.abs(h - h_ref)) <= 1e-10 * np.max(np.abs(h_ref))
    assert np.max(np.abs(s - s_ref)) <= 1e-10 * np.max(np.abs(s_ref))
    opt.close()


@pytest.mark.parametrize("n", [1, 2, 7, 30, 65])
def test_rsg_matches_scipy(env, n):
    scipy_linalg = pytest.importorskip("scipy.linalg")
    api, _ = env
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n))
    h = a + a.T
    b = rng.standard_normal((n, n))
    s = b @ b.T + n * np.eye(n)
    eig, w = api.rsg(h, s)
    ref = scipy_linalg.eigh(h, s, eigvals_only=True)
    assert np.max(np.abs(eig - ref)) <= 1e-12 * max(1.0, np.max(np.abs(ref)))
    assert np.allclose(w.T @ s @ w, np.eye(n), atol=1e-11)
    assert np.allclose(h @ w, s @ w * eig, atol=1e-10 * max(1.0, np.max(np.abs(ref))))


def test_rsg_rejects_an_indefinite_overlap(env):
    api, _ = env
    with pytest.raises(api.VSVBError):
        api.rsg(np.eye(3), np.diag([1.0, -1.0, 1.0]))


def _opt_cases(oracle_py):
    out = []
    for c in oracle_py.goldens()["cases"]:
        if c["converged"]:
            out.append(pytest.param(c, id=f'{c["suite"]}-{c["name"]}'))
    return out


@pytest.mark.parametrize("case", _opt_cases(__import__("tests.oracle_py", fromlist=["x"])))
def test_minimize_reproduces_optimised_goldens(env, case):
    api, oracle_py = env
    path = os.path.join(oracle_py.GOLDEN, case["input"])
    opt = api.Optimizer(path)
    res, c, csc = opt.minimize()
    tol = oracle_py.goldens()["tolerances"]["total_energy"]
    assert abs(res["energy"] - case["total_energy"]) < tol, (res, case["total_energy"])
    assert res["converged"] == 1
    opt.close()


def test_optimised_orbitals_file_round_trip(env, tmp_path):
    """minimize_energy, then the 'orbitals' file (xm_output) of the result
    written with the optimised weights and read back as an input: its guess
    energy is the optimised energy."""
    api, oracle_py = env
    path = _path(oracle_py, "examples", "li_opt")
    opt = api.Optimizer(path)
    res, c, csc = opt.minimize()
    d = api.read_input(path)
    txt = api.format_orbitals(d, c, res["energy"], res["etol"], res["converged"])
    api.lib().vsvb_free_desc(d)
    src = open(path).read().split("\n")
    # the input's orbital section is replaced by the new one (the header,
    # geometry, basis and coupling records stay)
    first = [ln for ln in txt.split("\n") if ln.strip()][0]
    k = [i for i, ln in enumerate(src) if ln.split() == first.split()][0]
    out = tmp_path / "li_opt.next"
    out.write_text("\n".join(src[:k]) + "\n" + txt)
    s = api.System(str(out))
    e = s.energy()["energy"]
    s.close()
    opt.close()
    assert abs(e - res["energy"]) < 1e-7, (e, res["energy"])


def test_spin_coupling_weights_per_evaluation(env):
    """vsvb_gpu_set_spin_coeffs: the energy with new coupling weights equals
    the oracle's with the same weights, also through a replayed graph."""
    api, oracle_py = env
    path = _path(oracle_py, "testing", "be-sc")
    s = api.System(path)
    o = oracle_py.OptOracle(path)
    for csc in ([0.3, -1.2], [1.0, 0.0], [0.7, 0.7]):
        s.set_spin_coeffs(csc)
        o.set_coeff_sc(csc)
        e_ref = o.guess_energy(0).energy
        assert abs(s.energy()["energy"] - e_ref) < 1e-9, (csc, s.energy()["energy"], e_ref)
        for _ in range(3):
            r, g = s.energy_grad()
        assert abs(r["energy"] - e_ref) < 1e-9
    s.close()


def test_minimize_writes_orbitals_files(env, tmp_path):
    """vsvb_opt_set_output: minimize writes 'orbitals' after every update and
    with the 'converged to' record at the end, and 'nelecwfn' with the
    optimised coupling weights."""
    api, oracle_py = env
    path = _path(oracle_py, "testing", "be-sc")
    opt = api.Optimizer(path)
    orb, wfn = tmp_path / "orbitals", tmp_path / "nelecwfn"
    opt.set_output(str(orb), str(wfn))
    res, c, csc = opt.minimize()
    opt.close()
    txt = orb.read_text()
    line = [ln for ln in txt.split("\n") if "total energy in atomic units" in ln][0]
    assert abs(float(line.split()[-1]) - res["energy"]) < 1e-12
    assert "converged to" in txt
    w = [float(ln.split()[0]) for ln in wfn.read_text().split("\n") if ln.strip() and "." in ln.split()[0]]
    assert np.allclose(w, csc, atol=5e-9)


@pytest.mark.parametrize("name", ["h2o-vdz", "lih-sv", "be-sc", "c2-pt-vshf-p2"])
def test_minimize_on_the_mixed_path(env, name):
    """The optimiser on the double-float mixed path (FP32 below the Schwarz
    bound 1e-6) lands on the reference's optimised energy within 1e-6 Eh."""
    api, oracle_py = env
    case = [c for c in oracle_py.goldens()["cases"] if c["converged"] and c["name"] == name][0]
    opt = api.Optimizer(os.path.join(oracle_py.GOLDEN, case["input"]), precision=api.MIXED_DF64)
    res, c, csc = opt.minimize()
    opt.close()
    assert abs(res["energy"] - case["total_energy"]) < 1e-6, (res["energy"], case["total_energy"])
