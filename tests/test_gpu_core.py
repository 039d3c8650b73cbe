"""Core mode (the determinant-pair sum over the shared doubly occupied core,
core.cu) against the reference's golden energies, the per-pair walk,
central differences and the optimisation-loop workload at full size."""
import json
import os

import numpy as np
import pytest

from tests.gpu_helpers import ROOT, built_lib, need_gpu

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def vg():
    need_gpu()
    built_lib()
    import valence_gb300
    return valence_gb300


def _cases():
    with open(os.path.join(GOLDEN, "reference_goldens.json")) as f:
        return json.load(f)["cases"]


def _core_system(vg, path, **kw):
    try:
        return vg.System(path, core_mode=1, **kw)
    except vg.VSVBError:
        return None  # no spin-coupled pairs, or unpaired orbitals


def test_core_goldens_match_reference(vg):
    """Every golden case with spin-coupled pairs and no unpaired orbitals
    (20 of them, up to 7 pairs / 16,384 determinant pairs, and
    n2.sc4val-b.p2 with its 9,600 singular pairs) in core mode: the
    reference's guess energy within 1e-8 Eh (testing/testing.py:22-24) and
    the per-pair walk within 1e-10 Eh."""
    n = 0
    for c in _cases():
        p = os.path.join(GOLDEN, c["input"])
        s = _core_system(vg, p)
        if s is None:
            continue
        assert s.core_stats()["on"]
        r = s.energy()
        assert abs(r["energy"] - c["guess_energy"]) < 1e-8, (c["name"], r["energy"], c["guess_energy"])
        r0 = vg.System(p, core_mode=-1).energy()
        assert abs(r["energy"] - r0["energy"]) < 1e-10, c["name"]
        if c["name"] == "n2.sc4val-b.p2":
            assert r["n_singular_pairs"] >= 9600  # the walk flags 9,600
        n += 1
    assert n >= 20


@pytest.mark.parametrize("name", ["testing/lih", "testing/be-sc", "testing/h2o-vdz-sc1", "testing/f2-scval-p2",
                                  "testing/n2.sc4val-b.p2"])
def test_core_gradient(vg, name):
    """The core-mode adjoint against the per-pair walk's gradient and central
    differences (h = 1e-5) of the core-mode energy on three weights."""
    p = os.path.join(GOLDEN, "cases", name)
    s = vg.System(p, core_mode=1)
    r, g = s.energy_grad()
    r0, g0 = vg.System(p, core_mode=-1).energy_grad()
    gmax = np.max(np.abs(g0))
    # the walk shifts singular blocks by 1e-8 of their scale; core mode extrapolates exactly
    tol = 1e-5 if r["n_singular_pairs"] else 1e-7
    assert np.max(np.abs(g - g0)) < tol * gmax
    rng = np.random.default_rng(7)
    for i in rng.choice(s.totlen, size=3, replace=False):
        w = s.coeff0.copy()
        w[i] += 1e-5
        ep = s.energy(w)["energy"]
        w[i] -= 2e-5
        em = s.energy(w)["energy"]
        assert abs((ep - em) / 2e-5 - g[i]) < 1e-6 * max(1.0, gmax), (name, i)


def test_core_mode_selection(vg):
    """Automatic from 4,096 determinant pairs; forced core mode refuses
    unpaired orbitals and the two-sweep gradient."""
    big = vg.System(os.path.join(GOLDEN, "cases", "testing", "f2-scval-p2"))  # 7 pairs: 16,384
    assert big.core_stats()["on"] and big.core_stats()["determinant_pairs"] == 16384
    small = vg.System(os.path.join(GOLDEN, "cases", "testing", "lih"))  # 2 pairs: 16
    assert not small.core_stats()["on"]
    unpaired = None
    for c in _cases():
        p = os.path.join(GOLDEN, c["input"])
        try:
            vg.System(p, core_mode=-1)
        except vg.VSVBError:
            continue
        if _core_system(vg, p) is None:
            unpaired = p
            break
    assert unpaired is not None
    with pytest.raises(vg.VSVBError):
        vg.System(unpaired, core_mode=1)
    s = vg.System(os.path.join(GOLDEN, "cases", "testing", "lih"), core_mode=1, grad_mode=1)
    with pytest.raises(vg.VSVBError):
        s.energy_grad()


def test_core_full_chain_two_pairs_matches_walk(vg, tmp_path):
    """The optimisation loop's 128-atom chain (1,576 functions, 117 DOCC)
    with 2 of its 8 pairs (16 determinant pairs, walkable): core mode and
    the per-pair walk agree in energy (1e-9 relative) and gradient."""
    from valence_gb300 import configs
    p = configs.alkane_chain(str(tmp_path / "ac2.inp"), npair=2)
    r, g = vg.System(p, core_mode=1).energy_grad()
    r0, g0 = vg.System(p, core_mode=-1).energy_grad()
    assert abs(r["energy"] - r0["energy"]) < 1e-9 * abs(r0["energy"])
    assert np.max(np.abs(g - g0)) < 1e-8 * np.max(np.abs(g0))


def test_core_full_chain_eight_pairs(vg, tmp_path):
    """The optimisation loop's workload itself (8 pairs: 65,536 determinant
    pairs) in core mode: mixed within 1e-6 Eh of FP64, gradients equal to
    1e-8 relative, FP64 gradient against central differences."""
    from valence_gb300 import configs
    p = configs.alkane_chain(str(tmp_path / "ac8.inp"))
    s64 = vg.System(p)
    assert s64.core_stats()["on"] and s64.core_stats()["determinant_pairs"] == 65536
    r64, g64 = s64.energy_grad()
    rm, gm = vg.System(p, precision=vg.MIXED_DF64).energy_grad()
    assert abs(rm["energy"] - r64["energy"]) < 1e-6
    gmax = np.max(np.abs(g64))
    assert np.max(np.abs(gm - g64)) < 1e-8 * gmax
    rng = np.random.default_rng(3)
    for i in rng.choice(s64.totlen, size=2, replace=False):
        w = s64.coeff0.copy()
        w[i] += 1e-5
        ep = s64.energy(w)["energy"]
        w[i] -= 2e-5
        em = s64.energy(w)["energy"]
        # central-difference noise: 1e-16 |E| / h
        assert abs((ep - em) / 2e-5 - g64[i]) < 1e-6 * gmax + 1e-16 * abs(r64["energy"]) / 1e-5


def test_descent_loop_on_the_chain(vg, tmp_path):
    """Two steps of the optimisation loop (valence_gb300.loop.descend) on the
    65,536-pair chain: mixed-path gradient steps lower the energy, and the
    FP64 energy at each accepted point is within 1e-6 Eh of the mixed one."""
    from valence_gb300 import configs, loop
    p = configs.alkane_chain(str(tmp_path / "ac8.inp"))
    smx = vg.System(p, precision=vg.MIXED_DF64)
    s64 = vg.System(p)
    e0 = smx.energy()["energy"]
    _, recs = loop.descend(smx, steps=2, check=s64)
    assert recs[0]["energy"] < e0 and recs[1]["energy"] < recs[0]["energy"]
    assert all(r["abs_dE_vs_check"] < 1e-6 for r in recs)


def test_chain_integrals_match_oracle(vg, tmp_path):
    """The optimisation loop's 128-atom chain at full basis size (1,576
    s/p/d functions, 117 DOCC; one coupled pair so that the oracle's
    normalisation pass is cheap): sampled orbital overlaps, core-Hamiltonian
    elements and orbital-quartet ERIs against the oracle's ovint / int1e /
    int2e (valence.F90:2891-3176, 3184-3438)."""
    from tests.gpu_helpers import built_oracle
    from valence_gb300 import configs
    o_mod = built_oracle()
    p = configs.alkane_chain(str(tmp_path / "ac1.inp"), npair=1)
    o = o_mod.Oracle(p)
    o.guess_energy_timed(0, 10 ** 9, 10 ** 9, 10 ** 12)  # normalised weights; one item per phase
    s = vg.System(p)
    s.energy()
    S, H = s.orbital_1e()
    n = S.shape[0]
    rng = np.random.default_rng(11)
    for i, j in rng.integers(0, n, (40, 2)):
        assert abs(S[i, j] - o.ovint(int(i) + 1, int(j) + 1)) < 1e-12 * max(1.0, abs(S[i, j]))
        assert abs(H[i, j] - o.int1e(int(i) + 1, int(j) + 1)) < 1e-11 * max(1.0, abs(H[i, j]))
    op = lambda a, b: a * (a + 1) // 2 + b if a >= b else b * (b + 1) // 2 + a
    # quartets of neighbouring orbitals (orbital k sits on carbons k mod 41 + 1, + 2)
    quads = [(0, 1, 2, 43), (3, 44, 3, 44), (5, 46, 6, 47), (10, 51, 11, 11), (20, 61, 21, 62),
             (0, 41, 1, 42), (100, 59, 101, 60), (7, 7, 48, 48)]
    quads = [q for q in quads if max(q) < n]
    got = s.orbital_eri_at([op(i, k) for i, k, j, l in quads], [op(j, l) for i, k, j, l in quads])
    for (i, k, j, l), g in zip(quads, got):
        ref = o.int2e(i + 1, k + 1, j + 1, l + 1)
        assert abs(g - ref) <= 1e-11 * max(1.0, abs(ref)), (i, k, j, l, g, ref)
    s.close()
