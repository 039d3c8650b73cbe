"""GPU parity of block mode (vsvb_options.block_mode): the orbital-pair ERI
matrix built per atom quartet (each shell quartet's (ab|cd) block staged per
atom quartet, then one four-index transform per atom quartet) against the
per-shell-quartet path, the CPU oracle and the reference goldens.

Bars: FP64 energies within 1e-8 Eh of the goldens and the oracle fixtures;
block and per-quartet orbital-pair ERIs within 1e-12 relative of each other
(the same integrals summed in another order); the mixed paths within 1e-6 Eh
and their own error estimate.
"""
import json
import os

import numpy as np
import pytest

from tests.gpu_helpers import ROOT, built_lib, built_oracle, need_gpu

pytestmark = pytest.mark.gpu

GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def vg():
    need_gpu()
    built_lib()
    import valence_gb300
    return valence_gb300


def _cases():
    from tests import oracle_py
    return oracle_py.goldens()["cases"]


# s/p golden inputs (every shell s or p) of both suites
SP_CASES = ["testing/h", "testing/be-sc", "testing/be+ndf", "testing/ethane", "testing/h2o-vdz-sc1", "examples/h2o",
            "examples/nme3", "examples/lih.SCval", "examples/c3h8"]


@pytest.mark.parametrize("name", SP_CASES)
def test_block_mode_golden(vg, name):
    case = {c["input"]: c for c in _cases()}["cases/" + name]
    s = vg.System(os.path.join(GOLD, case["input"]), block_mode=1)
    assert s.block_stats()["on"]
    r = s.energy()
    assert abs(r["energy"] - case["guess_energy"]) < 1e-8, (r["energy"], case["guess_energy"])
    s.close()


@pytest.mark.parametrize("precision", ["FP64", "MIXED", "MIXED_DF64"])
def test_block_mode_cluster_matches_fixture_and_quartet_path(vg, tmp_path, precision):
    from valence_gb300 import configs
    fx = json.load(open(os.path.join(GOLD, "synthetic.json")))["lif_cluster_small"]
    p = configs.lif_cluster_small(str(tmp_path / "lif.inp"), seed=fx["seed"])
    prec = getattr(vg, precision)
    b = vg.System(p, precision=prec, block_mode=1)
    q = vg.System(p, precision=prec, block_mode=-1)
    assert b.block_stats()["on"] and not q.block_stats()["on"]
    rb, rq = b.energy(), q.energy()
    d = abs(rb["energy"] - fx["energy"])
    if precision == "FP64":
        assert d < 1e-8  # Eh, absolute
        assert abs(rb["wfnorm"] - fx["wfnorm"]) < 1e-10
        Tb, Tq = b.orbital_eri(), q.orbital_eri()
        assert np.max(np.abs(Tb - Tq)) <= 1e-12 * max(1.0, np.max(np.abs(Tq)))
    else:
        assert d < 1e-6, d
        assert d <= rb["err_est"] + 1e-8, (d, rb["err_est"])
        assert abs(rb["energy"] - rq["energy"]) < 1e-6
    assert rb["n_quartets_fp64"] + rb["n_quartets_fp32"] == rq["n_quartets_fp64"] + rq["n_quartets_fp32"]
    b.close()
    q.close()


def test_block_mode_orbital_integrals_match_oracle(vg, tmp_path):
    """Orbital overlap, core Hamiltonian and sampled (i k | j l) of a 2x2x2
    cluster in block mode against the oracle's ovint / int1e / int2e."""
    from valence_gb300 import configs
    o_mod = built_oracle()
    p = configs.lif_cluster_small(str(tmp_path / "lif.inp"))
    o = o_mod.Oracle(p)
    o.guess_energy()  # the oracle's normalised weights and orbital integrals
    s = vg.System(p, block_mode=1)
    s.energy()
    n = s.orbital_1e()[0].shape[0]
    S, H = s.orbital_1e()
    for i in range(n):
        for j in range(n):
            assert abs(S[i, j] - o.ovint(i + 1, j + 1)) < 1e-12 * max(1.0, abs(S[i, j]))
            assert abs(H[i, j] - o.int1e(i + 1, j + 1)) < 1e-11 * max(1.0, abs(H[i, j]))
    op = lambda a, b: a * (a + 1) // 2 + b if a >= b else b * (b + 1) // 2 + a
    rng = np.random.default_rng(1)
    quads = [tuple(int(x) for x in rng.integers(0, n, 4)) for _ in range(40)]
    got = s.orbital_eri_at([op(i, k) for i, k, j, l in quads], [op(j, l) for i, k, j, l in quads])
    for (i, k, j, l), g in zip(quads, got):
        ref = o.int2e(i + 1, k + 1, j + 1, l + 1)
        assert abs(g - ref) <= 1e-11 * max(1.0, abs(ref)), (i, k, j, l, g, ref)
    s.close()


def test_block_mode_three_cube(vg, tmp_path):
    """A 3x3x3 cluster (27 atoms, 243 functions): block mode and the
    per-quartet path give the same FP64 energy and orbital-pair ERIs."""
    from valence_gb300 import configs
    p = configs.lif_cluster(str(tmp_path / "lif27.inp"), n=3, ndocc=40)
    b = vg.System(p, block_mode=1)
    q = vg.System(p, block_mode=-1)
    rb, rq = b.energy(), q.energy()
    st = b.block_stats()
    assert st["on"] and st["atom_quartets"] > 0 and st["chunks"] >= 1
    assert abs(rb["energy"] - rq["energy"]) < 1e-8, (rb["energy"], rq["energy"])
    Tb, Tq = b.orbital_eri(), q.orbital_eri()
    assert np.max(np.abs(Tb - Tq)) <= 1e-12 * max(1.0, np.max(np.abs(Tq)))
    b.close()
    q.close()


def test_block_mode_refuses_d_shells_and_gradients(vg, tmp_path):
    from valence_gb300 import configs
    p = configs.ch_chain(str(tmp_path / "ch.inp"))
    with pytest.raises(vg.VSVBError):
        vg.System(p, block_mode=1)
    w = configs.water_vshf(str(tmp_path / "w.inp"))
    s = vg.System(w, block_mode=1)
    with pytest.raises(vg.VSVBError):
        s.energy_grad()
    s.close()
