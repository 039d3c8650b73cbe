"""Adjoint weight gradient: dE/d(raw LCAO weights).

Checked against central finite differences (step 1e-5) of the GPU energy and
of the CPU oracle's energy (the literal restatement of the reference), to
1e-6 Eh per unit weight; the single-sweep and two-sweep adjoints must agree;
and, since normal() (valence.F90:2157-2182) makes E invariant to the scale
of each orbital's weights, sum_j c_j dE/dc_j = 0 per orbital.
"""
import os

import numpy as np
import pytest

from tests.gpu_helpers import ROOT, built_lib, built_oracle, need_gpu

pytestmark = pytest.mark.gpu
H = 1e-5


@pytest.fixture(scope="module")
def vg():
    need_gpu()
    built_lib()
    import valence_gb300
    return valence_gb300


def _orbital_ranges(path):
    from valence_gb300 import api
    d = api.read_input(path).contents
    norbs = 2 * d.npair + d.nunpd + d.ndocc + d.ndf
    m = np.ctypeslib.as_array(d.map_orbs, shape=(norbs + 1,))
    return [(m[i] - 1, m[i + 1] - 1) for i in range(norbs)]


def test_water_gradient_vs_fd_gpu_and_oracle(vg, tmp_path):
    from valence_gb300 import configs
    oracle = built_oracle()
    p = configs.water_vshf(str(tmp_path / "water.inp"))
    s = vg.System(p)
    r, g = s.energy_grad()
    c0 = s.coeff0.copy()
    o = oracle.Oracle(p)
    for j in range(len(c0)):
        cp, cm = c0.copy(), c0.copy()
        cp[j] += H
        cm[j] -= H
        fd = (s.energy(cp)["energy"] - s.energy(cm)["energy"]) / (2 * H)
        assert abs(g[j] - fd) < 1e-6, (j, g[j], fd)
        if j % 7 == 0:
            o.set_coeff(cp)
            ep = o.guess_energy().energy
            o.set_coeff(cm)
            em = o.guess_energy().energy
            assert abs(g[j] - (ep - em) / (2 * H)) < 1e-6, (j, g[j], (ep - em) / (2 * H))
    for a, b in _orbital_ranges(p):
        assert abs(np.dot(c0[a:b], g[a:b])) < 1e-8 * max(1.0, np.abs(g[a:b]).max())


def test_chain_gradient_modes_and_fd(vg, tmp_path):
    from valence_gb300 import configs
    p = configs.ch_chain(str(tmp_path / "chain.inp"))
    s0 = vg.System(p, grad_mode=0)
    s1 = vg.System(p, grad_mode=1)
    r0, g0 = s0.energy_grad()
    r1, g1 = s1.energy_grad()
    assert abs(r0["energy"] - r1["energy"]) < 1e-9
    assert np.max(np.abs(g0 - g1)) < 1e-8 * max(1.0, np.abs(g1).max())
    c0 = s0.coeff0.copy()
    rng = np.random.default_rng(3)
    for j in rng.choice(len(c0), 10, replace=False):
        cp, cm = c0.copy(), c0.copy()
        cp[j] += H
        cm[j] -= H
        fd = (s0.energy(cp)["energy"] - s0.energy(cm)["energy"]) / (2 * H)
        assert abs(g0[j] - fd) < 1e-6, (j, g0[j], fd)
    for a, b in _orbital_ranges(p):
        assert abs(np.dot(c0[a:b], g0[a:b])) < 1e-8 * max(1.0, np.abs(g0[a:b]).max())


def test_torch_autograd_function(vg, tmp_path):
    torch = pytest.importorskip("torch")
    from valence_gb300 import configs
    p = configs.water_vshf(str(tmp_path / "water.inp"))
    s = vg.System(p)
    w = torch.tensor(s.coeff0, dtype=torch.float64, requires_grad=True)
    e = vg.VSVBEnergy.apply(w, s)
    e.backward()
    r, g = s.energy_grad()
    assert abs(e.item() - r["energy"]) < 1e-12
    # the two calls differ only in the order of floating-point atomics
    d = np.abs(w.grad.numpy() - g).max()
    assert d < 1e-11 * max(1.0, np.abs(g).max()), d


def test_mixed_precision_error_bound(vg, tmp_path):
    from valence_gb300 import configs
    p = configs.ch_chain(str(tmp_path / "chain.inp"))
    e64 = vg.System(p, precision=vg.FP64).energy()["energy"]
    rm = vg.System(p, precision=vg.MIXED).energy()
    assert rm["n_quartets_fp32"] > 0
    assert abs(rm["energy"] - e64) <= 1e-6
    assert abs(rm["energy"] - e64) <= rm["err_est"]


@pytest.mark.parametrize("thr", [1e-6, 1e-4, 1e-3])
def test_mixed_error_estimate_covers_error(vg, tmp_path, thr):
    """err_est (FP32 rounding of the untransferred integral sizes behind the
    FP32 quartets, in units of |e2|/W per Schwarz-bound mass) must cover the
    measured |E_mixed - E_fp64| at every threshold without overshooting it
    by more than 10^3 where that difference is above FP64-class rounding."""
    from valence_gb300 import configs
    p = configs.ch_chain(str(tmp_path / "chain.inp"))
    e64 = vg.System(p, precision=vg.FP64).energy()["energy"]
    for prec in (vg.MIXED, vg.MIXED_DF64):
        r = vg.System(p, precision=prec, mixed_threshold=thr).energy()
        assert r["err_est"] > 0.0
        assert abs(r["energy"] - e64) <= r["err_est"], (prec, thr, r["energy"] - e64, r["err_est"])
        if abs(r["energy"] - e64) > 1e-9:  # below that the FP64-class rounding dominates the difference
            assert r["err_est"] <= 1e3 * abs(r["energy"] - e64), (prec, thr, r["energy"] - e64, r["err_est"])
    assert vg.System(p, precision=vg.FP64).energy()["err_est"] == 0.0


def test_double_float_path_matches_fp64(vg, tmp_path):
    """VSVB_MIXED_DF64 runs the FP64-designated quartets in double-float
    (FP32 pairs) with double-float Rys roots; with threshold 0 every quartet
    takes that path and must reproduce FP64 to near FP64 accuracy."""
    from valence_gb300 import configs
    p = configs.ch_chain(str(tmp_path / "chain.inp"))
    r64, g64 = vg.System(p, precision=vg.FP64).energy_grad()
    rdf, gdf = vg.System(p, precision=vg.MIXED_DF64, mixed_threshold=0.0).energy_grad()
    assert rdf["n_quartets_fp32"] == 0
    assert abs(rdf["energy"] - r64["energy"]) < 1e-10 * abs(r64["energy"])
    assert np.max(np.abs(gdf - g64)) < 1e-9 * max(1.0, np.abs(g64).max())
    rm, gm = vg.System(p, precision=vg.MIXED_DF64).energy_grad()
    assert rm["n_quartets_fp32"] > 0
    assert abs(rm["energy"] - r64["energy"]) <= 1e-6


def test_double_float_golden(vg):
    """A spin-coupled golden case through the double-float path."""
    import json
    from tests import oracle_py
    g = {c["name"]: c for c in oracle_py.goldens()["cases"] if c["suite"] == "testing"}
    for name in ("h2o-vdz", "c2-pt-vshf-p2", "cu+"):
        s = vg.System(os.path.join(ROOT, "tests", "golden", g[name]["input"]), precision=vg.MIXED_DF64,
                      mixed_threshold=0.0)
        assert abs(s.energy()["energy"] - g[name]["guess_energy"]) < 1e-8, name


def test_sweep_timing_reports_every_class(vg, tmp_path):
    """In-situ ERI class timing: one entry per class launch of the last
    sweep, positive durations, and FLOP counts that include the adjoint on
    the fused gradient path."""
    from valence_gb300 import configs
    p = configs.water_vshf(str(tmp_path / "water.inp"))
    s = vg.System(p)
    assert s.sweep_times() == []
    s.set_sweep_timing(True)
    s.energy()
    fwd = {x["cls"]: x for x in s.sweep_times()}
    s.energy_grad()
    both = {x["cls"]: x for x in s.sweep_times()}
    assert fwd and set(fwd) == set(both)
    for c in fwd:
        assert fwd[c]["ms"] > 0 and both[c]["ms"] > 0
        assert both[c]["flops"] > fwd[c]["flops"] > 0
    wall = s.sweep_wall_ms()
    assert wall >= 0.99 * max(x["ms"] for x in both.values())


@pytest.mark.parametrize("name", ["be+ndf", "h+ndf", "cu+", "c2-pt-vshf-p2"])
def test_gradient_through_derived_basis_functions(vg, name):
    """Inputs whose orbitals expand over derived basis functions (NDFs,
    ndf2obs, valence.F90:2191-2247): the gradient with respect to every
    weight, the NDFs' own expansion weights included, against central
    differences of the GPU energy, in both adjoint modes."""
    oracle = built_oracle()
    p = os.path.join(oracle.GOLDEN, "cases", "testing", name)
    s0 = vg.System(p, grad_mode=0)
    s1 = vg.System(p, grad_mode=1)
    c0 = s0.coeff0.copy() * (1.0 + 0.02 * np.random.default_rng(4).standard_normal(s0.totlen))
    r0, g0 = s0.energy_grad(c0)
    r1, g1 = s1.energy_grad(c0)
    assert np.max(np.abs(g0 - g1)) < 1e-8 * max(1.0, np.abs(g1).max())
    js = range(len(c0)) if len(c0) <= 40 else np.random.default_rng(5).choice(len(c0), 40, replace=False)
    for j in js:
        cp, cm = c0.copy(), c0.copy()
        cp[j] += H
        cm[j] -= H
        fd = (s0.energy(cp)["energy"] - s0.energy(cm)["energy"]) / (2 * H)
        assert abs(g0[j] - fd) < 1e-6, (j, g0[j], fd)


def test_gradient_through_singular_pairs(vg):
    """n2.sc4val-b.p2 at its input weights has exactly singular determinant
    pairs (symmetry-equal coupled orbitals; overlap blocks of rank deficiency
    1 and 2).  Their energy comes from exact struck determinants and their
    adjoint from the determinant and inverse of the shifted block A + delta I:
    the gradient matches central differences of the GPU energy in both
    adjoint modes, weight 6 (of an orbital with a derived-function entry)
    included, and sum_j c_j dE/dc_j = 0 per orbital."""
    oracle = built_oracle()
    p = os.path.join(oracle.GOLDEN, "cases", "testing", "n2.sc4val-b.p2")
    s0 = vg.System(p, grad_mode=0)
    s1 = vg.System(p, grad_mode=1)
    c0 = s0.coeff0.copy()
    r0, g0 = s0.energy_grad(c0)
    r1, g1 = s1.energy_grad(c0)
    assert r0["n_singular_pairs"] > 0
    assert abs(r0["energy"] - s0.energy(c0)["energy"]) < 1e-10
    assert np.max(np.abs(g0 - g1)) < 1e-8 * max(1.0, np.abs(g1).max())
    js = sorted(set([6]) | set(np.random.default_rng(7).choice(len(c0), 24, replace=False).tolist()))
    worst = 0.0
    for j in js:
        cp, cm = c0.copy(), c0.copy()
        cp[j] += H
        cm[j] -= H
        fd = (s0.energy(cp)["energy"] - s0.energy(cm)["energy"]) / (2 * H)
        worst = max(worst, abs(g0[j] - fd))
        assert abs(g0[j] - fd) < 1e-6, (j, g0[j], fd)
    print(f"n2 singular-pair gradient: largest |adjoint - central difference| {worst:.3e}")
    for b0, b1 in _orbital_ranges(p):
        assert abs(np.dot(c0[b0:b1], g0[b0:b1])) < 1e-8 * max(1.0, np.abs(g0[b0:b1]).max()), (b0, b1)


def test_first_order_hs_through_singular_pairs(vg):
    """first_order_opt's matrices on n2.sc4val-b.p2 (singular determinant
    pairs at its input weights): v^T H v / v^T S v + E_nuc is the energy of
    the orbital's own weights v."""
    from valence_gb300 import api
    oracle = built_oracle()
    p = os.path.join(oracle.GOLDEN, "cases", "testing", "n2.sc4val-b.p2")
    opt = api.Optimizer(p)
    sysm = api.System(p)
    r = sysm.energy(opt.coeff0)
    assert r["n_singular_pairs"] > 0
    for iorb in (1, 2, 11):
        h, s = opt.first_order_hs(iorb)
        b0, b1 = opt.map_orbs[iorb - 1] - 1, opt.map_orbs[iorb] - 1
        v = opt.coeff0[b0:b1]
        err = abs(v @ h @ v / (v @ s @ v) + r["enucrep"] - r["energy"])
        print(f"n2 first-order H/S orbital {iorb}: quadratic-form energy error {err:.3e}")
        assert err < 1e-9, iorb
    opt.close()
    sysm.close()
