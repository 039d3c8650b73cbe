"""Batched evaluation (one CUDA graph over many molecules) and the
single-handle graph replay, against eager per-molecule evaluation."""
import os

import numpy as np
import pytest

from tests.gpu_helpers import ROOT, built_lib, need_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def vg():
    need_gpu()
    built_lib()
    import valence_gb300
    return valence_gb300


def _molecules(vg, tmp_path, n, precision):
    from valence_gb300 import configs
    systems = []
    seed = 2000
    while len(systems) < n:
        p = configs.random_molecule(str(tmp_path / f"m{seed}.inp"), seed)
        seed += 1
        try:
            s = vg.System(p, precision=precision)
            r, _ = s.energy_grad()
        except vg.VSVBError:
            continue  # an unusable orbital set
        if r["n_singular_pairs"]:
            s.close()
            continue  # singular determinant pairs: covered in test_gpu_gradient.py
        systems.append(s)
    return systems


def test_graph_replay_matches_eager(vg, tmp_path):
    """The second call captures the evaluation as a CUDA graph and later
    calls replay it: same energy and gradient as the eager first call."""
    from valence_gb300 import configs
    p = configs.ch_chain(str(tmp_path / "chain.inp"))
    s = vg.System(p, precision=vg.MIXED_DF64)
    r0, g0 = s.energy_grad()          # eager
    r1, g1 = s.energy_grad()          # capture + replay
    r2, g2 = s.energy_grad()          # replay
    for r, g in ((r1, g1), (r2, g2)):
        assert abs(r["energy"] - r0["energy"]) < 1e-9
        assert np.max(np.abs(g - g0)) < 1e-9
        assert r["n_kernel_launches"] == r0["n_kernel_launches"]
    w = s.coeff0 * 1.01
    r3, g3 = s.energy_grad(w)         # new weights through the same graph
    s_ref = vg.System(p, precision=vg.MIXED_DF64, )
    r4, g4 = s_ref.energy_grad(w)     # eager on a fresh handle
    assert abs(r3["energy"] - r4["energy"]) < 1e-9
    assert np.max(np.abs(g3 - g4)) < 1e-9


@pytest.mark.parametrize("precision", ["FP64", "MIXED_DF64"])
def test_batch_matches_individual(vg, tmp_path, precision):
    torch = pytest.importorskip("torch")
    prec = getattr(vg, precision)
    systems = _molecules(vg, tmp_path, 6, prec)
    ref = [s.energy_grad() for s in systems]
    ws = [torch.tensor(s.coeff0, dtype=torch.float64, device="cuda") for s in systems]
    gs = [torch.zeros(s.totlen, dtype=torch.float64, device="cuda") for s in systems]
    b = vg.Batch(systems)
    for _ in range(2):  # capture, then replay
        res = b.energy_grad_device([w.data_ptr() for w in ws], [g.data_ptr() for g in gs])
        for (r0, g0), r, g in zip(ref, res, gs):
            assert abs(r["energy"] - r0["energy"]) < 1e-9 * max(1.0, abs(r0["energy"]))
            assert np.max(np.abs(g.cpu().numpy() - g0)) < 1e-9 * max(1.0, np.abs(g0).max())
    assert b.launches > 0
    # one merged ERI sweep for all molecules: fewer launches than the
    # molecules' own evaluations together
    assert b.launches < sum(r0["n_kernel_launches"] for r0, _ in ref)
    # new weights for one molecule, same pointers: replay sees them
    ws[0].mul_(0.5)
    res = b.energy_grad_device([w.data_ptr() for w in ws], [g.data_ptr() for g in gs])
    r0, g0 = systems[0].energy_grad(ws[0].cpu().numpy())
    assert abs(res[0]["energy"] - r0["energy"]) < 1e-9 * max(1.0, abs(r0["energy"]))
    b.close()


def test_autotune_changes_geometry_not_results(vg, tmp_path):
    from valence_gb300 import configs
    p = configs.ch_chain(str(tmp_path / "chain.inp"))
    r0, g0 = vg.System(p, precision=vg.MIXED_DF64).energy_grad()
    s = vg.System(p, precision=vg.MIXED_DF64, autotune=1)
    cfg = s.launch_config()
    assert cfg["nsplit"] >= 1 and cfg["eri"]
    assert all(b in (2, 4, 8, 16) for _, b in cfg["eri"])
    r1, g1 = s.energy_grad()
    assert abs(r1["energy"] - r0["energy"]) < 1e-9
    assert np.max(np.abs(g1 - g0)) < 1e-9


def _batch_fixture():
    import json
    return json.load(open(os.path.join(ROOT, "tests", "golden", "synthetic.json")))["batch_molecules"]["molecules"]


def test_batch_molecules_match_oracle(vg, tmp_path):
    """The batched configuration's random molecules (configs.random_molecule,
    seeds 1000-1015: 2-12 atoms, Z in {1,3,6,7,8,9}, s/p/d, 0-2 coupled
    pairs, an unpaired orbital for odd electron counts) against the CPU
    oracle's energies (tests/golden/make_synthetic.py): FP64 within 1e-8 Eh;
    the mixed path within 1e-6 Eh and its own error estimate, evaluated one by
    one and as one batch graph."""
    torch = pytest.importorskip("torch")
    from valence_gb300 import configs
    fx = _batch_fixture()
    paths = [configs.random_molecule(str(tmp_path / f"m{m['seed']}.inp"), m["seed"]) for m in fx]
    mixed = []
    for m, p in zip(fx, paths):
        s = vg.System(p)
        r = s.energy()
        assert abs(r["energy"] - m["energy"]) < 1e-8, (m["seed"], r["energy"], m["energy"])  # Eh, absolute
        assert abs(r["wfnorm"] - m["wfnorm"]) < 1e-10 * max(1.0, abs(m["wfnorm"]))
        s.close()
        sm = vg.System(p, precision=vg.MIXED_DF64)
        rm = sm.energy()
        d = abs(rm["energy"] - m["energy"])
        assert d < 1e-6 and d <= rm["err_est"] + 1e-8, (m["seed"], d, rm["err_est"])
        mixed.append(sm)
    ws = [torch.tensor(s.coeff0, dtype=torch.float64, device="cuda") for s in mixed]
    gs = [torch.zeros(s.totlen, dtype=torch.float64, device="cuda") for s in mixed]
    b = vg.Batch(mixed)
    res = b.energy_grad_device([w.data_ptr() for w in ws], [g.data_ptr() for g in gs])
    for m, r in zip(fx, res):
        assert abs(r["energy"] - m["energy"]) < 1e-6, (m["seed"], r["energy"], m["energy"])
    b.close()
    for s in mixed:
        s.close()
