"""Host-side checks of the C ABI (no GPU needed).

* the shared library exports every function include/vsvb_gpu.h declares;
* vsvb_read_input (the product's reader, xm_module.F90:25-335 semantics)
  agrees with an independent record-by-record parse of every golden input;
* entry points fail with a status code, never a crash, when no GPU is present
  or a request is malformed.
"""
import ctypes
import math
import os
import re
import subprocess

import numpy as np
import pytest

from tests import oracle_py

ROOT = oracle_py.ROOT


@pytest.fixture(scope="module")
def lib():
    from valence_gb300 import api, build
    build.build()
    return api.lib()


def _declared():
    h = open(os.path.join(ROOT, "include", "vsvb_gpu.h")).read()
    h = re.sub(r"/\*.*?\*/", "", h, flags=re.S)
    return sorted(set(re.findall(r"\b(vsvb_[a-z0-9_]+)\s*\(", h)))


def test_library_exports_every_declared_symbol(lib):
    from valence_gb300 import api
    out = subprocess.run(["nm", "-D", "--defined-only", api.library_path()], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (vsvb_\w+)", out))
    names = _declared()
    assert len(names) >= 15
    missing = [n for n in names if n not in exported]
    assert not missing, missing


class _Rec:
    """independent Fortran list-directed record reader for the check"""

    def __init__(self, path):
        self.lines = open(path).read().split("\n")
        self.pos = 0

    def read(self, types):
        vals = []
        while len(vals) < len(types):
            toks = self.lines[self.pos].replace(",", " ").split()
            self.pos += 1
            vals += toks[: len(types) - len(vals)]
        return [t(v.replace("d", "e").replace("D", "e")) for t, v in zip(types, vals)]


def _parse(path):
    r = _Rec(path)
    d = r.read([int] * 15)
    natom, natom_t, npair, nunpd, ndocc, totlen = d[:6]
    nspinc, nset, nxorb, mxctr = d[7], d[12], d[13], d[14]
    ndf = d[11]
    tol = r.read([int] * 6 + [float] * 2 + [int] * (2 * nset))
    atoms = [r.read([int, float, float, float]) for _ in range(natom)]
    exps, ncoef = [], []
    for _ in range(natom_t):
        z, ns = r.read([float, int])
        for _ in range(ns):
            l, nc = r.read([int, int])
            for _ in range(nc):
                v = r.read([float] if nc == 1 else [float, float])
                exps.append(v[0])
    if npair > 0:
        r.read(([float] if nspinc > 1 else []) * 1 + [int] * (2 * npair)) if nspinc == 1 else \
            r.read(([float] + [int] * (2 * npair)) * nspinc)
    if nxorb > 0:
        r.read([int] * (2 * nxorb))
    coeff = []
    for _ in range(2 * npair + nunpd + ndocc + ndf):
        head = r.read([int])
        n_at = head[0]
        r.pos -= 1
        head = r.read([int] * (n_at + 2))
        vals = r.read([int, float] * head[-1])
        coeff += vals[1::2]
    return dict(natom=natom, ntol_d=tol[1], ntol_i=tol[2], xyz=np.array([a[1:] for a in atoms]).ravel(),
                exps=np.array(exps), coeff=np.array(coeff))


@pytest.mark.parametrize("case", oracle_py.goldens()["cases"],
                         ids=[f'{c["suite"]}/{c["name"]}' for c in oracle_py.goldens()["cases"]])
def test_reader_matches_independent_parse(lib, case):
    from valence_gb300 import api
    path = os.path.join(oracle_py.GOLDEN, case["input"])
    d = api.read_input(path).contents
    ref = _parse(path)
    assert d.natom == ref["natom"] and d.ntol_d == ref["ntol_d"] and d.ntol_i == ref["ntol_i"]
    xyz = np.ctypeslib.as_array(d.coords, shape=(3 * d.natom,))
    assert np.allclose(xyz, ref["xyz"] * 1.889725987722, rtol=0, atol=1e-12)
    assert d.num_pr == len(ref["exps"])
    assert np.array_equal(np.ctypeslib.as_array(d.exponent, shape=(d.num_pr,)), ref["exps"])
    assert d.totlen >= len(ref["coeff"])
    assert np.array_equal(np.ctypeslib.as_array(d.coeff, shape=(len(ref["coeff"]),)), ref["coeff"])


def test_reader_rejects_malformed_input(lib, tmp_path):
    from valence_gb300 import api
    p = tmp_path / "bad.inp"
    p.write_text("1 1 1 0 0 4 4 0 1 1 0 0 0 0 1\n20 10 10 2 2 0 0.0 0.0\n")
    with pytest.raises(api.VSVBError, match="no spin couplings"):
        api.read_input(str(p))
    p.write_text("1 1 0 0 1\n")
    with pytest.raises(api.VSVBError):
        api.read_input(str(p))
    with pytest.raises(api.VSVBError):
        api.read_input(str(tmp_path / "missing.inp"))


def test_no_gpu_errors_are_status_codes(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from valence_gb300 import api
    with pytest.raises(api.VSVBError, match="vsvb_gpu_create failed"):
        api.System(os.path.join(oracle_py.GOLDEN, "cases", "testing", "h"))
    null = ctypes.c_void_p(1)
    assert lib.vsvb_det_factor_noalloc(null, 64, 65, null, null, null, None) == 8
    assert lib.vsvb_det_factor(None, 4, 1, null, null, null, None) == 1


def test_bench_reference_arm_two_gloo_ranks():
    """bench.py under torchrun with 2 ranks (gloo, CPU): rank 0 alone runs the
    CPU reference arm and prints one JSON line; rank 1 exits cleanly."""
    import json
    cmd = ["python", "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", "29517", os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--workload", "water_vshf", "--steps", "2", "--warmup", "1", "--gpus", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(l) for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = lines[0]
    assert j["impl"] == "reference" and j["n_gpus"] == 2 and j["value"] > 0
    assert j["cpu_baseline"]["kind"] == "port"


def test_orbitals_writer_reproduces_reference_sections(lib):
    """vsvb_format_orbitals (xm_output's format(5x,i2,5x,10i4) and
    format(4(i4,1x,f13.8))) against the orbital sections of the golden
    inputs that xm_output wrote: every line, byte for byte, in order."""
    from valence_gb300 import api
    matched = 0
    for c in oracle_py.goldens()["cases"]:
        path = os.path.join(oracle_py.GOLDEN, c["input"])
        d = api.read_input(path)
        txt = api.format_orbitals(d)
        lib.vsvb_free_desc(d)
        lines = [ln for ln in txt.split("\n total energy")[0].split("\n") if ln.strip()]
        src = open(path).read().split("\n")
        if lines[0] not in src or lines[1] not in src:
            continue  # a hand-written or older-layout orbital section
        pos = 0
        for ln in lines:
            assert ln in src[pos:], (c["name"], ln)
            pos = src.index(ln, pos) + 1
        matched += 1
    assert matched >= 35


def test_orbitals_writer_energy_trailer(lib):
    """format(/,1x,'total energy in atomic units ',f32.16) and
    format(1x,'converged to ',e10.2,' kCal/mol') as the reference wrote them
    at the end of testing/be-sv."""
    from valence_gb300 import api
    path = os.path.join(oracle_py.GOLDEN, "cases", "testing", "be-sv")
    d = api.read_input(path)
    txt = api.format_orbitals(d, energy=-14.5763526671381989, etol=1e-6, done=True)
    lib.vsvb_free_desc(d)
    lines = txt.split("\n")
    src = open(path).read().split("\n")
    k = lines.index(" total energy in atomic units             -14.5763526671381989")
    assert lines[k - 1] == "" and lines[k + 1] == " converged to   0.10E-05 kCal/mol"
    j = src.index(lines[k])
    assert src[j - 1:j + 2] == lines[k - 1:k + 2]
    d = api.read_input(path)
    txt = api.format_orbitals(d, energy=-1.0, etol=1e-4, done=False)
    lib.vsvb_free_desc(d)
    assert "converged" not in txt


def test_orbitals_writer_round_trip(lib, tmp_path):
    """Weights written with f13.8 read back within rounding."""
    import numpy as np
    from valence_gb300 import api
    path = os.path.join(oracle_py.GOLDEN, "cases", "testing", "h2o-vdz")
    d = api.read_input(path)
    dd = d.contents
    w = np.random.default_rng(5).uniform(-1, 1, dd.totlen)
    out = tmp_path / "orbitals"
    assert lib.vsvb_write_orbitals(str(out).encode(), d, w.ctypes.data_as(api.ctypes.POINTER(api.ctypes.c_double)),
                                   -76.0, 0.0, 0) == 0
    vals = []
    for ln in open(out).read().split("\n"):
        if "total energy" in ln or not ln.strip():
            continue
        if ln.startswith("     ") and ln[5:7].strip() and ln[7:12] == "     ":
            continue  # an atom-list record
        for k in range(0, len(ln), 18):
            vals.append(float(ln[k + 5:k + 18]))
    lib.vsvb_free_desc(d)
    assert np.max(np.abs(np.array(vals) - w)) <= 5.1e-9


def test_nelecwfn_writer_reproduces_reference_records(lib):
    """vsvb_format_nelecwfn (xm_output's format(1x,1f13.8,7(2i3,2x)) per
    coupling and format(1x,7(2i3,2x)) for the excited-state roots): the
    records the reference wrote into its multi-coupling inputs, verbatim."""
    from valence_gb300 import api
    checked = 0
    for name in ("be-sc", "be-scv3s+2sc", "f2-scval-p2", "n2.sc4val-b.p2"):
        path = os.path.join(oracle_py.GOLDEN, "cases", "testing", name)
        d = api.read_input(path)
        if d.contents.nspinc < 2:
            lib.vsvb_free_desc(d)
            continue
        txt = api.format_nelecwfn(d)
        lib.vsvb_free_desc(d)
        src = open(path).read().split("\n")
        recs = [ln for ln in txt.split("\n") if ln.strip()]
        for ln in recs:
            assert ln in src, (name, ln)
        checked += 1
    assert checked >= 2


def test_plain_c_host_compiles_links_and_runs(lib, tmp_path):
    """include/vsvb_gpu.h is a C header: a C99 host (tests/c_host/host.c)
    compiles against it with warnings as errors, links the library and runs
    the input reader and writers; handle creation returns a status code."""
    import shutil
    import torch
    from valence_gb300 import api
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / "host")
    libdir = os.path.dirname(api.library_path())
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "c_host", "host.c"), "-L", libdir, "-lvsvb_gb300",
                        "-Wl,-rpath," + libdir, "-o", exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    inp = os.path.join(oracle_py.GOLDEN, "cases", "testing", "be-sc")
    r = subprocess.run([exe, inp], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    out = dict((ln.split()[0], ln.split()[1:]) for ln in r.stdout.splitlines())
    assert out["read"][0] == "0" and out["read"][8] == "2"
    assert out["orbitals"][0] == "0" and int(out["orbitals"][1]) > 0
    assert out["nelecwfn"][0] == "0"
    if not torch.cuda.is_available():
        assert out["create"][0] != "0" and out["opt_create"][0] != "0"
    else:
        assert out["create"][0] == "0" and out["opt_create"][0] == "0"


@pytest.mark.parametrize("name", ["water_vshf", "ch_chain", "lif_cluster", "lif_cluster_small", "lif_cluster_3",
                                  "singular_pair_large", "alkane_chain"])
def test_workload_generators_parse(lib, tmp_path, name):
    """Every seeded benchmark workload is a valid VALENCE input for the
    library's reader, with the counts configs.describe reports."""
    from valence_gb300 import api, configs
    p = configs.WORKLOADS[name](str(tmp_path / (name + ".inp")))
    d = api.read_input(p)
    c = d.contents
    dsc = configs.describe(p)
    assert (c.natom, c.npair, c.nunpd, c.ndocc, c.totlen) == (dsc["atoms"], dsc["coupled_pairs"], dsc["unpaired"],
                                                             dsc["docc"], dsc["weights"])
    lib.vsvb_free_desc(d)
