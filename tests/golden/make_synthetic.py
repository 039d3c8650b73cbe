"""Regenerate tests/golden/synthetic.json: CPU-oracle energies of the seeded
synthetic workloads (valence_gb300.configs), used as fixtures by the GPU
parity tests.  Run from the repository root:

    python tests/golden/make_synthetic.py [case ...]

(with case names, only those entries are recomputed).
"""
import json
import os
import subprocess
import sys
import tempfile

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from valence_gb300 import configs  # noqa: E402

CASES = {"ch_chain": dict(fn=configs.ch_chain, seed=2), "lif_cluster_small": dict(fn=configs.lif_cluster_small, seed=3),
         "singular_pair_large": dict(fn=configs.singular_pair_large, seed=5)}


N_BATCH = 16


def main(only=None):
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    exe = os.path.join(ROOT, "oracle", "_build", "vsvb_oracle")
    nthreads = os.cpu_count() or 1
    fx = os.path.join(ROOT, "tests", "golden", "synthetic.json")
    out = json.load(open(fx)) if only and os.path.exists(fx) else {}
    with tempfile.TemporaryDirectory() as d:
        for name, c in CASES.items():
            if only and name not in only:
                continue
            path = c["fn"](os.path.join(d, name + ".inp"), seed=c["seed"])
            txt = subprocess.run([exe, path, str(nthreads)], capture_output=True, text=True, check=True).stdout
            e = float([ln for ln in txt.splitlines() if "guess energy" in ln][0].split()[2])
            f = [ln for ln in txt.splitlines() if ln.strip().startswith("e1")][0].split()
            out[name] = {"seed": c["seed"], "energy": e, "wfnorm": float(f[5]), "e1": float(f[1]), "e2": float(f[3]),
                         "source": f"oracle/_build/vsvb_oracle on valence_gb300.configs.{c['fn'].__name__}"
                                   f"(seed={c['seed']}), {nthreads} threads"}
        if not only or "batch_molecules" in only:
            # the batched configuration's random molecules (seeds 1000 ...)
            mols = []
            for seed in range(1000, 1000 + N_BATCH):
                path = configs.random_molecule(os.path.join(d, f"m{seed}.inp"), seed)
                txt = subprocess.run([exe, path, str(nthreads)], capture_output=True, text=True, check=True).stdout
                e = float([ln for ln in txt.splitlines() if "guess energy" in ln][0].split()[2])
                f = [ln for ln in txt.splitlines() if ln.strip().startswith("e1")][0].split()
                mols.append({"seed": seed, "energy": e, "wfnorm": float(f[5])})
            out["batch_molecules"] = {"molecules": mols,
                                      "source": f"oracle/_build/vsvb_oracle on valence_gb300.configs.random_molecule"
                                                f"(seed), {nthreads} threads"}
    with open(os.path.join(ROOT, "tests", "golden", "synthetic.json"), "w") as fh:
        json.dump(out, fh, indent=1)


if __name__ == "__main__":
    main(sys.argv[1:] or None)
