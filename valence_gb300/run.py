"""Run one workload through the GPU path and print the result as JSON.

    python -m valence_gb300.run --workload ch_chain --precision mixed_df64 --grad
    python -m valence_gb300.run --input h2o.inp --precision fp64

A workload name writes the seeded synthetic input (valence_gb300.configs);
--input runs any file in VALENCE's input format.  --repeat N evaluates N
times (the single-kernel profiles of the ERI and assembly kernels are taken
on this command).
"""
import argparse
import json
import os
import tempfile

import valence_gb300 as vg
from valence_gb300 import configs

PRECISIONS = {"fp64": vg.FP64, "mixed": vg.MIXED, "mixed_df64": vg.MIXED_DF64}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    g = ap.add_mutually_exclusive_group(required=True)
    g.add_argument("--workload", choices=sorted(configs.WORKLOADS))
    g.add_argument("--input")
    ap.add_argument("--precision", choices=sorted(PRECISIONS), default="fp64")
    ap.add_argument("--mixed-threshold", type=float, default=1e-6)
    ap.add_argument("--grad", action="store_true", help="energy + adjoint gradient")
    ap.add_argument("--repeat", type=int, default=1)
    a = ap.parse_args(argv)
    with tempfile.TemporaryDirectory() as d:
        path = a.input or configs.WORKLOADS[a.workload](os.path.join(d, a.workload + ".inp"))
        s = vg.System(path, precision=PRECISIONS[a.precision], mixed_threshold=a.mixed_threshold)
    for _ in range(a.repeat):
        if a.grad:
            r, gr = s.energy_grad()
            r["grad_norm"] = float((gr * gr).sum() ** 0.5)
        else:
            r = s.energy()
    print(json.dumps(r))


if __name__ == "__main__":
    main()
