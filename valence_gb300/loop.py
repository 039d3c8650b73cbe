"""Gradient-driven orbital optimisation: steepest descent on the LCAO weights
with the GPU adjoint gradient of one precision (normally the mixed path) and
the energy at every accepted point re-evaluated by a second handle (normally
plain FP64).

The reference optimises orbital by orbital (minimize_energy,
valence.F90:2744-2885, built here as vsvb_opt_*); this loop instead steps
all weights along -dE/dw at once.  The energy is invariant to each orbital's
scale (the weights are normalised internally), so the gradient is
orthogonal to every orbital's weight vector.  The step length follows an
Armijo backtracking line search on the same handle's energies:
E(w - a g) <= E(w) - c1 a |g|^2, a halved (from the last accepted length
times 2) until it holds."""
import time

import numpy as np


def descend(system, steps=20, check=None, weights=None, c1=1e-4, max_backtrack=30):
    """Run `steps` accepted descent steps from `weights` (default: the
    input's weights).  Returns (weights, records): one record per step with
    the energy, the check handle's energy at the same weights and their
    difference, the gradient norm, the step length and the evaluations and
    seconds it took."""
    w = np.array(system.coeff0 if weights is None else weights, dtype=np.float64)
    r, g = system.energy_grad(w)
    e = r["energy"]
    gn2 = float(g @ g)
    alpha = 0.1 * float(np.max(np.abs(w))) / max(float(np.max(np.abs(g))), 1e-300)
    records = []
    for k in range(steps):
        t0 = time.perf_counter()
        evals = 0
        a = 2.0 * alpha
        for _ in range(max_backtrack):
            wt = w - a * g
            et = system.energy(wt)["energy"]
            evals += 1
            if et <= e - c1 * a * gn2:
                break
            a *= 0.5
        else:
            raise RuntimeError(f"no descent step found at step {k}")
        alpha = a
        w = wt
        r, g = system.energy_grad(w)
        evals += 1
        e_new = r["energy"]
        gn2 = float(g @ g)
        rec = {"step": k + 1, "energy": e_new, "decrease": e - e_new, "grad_norm": gn2 ** 0.5, "alpha": a,
               "evaluations": evals, "seconds": time.perf_counter() - t0}
        e = e_new
        if check is not None:
            t1 = time.perf_counter()
            ec = check.energy(w)["energy"]
            rec.update({"check_energy": ec, "abs_dE_vs_check": abs(e - ec),
                        "check_seconds": time.perf_counter() - t1})
        records.append(rec)
    return w, records
