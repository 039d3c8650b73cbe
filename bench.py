"""Benchmark: VSVB evaluations per second on one GB300, mixed precision
against plain FP64.

Workload (default, the largest configuration that runs on one GPU): the
128-atom alkane-like chain -- 42 Z=6 atoms in a zigzag at 1.54 A with 86 Z=1
atoms at 1.09 A, s/p/d basis of 1,576 Cartesian functions (C: 3s 2p 1d, H:
2s 1p 1d; 3-6 primitives, exponents log-uniform in [0.08, 3000]), 8 Rumer
spin-coupled pairs on neighbouring carbons (256 determinants per side,
65,536 determinant pairs) and 117 doubly occupied orbitals on 1-2 atoms with
seeded uniform(-1, 1) weights (valence_gb300.configs.alkane_chain, seed 4).
A step is one energy + adjoint gradient with respect to all 3,120 weights;
the determinant pairs are summed over their shared doubly occupied core in
closed form (vsvb_options.core_mode).  The same line reports the optimisation
loop that configuration defines ("loop": 20 descent steps on the mixed
path's gradient, each energy re-evaluated in FP64), the 64-atom Li/F cluster
("lif_cluster": 576 functions, 304 DOCC, energy only, block mode) and the
spin-coupled C/H chain ("ch_chain": 104 functions, 256 determinant pairs,
energy + gradient).

The headline value is the mixed path (VSVB_MIXED_DF64: FP32 for shell
quartets whose Schwarz bound is below 1e-6, double-float -- pairs of FP32
numbers, ~48-bit -- for the rest); the plain FP64 path and the FP32 +
native-FP64 split (VSVB_MIXED) are timed beside it, and |dE| of each against
FP64 is reported.

  value          device-resident weights
  e2e            public host API (vsvb_gpu_energy / vsvb_gpu_energy_grad):
                 pinned host weights copied in and the results copied out
                 every step
  roofline       block mode: the ERI launches and atom-quartet transforms of
                 the step (fork to join, CUDA events on the stream the
                 library launches on), algorithmic FLOPs per kind against the
                 FMA rates measured on this device (vsvb_gpu_fma_peak);
                 per-quartet mode: the ERI sweep's class launches
  cpu_baseline   the CPU oracle (a literal C restatement of the reference,
                 energy only) on all host cores: one full evaluation where it
                 finishes in seconds; on the cluster a bounded sample of every
                 phase (Schwarz table, one-electron loop, task loop),
                 extrapolated phase by phase and labelled so

--impl reference times that CPU restatement on the same workload and prints
the same metric.  Multi-GPU (torchrun): independent replicas, one per rank
("weak" scaling); the path needs no collective.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "VSVB energy+grad evals/s, mixed vs plain FP64 on 1 GB300 at |ΔE|<=1e-6 Eh"
# workloads whose configuration defines an energy evaluation only; any
# workload run in block mode is timed as energy evaluations as well
ENERGY_ONLY = {"lif_cluster", "lif_cluster_3"}
# workloads of seconds per step: their FP64 and FP32 + native-FP64 arms run
# fewer steps than the headline arm
LARGE = {"lif_cluster", "lif_cluster_3", "alkane_chain"}
# bounded CPU-oracle samples per phase (Schwarz entries, one-electron terms,
# two-electron tasks) for workloads whose full CPU evaluation takes hours;
# on the alkane chain one one-electron term or task of the oracle runs its
# factorisations of all 65,536 determinant pairs (about a minute)
CPU_SAMPLE = {"lif_cluster": (16, 16, 12), "lif_cluster_3": (16, 16, 12), "alkane_chain": (2, 2, 3)}


# dram__bytes_read.sum + dram__bytes_write.sum per launch of the dominant
# kernel, from the ncu captures summarised in profiles/.  Block mode: one
# blk_transform_kernel<df64> launch (a chunk of atom quartets) of the 4x4x4
# cluster, scaled from the 3x3x3 cluster's capture (149 KB per atom quartet,
# profiles/transform_lif_cluster_3.md) by the 15,570 atom quartets of a
# chunk.  Per-quartet path: keys (workload, class code).
PROFILED_TRAFFIC = {("lif_cluster", "transform_df64"): 2322444656,
                    # eri_kernel<2,2,2,1,df64,3> on the chain (profiles/eri_ch_chain.md)
                    ("ch_chain", 254): 1279232,
                    # eri_kernel<2,1,2,0,df64,3> on the 128-atom chain: the mean of its
                    # two launches per sweep (profiles/eri_alkane_chain.md)
                    ("alkane_chain", 243): 365088718}


def eri_roofline(sweep, sweep_wall, fp64_peak, fp32_peak, step_ms, workload):
    """Roofline of the ERI kernel: all class launches of one step's sweep, run
    concurrently on the library's side streams, timed in situ.

    sweep: {class code: [summed ms, summed FLOPs, launches]} over the timed
    steps; sweep_wall: fork-to-join ms per step.  Class code = 100*kind +
    10*bra + ket; kinds 0 FP64, 1 FP32, 2 double-float, 3 the FP32 tail
    (small primitive quartets) of an FP64-class schedule.  Per kind the bound
    rate for the algorithmic FLOPs (eri_flops: mostly component updates
    acc += x*y*z, 3 flops) is the measured FMA instruction rate (FMA peak / 2)
    times 3 flops per update over the instructions one update takes: 2 for
    FP32 and FP64 (MUL + FMA), 16 for double-float.
    T* = sum_kind W_kind / P_kind; frac = T* / T_sweep."""
    rate = {0: fp64_peak / 2 * 3 / 2, 1: fp32_peak / 2 * 3 / 2, 2: fp32_peak / 2 * 3 / 16, 3: fp32_peak / 2 * 3 / 2}
    kind_name = {0: "fp64", 1: "fp32", 2: "double-float", 3: "fp32 tail"}
    pair_l = ["s s", "p s", "p p", "d s", "d p", "d d"]
    W = {k: 0.0 for k in rate}
    for c, (_, fl, cnt) in sweep.items():
        W[c // 100] += fl / cnt
    t_star = sum(W[k] / rate[k] for k in rate)
    t_sweep = sum(sweep_wall) / len(sweep_wall) * 1e-3
    w_tot = sum(W.values())
    cls_top, (t_top, f_top, n_top) = max(sweep.items(), key=lambda kv: kv[1][0])
    return {"bound": "fp32_pipe",
            "kernel": "eri_kernel: every class launch of the step's ERI sweep (forward + adjoint), "
                      "concurrent on 6 streams",
            "achieved": w_tot / t_sweep / 1e12, "peak": w_tot / t_star / 1e12, "unit": "TFLOP/s",
            "frac": t_star / t_sweep,
            "achieved_unit_note": "algorithmic FP64-equivalent FLOPs of the Rys formulation (eri_flops) per "
                                  "second of sweep wall time",
            "peak_basis": "T* = sum over kinds of W_kind / P_kind; P = measured FMA instruction rate "
                          "(vsvb_gpu_fma_peak / 2) x 3 flops per component update / instructions per update "
                          "(2 FP32 or FP64, 16 double-float)",
            "flops_per_step": {kind_name[k]: W[k] for k in W}, "sweep_ms": t_sweep * 1e3,
            "sweeps_timed": len(sweep_wall), "share_of_step": t_sweep * 1e3 / step_ms,
            "traffic": PROFILED_TRAFFIC.get((workload, cls_top)),
            "traffic_note": "dram read+write bytes per launch of the longest class launch "
                            "(ncu capture summarised in profiles/)",
            "longest_launch": {"class": f"({pair_l[(cls_top // 10) % 10]}|{pair_l[cls_top % 10]}) "
                                        f"{kind_name[cls_top // 100]}",
                               "ms_in_situ": t_top / n_top, "flops": f_top / n_top},
            "fp64_fma_tflops": fp64_peak / 1e12, "fp32_fma_tflops": fp32_peak / 1e12}


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="alkane_chain")
    ap.add_argument("--mixed-threshold", type=float, default=1e-6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="time only the headline mixed arm (used for per-kernel launch lists)")
    ap.add_argument("--no-optimizer", action="store_true", help="skip the optimiser-path figures")
    ap.add_argument("--loop-steps", type=int, default=20,
                    help="descent steps of the alkane chain's optimisation loop; 0 skips it")
    ap.add_argument("--block-mode", default="auto", choices=["auto", "on", "off"],
                    help="vsvb_options.block_mode of the headline workload (auto: on for large s/p systems)")
    ap.add_argument("--batch", type=int, default=256,
                    help="molecules in the batched (one CUDA graph) measurement; 0 skips it")
    return ap.parse_args()


def _workload(name, d):
    from valence_gb300 import configs
    return configs.WORKLOADS[name](os.path.join(d, name + ".inp"))


class Clocks:
    """nvidia-smi sampler for the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.lines = []
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None

    def _read(self):
        for ln in self.p.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _oracle_energy_time(path, nthreads):
    """One full CPU-oracle energy evaluation (literal restatement of the
    reference) with nthreads host threads; returns seconds."""
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    exe = os.path.join(ROOT, "oracle", "_build", "vsvb_oracle")
    t = time.perf_counter()
    out = subprocess.run([exe, path, str(nthreads)], capture_output=True, text=True, check=True).stdout
    dt = time.perf_counter() - t
    e = float([ln for ln in out.splitlines() if "guess energy" in ln][0].split()[2])
    return dt, e


def _oracle_sampled_time(path, nthreads, samples):
    """Extrapolated CPU-oracle seconds of one full evaluation from bounded
    samples of every phase: every k-th Schwarz entry, one-electron term and
    two-electron task (vo_guess_energy_timed); each phase's time is scaled by
    its own sampling factor, the set-up counts once."""
    import math

    from tests import oracle_py
    from valence_gb300 import configs
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    dsc = configs.describe(path)
    nsp = dsc["spatial_orbitals"]
    nelec = 2 * (dsc["coupled_pairs"] + dsc["docc"]) + dsc["unpaired"]
    npairs = nsp * (nsp + 1) // 2
    n1, ntasks = nelec * nelec, npairs * (npairs + 1) // 2
    totals = (npairs, n1, ntasks)
    strides = tuple(max(1, n // k) for n, k in zip(totals, samples))
    o = oracle_py.Oracle(path)
    t = time.perf_counter()
    _, ph = o.guess_energy_timed(nthreads, *strides)
    wall = time.perf_counter() - t
    visited = [math.ceil(n / st) for n, st in zip(totals, strides)]
    full = ph[0] + sum(ph[k + 1] * totals[k] / visited[k] for k in range(3))
    sample = (f"extrapolated: the CPU oracle (literal C restatement of valence.F90's guess energy, energy only) "
              f"timed on every {strides[0]}th Schwarz entry ({visited[0]} of {npairs}), every {strides[1]}th "
              f"one-electron term ({visited[1]} of {n1}) and every {strides[2]}th task ({visited[2]} of {ntasks}); "
              f"each phase scaled by its sampling factor, set-up once; phase seconds {[round(x, 3) for x in ph]}, "
              f"sample wall {wall:.1f} s")
    return full, wall, sample


def _cpu_seconds(workload, path, cores):
    """(seconds of one full CPU-oracle evaluation, sample description)."""
    if workload in CPU_SAMPLE:
        full, _, sample = _oracle_sampled_time(path, cores, CPU_SAMPLE[workload])
        return full, sample
    dt, _ = _oracle_energy_time(path, cores)
    return dt, ("one full energy evaluation of the same workload by the CPU oracle (literal C restatement of "
                "valence.F90's guess energy, cached AO shell-quartet blocks); energy only, the reference has no "
                "gradient")


def _config(a, workload, path, world, grad=None):
    import inspect

    from valence_gb300 import configs
    c = {"workload": workload,
         "seed": inspect.signature(configs.WORKLOADS[workload]).parameters["seed"].default}
    c.update(configs.describe(path))
    if grad is None:
        grad = workload not in ENERGY_ONLY
    c["step"] = ("one energy + adjoint gradient with respect to every weight" if grad
                 else "one guess energy (the configuration defines no gradient)")
    c.update({"mixed_threshold": a.mixed_threshold, "l2": "flushed (256 MB write) between timed steps",
              "replicas": world})
    return c


def run_reference(a, rank, world):
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    steps = max(1, min(a.steps, (1 if a.workload == "alkane_chain" else 2) if a.workload in CPU_SAMPLE else 3))
    with tempfile.TemporaryDirectory() as d:
        path = _workload(a.workload, d)
        times = []
        for _ in range(steps):
            dt, sample = _cpu_seconds(a.workload, path, cores)
            times.append(dt)
        cfg = _config(a, a.workload, path, world)
    v = 1.0 / statistics.mean(times)
    sample = f"{steps} step(s), each: " + sample + f"; steps capped at {steps}"
    print(json.dumps({"impl": "reference", "metric": METRIC, "value": v, "unit": "evals/s", "n_gpus": world,
                      "steps": steps, "warmup": 0, "ms_per_step": 1e3 * statistics.mean(times),
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic", "config": cfg,
                      "cpu_baseline": {"value": v, "unit": "evals/s", "cores": cores, "kind": "port",
                                       "sample": sample},
                      "e2e": {"value": v, "unit": "evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))


def block_roofline(stats, block_ms, fp64_peak, fp32_peak, step_ms):
    """Roofline of block mode: the ERI launches (one lane per shell quartet
    for the small s/p classes, the CTA kernel for (pp|pp)) and the
    per-atom-quartet transforms of one step, chunk after chunk, on 6 side
    streams and the handle's stream, timed fork to join by CUDA events on
    those streams (block_ms per step).  Per kind the bound rate for the
    algorithmic FLOPs: ERIs as in eri_roofline (FMA instruction rate x 3
    flops per component update / 2 instructions, 16 in double-float);
    transforms FP64 / FP32 at the FMA FLOP rate, double-float at 2 flops per
    multiply-add of 12 FP32 instructions.  T* = sum W_kind / P_kind,
    frac = T* / T_block."""
    rate = {("eri", "fp64"): fp64_peak / 2 * 3 / 2, ("eri", "fp32"): fp32_peak / 2 * 3 / 2,
            ("eri", "df64"): fp32_peak / 2 * 3 / 16, ("transform", "fp64"): fp64_peak,
            ("transform", "fp32"): fp32_peak, ("transform", "df64"): fp32_peak / 12}
    W = {("eri", k): v for k, v in stats["eri_flops"].items()}
    W.update({("transform", k): v for k, v in stats["transform_flops"].items()})
    t_star = sum(W[k] / rate[k] for k in W)
    t_block = statistics.mean(block_ms) * 1e-3
    w_tot = sum(W.values())
    return {"bound": "fp32_pipe",
            "kernel": "block mode: eri_lane_kernel / eri_kernel<1,1,1,1,*,4> ERI launches and "
                      "blk_transform_kernel per chunk of atom quartets (one step: "
                      f"{stats['chunks']} chunks, {stats['launches']} launches)",
            "achieved": w_tot / t_block / 1e12, "peak": w_tot / t_star / 1e12, "unit": "TFLOP/s",
            "frac": t_star / t_block,
            "achieved_unit_note": "algorithmic FLOPs (eri_flops per primitive quartet + transfer; four quarter "
                                  "transforms per atom quartet) per second of the block phase",
            "peak_basis": "T* = sum over kinds of W_kind / P_kind with the FMA rates of vsvb_gpu_fma_peak",
            "flops_per_step": {f"{a}_{b}": v for (a, b), v in W.items()},
            "block_phase_ms": t_block * 1e3, "share_of_step": t_block * 1e3 / step_ms,
            "traffic": PROFILED_TRAFFIC.get(("lif_cluster", "transform_df64")),
            "traffic_note": "dram read+write bytes per launch of blk_transform_kernel<df64> (one chunk of atom "
                            "quartets), from the ncu capture summarised in profiles/",
            "fp64_fma_tflops": fp64_peak / 1e12, "fp32_fma_tflops": fp32_peak / 1e12}


def measure(a, workload, world, dev, stream, flush, steps, warmup, side_steps, side_warmup, cpu=True):
    """One workload: the mixed (double-float) arm over exactly `steps` timed
    steps with its roofline timing, then the FP64 and VSVB_MIXED arms
    (side_steps each) and the host-API arm (steps), one handle at a time."""
    import torch

    import valence_gb300 as vg
    from valence_gb300 import api
    bm = {"auto": 0, "on": 1, "off": -1}[a.block_mode] if workload == a.workload else 0
    grad = workload not in ENERGY_ONLY and bm != 1

    def timed(fn, steps, warmup, after_step=None):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ms, launches, last = [], 0, None
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            last = fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            launches += last["n_kernel_launches"]
            if after_step is not None:
                after_step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        return ms, launches, last

    def agg(ms):
        t = torch.tensor([sum(ms)], dtype=torch.float64, device="cuda")
        if world > 1:
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        return t.item()

    with tempfile.TemporaryDirectory() as d:
        path = _workload(workload, d)
        cfg = _config(a, workload, path, world, grad)

        def system(prec):
            s = vg.System(path, precision=prec, mixed_threshold=a.mixed_threshold, device=dev, block_mode=bm)
            s.set_stream(stream.cuda_stream)
            return s

        def dev_step(s, w_dev, g_dev):
            if grad:
                return lambda: s.energy_grad_device(w_dev.data_ptr(), g_dev.data_ptr())
            return lambda: s.energy_device(w_dev.data_ptr())

        def host_step(s, w_pin, g_pin):
            P = api.ctypes.POINTER(api.ctypes.c_double)

            def f():
                r = api.Result()
                if grad:
                    rc = api.lib().vsvb_gpu_energy_grad(s._h, w_pin.numpy().ctypes.data_as(P), api.ctypes.byref(r),
                                                        g_pin.numpy().ctypes.data_as(P))
                else:
                    rc = api.lib().vsvb_gpu_energy(s._h, w_pin.numpy().ctypes.data_as(P), api.ctypes.byref(r))
                if rc:
                    raise api.VSVBError(api.lib().vsvb_gpu_last_error(s._h).decode())
                return r.as_dict()
            return f

        out = {"config": cfg}
        smx = system(vg.MIXED_DF64)
        n = smx.totlen
        w_dev = torch.from_numpy(smx.coeff0.copy()).to("cuda")
        g_dev = torch.zeros(n, dtype=torch.float64, device="cuda")
        w_pin = torch.from_numpy(smx.coeff0.copy()).pin_memory()
        g_pin = torch.zeros(n, dtype=torch.float64).pin_memory()
        stats = smx.block_stats()
        core = smx.core_stats()
        if core["on"]:
            cfg["determinant_pair_sum"] = (f"core mode (vsvb_options.core_mode): {core['determinant_pairs']} "
                                           f"determinant pairs summed over the shared doubly occupied core in "
                                           f"closed form; pair sums in FP64, the orbital-pair GEMMs in "
                                           f"double-float on the mixed path (FP64 on the FP64 path); "
                                           f"pair-summed density GEMM {core['gemm_fma']:.3g} FMAs per energy")
        sweep, sweep_wall = {}, []

        def collect():
            if not stats["on"]:
                for x in smx.sweep_times():
                    acc = sweep.setdefault(x["cls"], [0.0, 0.0, 0])
                    acc[0] += x["ms"]
                    acc[1] += x["flops"]
                    acc[2] += 1
            sweep_wall.append(smx.sweep_wall_ms())

        smx.set_sweep_timing(True)
        clk = Clocks(dev)
        clk.start()
        ms_mx, launches_mx, r_mx = timed(dev_step(smx, w_dev, g_dev), steps, warmup, after_step=collect)
        out["clocks"] = clk.stop()
        smx.set_sweep_timing(False)
        out["ms_mx"], out["launches"], out["r_mx"] = ms_mx, launches_mx, r_mx
        out["value"] = world * steps / (agg(ms_mx) * 1e-3)
        fp64_peak, fp32_peak = api.fma_peak(dev)
        if stats["on"]:
            out["roofline"] = block_roofline(stats, sweep_wall, fp64_peak, fp32_peak, statistics.mean(ms_mx))
        else:
            out["roofline"] = eri_roofline(sweep, sweep_wall, fp64_peak, fp32_peak, statistics.mean(ms_mx), workload)
        if a.headline_only:
            smx.close()
            return out
        ms_e2e, _, _ = timed(host_step(smx, w_pin, g_pin), steps, warmup)
        out["e2e"] = {"value": world * steps / (agg(ms_e2e) * 1e-3), "unit": "evals/s",
                      "h2d_bytes_per_step": 8 * n,
                      "d2h_bytes_per_step": (8 * n if grad else 0) + 8 * 7 + 8 * 5 + 4 * 2}
        smx.close()
        for name, prec in (("fp64", vg.FP64), ("mixed_native_fp64", vg.MIXED)):
            s = system(prec)
            ms_s, _, r_s = timed(dev_step(s, w_dev, g_dev), side_steps, side_warmup)
            out[name] = {"value": world * side_steps / (agg(ms_s) * 1e-3), "unit": "evals/s",
                         "ms_per_step": statistics.mean(ms_s), "steps": side_steps, "warmup": side_warmup,
                         "energy": r_s["energy"], "err_est": r_s["err_est"]}
            s.close()
        e64 = out["fp64"]["energy"]
        out["mixed_native_fp64"]["abs_dE_vs_fp64"] = abs(out["mixed_native_fp64"]["energy"] - e64)
        out["mixed_over_fp64"] = out["value"] / out["fp64"]["value"]
        out["mixed_native_over_fp64"] = out["mixed_native_fp64"]["value"] / out["fp64"]["value"]
        out["abs_dE_mixed_vs_fp64"] = abs(r_mx["energy"] - e64)
        out["err_est_mixed"] = r_mx["err_est"]
        if world == 1 and cpu and not a.no_cpu_baseline:
            cores = os.cpu_count() or 1
            dt, sample = _cpu_seconds(workload, path, cores)
            out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "evals/s", "cores": cores, "kind": "port",
                                   "sample": sample}
    return out


def run_ours(a, rank, world):
    import torch

    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")  # 256 MB > 126 MB L2
    large = a.workload in LARGE or a.block_mode == "on"
    # the FP64 and FP32 + native FP64 arms of a large workload are timed on
    # fewer steps than the headline arm: they are reported beside it, not as
    # the headline
    side_steps = min(a.steps, 3) if large else a.steps
    side_warmup = 1 if large else a.warmup
    m = measure(a, a.workload, world, dev, stream, flush, a.steps, a.warmup, side_steps, side_warmup)
    if rank != 0:
        return
    r = m["r_mx"]
    out = {"metric": METRIC, "value": m["value"], "unit": "evals/s", "n_gpus": world, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": statistics.mean(m["ms_mx"]), "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None,
           "dtype": ("f32 (Schwarz < 1e-6) + double-float (2xf32) elsewhere; f64 determinants and reductions"),
           "data": "synthetic", "config": m["config"], "gpu_launches": m["launches"],
           "roofline": m["roofline"], "clocks": m["clocks"],
           "quartets": {"fp64": r["n_quartets_fp64"], "fp32": r["n_quartets_fp32"],
                        "total": r["n_quartets_fp64"] + r["n_quartets_fp32"],
                        "primitive": r["n_prim_quartets"], "primitive_fp32": r["n_prim_quartets_fp32"]},
           "tasks": r["n_tasks"], "energy_mixed": r["energy"]}
    if a.headline_only:
        out["note"] = "headline mixed arm only (per-kernel launch-list run)"
        print(json.dumps(out))
        return
    for k in ("e2e", "fp64", "mixed_native_fp64", "mixed_over_fp64", "mixed_native_over_fp64",
              "abs_dE_mixed_vs_fp64", "err_est_mixed", "cpu_baseline"):
        out[k] = m.get(k)
    # the figures below run on rank 0 alone (the other ranks have left):
    # one replica, no cross-rank barrier
    if a.workload == "alkane_chain" and a.loop_steps > 0:
        out["loop"] = run_loop(a, dev, stream)
    if a.workload != "lif_cluster":
        c = measure(a, "lif_cluster", 1, dev, stream, flush, min(a.steps, 3), 1, 2, 1, cpu=False)
        out["lif_cluster"] = {"config": c["config"], "value": c["value"], "unit": "energy evals/s",
                              "ms_per_step": statistics.mean(c["ms_mx"]), "e2e": c["e2e"], "fp64": c["fp64"],
                              "mixed_native_fp64": c["mixed_native_fp64"], "mixed_over_fp64": c["mixed_over_fp64"],
                              "mixed_native_over_fp64": c["mixed_native_over_fp64"],
                              "abs_dE_mixed_vs_fp64": c["abs_dE_mixed_vs_fp64"], "err_est_mixed": c["err_est_mixed"],
                              "roofline": c["roofline"], "gpu_launches": c["launches"], "clocks": c["clocks"],
                              "cpu_baseline_note": "the CPU oracle's sampled cluster evaluation is timed by "
                                                   "bench.py --workload lif_cluster"}
    if a.workload != "ch_chain":
        c = measure(a, "ch_chain", 1, dev, stream, flush, a.steps, a.warmup, a.steps, a.warmup)
        out["ch_chain"] = {"config": c["config"], "value": c["value"], "unit": "energy+grad evals/s",
                           "ms_per_step": statistics.mean(c["ms_mx"]), "e2e": c["e2e"], "fp64": c["fp64"],
                           "mixed_native_fp64": c["mixed_native_fp64"], "mixed_over_fp64": c["mixed_over_fp64"],
                           "mixed_native_over_fp64": c["mixed_native_over_fp64"],
                           "abs_dE_mixed_vs_fp64": c["abs_dE_mixed_vs_fp64"], "roofline": c["roofline"],
                           "cpu_baseline": c.get("cpu_baseline"), "gpu_launches": c["launches"]}

    def timed_simple(fn, steps, warmup):
        import torch
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        ms, launches, last = [], 0, None
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            last = fn()
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
            launches += last["n_kernel_launches"]
        torch.cuda.synchronize()
        return ms, launches, last

    out["water"] = run_water(a, timed_simple, dev)
    if a.batch > 0:
        out["batch"] = run_batch(a, timed_simple, 1)
    if not a.no_optimizer:
        out["optimizer"] = run_optimizer(a, dev)
    print(json.dumps(out))


def run_loop(a, dev, stream):
    """The alkane chain's optimisation loop: a.loop_steps steepest-descent
    steps on all weights with the mixed path's adjoint gradient and an Armijo
    line search on mixed energies (valence_gb300.loop.descend), each
    accepted point's energy re-evaluated in plain FP64 (|dE| <= 1e-6 Eh is
    the acceptance bar of the configuration)."""
    import valence_gb300 as vg
    from valence_gb300 import loop
    with tempfile.TemporaryDirectory() as d:
        path = _workload("alkane_chain", d)
        smx = vg.System(path, precision=vg.MIXED_DF64, mixed_threshold=a.mixed_threshold, device=dev)
        s64 = vg.System(path, precision=vg.FP64, device=dev)
        smx.set_stream(stream.cuda_stream)
        s64.set_stream(stream.cuda_stream)
        smx.energy_grad()
        s64.energy()
        t = time.perf_counter()
        _, recs = loop.descend(smx, steps=a.loop_steps, check=s64)
        wall = time.perf_counter() - t
        smx.close()
        s64.close()
    dmax = max(r["abs_dE_vs_check"] for r in recs)
    return {"steps": len(recs), "wall_s": wall, "s_per_step": wall / len(recs),
            "mixed_s_per_step": sum(r["seconds"] for r in recs) / len(recs),
            "fp64_check_s_per_step": sum(r["check_seconds"] for r in recs) / len(recs),
            "evaluations": sum(r["evaluations"] for r in recs),
            "energy_first": recs[0]["energy"], "energy_last": recs[-1]["energy"],
            "max_abs_dE_mixed_vs_fp64": dmax, "within_1e-6": dmax <= 1e-6,
            "energies": [r["energy"] for r in recs], "abs_dE": [r["abs_dE_vs_check"] for r in recs],
            "method": "steepest descent on all weights, Armijo backtracking on mixed energies "
                      "(valence_gb300.loop.descend); FP64 energy at every accepted point"}


def run_optimizer(a, dev):
    """The optimiser path (vsvb_opt_*: first_order_opt's H/S as adjoint
    columns, rsg, minimize_energy) on the reference's own optimisation test
    input c2-pt-vshf-p2 (a committed fixture; its optimised energy is pinned
    at 1e-6 Eh by testing/testing.py) with the CPU oracle's literal H/S build
    of the same orbital -- nb(nb+1)/2 transition energies, valence.F90:679-703
    -- timed beside it, and the H/S build of one DOCC orbital of the headline
    workload in FP64 and double-float."""
    import numpy as np

    from valence_gb300 import api
    from tests import oracle_py
    case = [c for c in oracle_py.goldens()["cases"] if c["converged"] and c["name"] == "c2-pt-vshf-p2"][0]
    path = os.path.join(oracle_py.GOLDEN, case["input"])
    opt = api.Optimizer(path, device=dev)
    iorb = 3
    opt.first_order_hs(iorb)
    t = time.perf_counter()
    h, s = opt.first_order_hs(iorb)
    t_hs = time.perf_counter() - t
    t = time.perf_counter()
    res, _, _ = opt.minimize()
    t_min = time.perf_counter() - t
    opt.close()
    cores = os.cpu_count() or 1
    o = oracle_py.OptOracle(path)
    t = time.perf_counter()
    h_ref, s_ref = o.first_order_hs(iorb, cores)
    t_cpu = time.perf_counter() - t
    out = {"input": "c2-pt-vshf-p2 (reference test input; C2, 2 unpaired + 5 DOCC, 76 weights)",
           "hs_orbital": iorb, "hs_order": int(h.shape[0]),
           "hs_gpu_ms": 1e3 * t_hs, "hs_cpu_oracle_s": t_cpu, "hs_cpu_cores": cores,
           "hs_speedup": t_cpu / t_hs, "hs_max_rel_diff": float(np.max(np.abs(h - h_ref)) / np.max(np.abs(h_ref))),
           "minimize_s": t_min, "minimize_energy": res["energy"], "golden_energy": case["total_energy"],
           "minimize_abs_dE": abs(res["energy"] - case["total_energy"]), "iterations": res["iterations"],
           "hs_builds": res["n_hs_builds"]}
    with tempfile.TemporaryDirectory() as d:
        wpath = _workload("ch_chain", d)
        for name, prec in (("fp64", api.FP64), ("double_float", api.MIXED_DF64)):
            opt = api.Optimizer(wpath, precision=prec, device=dev)
            iorb = opt.desc_counts()["nnd"] + 1  # the first DOCC orbital
            opt.first_order_hs(iorb)
            t = time.perf_counter()
            opt.first_order_hs(iorb)
            out[f"ch_chain_hs_{name}_ms"] = 1e3 * (time.perf_counter() - t)
            out["ch_chain_hs_order"] = int(opt.map_orbs[iorb] - opt.map_orbs[iorb - 1])
            opt.close()
    return out


def run_water(a, timed, dev):
    """The reference's CPU-runnable configuration (H2O, 13 functions, 5
    DOCC; a parity case): energy + gradient per second in FP64 and on the
    mixed path, device-resident weights, with the oracle's energy beside it."""
    import torch

    import valence_gb300 as vg
    from valence_gb300 import configs
    out = {"workload": "water_vshf (H2O, 13 functions, 5 DOCC)"}
    with tempfile.TemporaryDirectory() as d:
        p = configs.water_vshf(os.path.join(d, "water.inp"))
        for name, prec in (("fp64", vg.FP64), ("mixed_df64", vg.MIXED_DF64)):
            s = vg.System(p, precision=prec, device=dev)
            s.set_stream(torch.cuda.current_stream().cuda_stream)
            w = torch.tensor(s.coeff0, dtype=torch.float64, device="cuda")
            g = torch.zeros(s.totlen, dtype=torch.float64, device="cuda")
            ms, _, r = timed(lambda: s.energy_grad_device(w.data_ptr(), g.data_ptr()), max(a.steps, 10), a.warmup)
            out[name] = {"value": 1e3 / statistics.mean(ms), "unit": "evals/s", "ms_per_step": statistics.mean(ms),
                         "energy": r["energy"]}
            s.close()
        if not a.no_cpu_baseline:
            dt, e = _oracle_energy_time(p, os.cpu_count() or 1)
            out["cpu_baseline"] = {"value": 1.0 / dt, "unit": "evals/s", "cores": os.cpu_count() or 1,
                                   "kind": "port", "sample": "one full energy evaluation by the CPU oracle",
                                   "dE_vs_gpu_fp64": abs(e - out["fp64"]["energy"])}
    return out


def run_batch(a, timed, world):
    """Batched energy + gradient: a.batch independent random molecules (2-12
    atoms, Z in {1,3,6,7,8,9}, 4-80 functions, 0-2 coupled pairs; seeds from
    1000, every draw kept -- those with singular determinant pairs counted)
    on the mixed path, all evaluated by one CUDA-graph launch per step
    (vsvb_batch)."""
    import torch

    import valence_gb300 as vg
    from valence_gb300 import configs
    systems, singular, seed = [], 0, 1000
    with tempfile.TemporaryDirectory() as d:
        while len(systems) < a.batch:
            p = configs.random_molecule(os.path.join(d, f"m{seed}.inp"), seed)
            seed += 1
            s = vg.System(p, precision=vg.MIXED_DF64)
            r, _ = s.energy_grad()
            singular += r["n_singular_pairs"] > 0
            systems.append((s, p))
        # CPU baseline: the oracle on every 16th molecule, all host cores
        cpu_s, sample = 0.0, systems[::16]
        if not a.no_cpu_baseline:
            for _, p in sample:
                dt, _ = _oracle_energy_time(p, os.cpu_count() or 1)
                cpu_s += dt
    systems = [s for s, _ in systems]
    ws = [torch.tensor(s.coeff0, dtype=torch.float64, device="cuda") for s in systems]
    gs = [torch.zeros(s.totlen, dtype=torch.float64, device="cuda") for s in systems]
    b = vg.Batch(systems)
    stream = torch.cuda.current_stream().cuda_stream
    wp, gp = [w.data_ptr() for w in ws], [g.data_ptr() for g in gs]

    def step():
        res = b.energy_grad_device(wp, gp, stream=stream)
        return {"n_kernel_launches": b.launches, "energy": res[0]["energy"]}
    ms, launches, _ = timed(step, max(2, min(a.steps, 5)), a.warmup)
    t = sum(ms) / len(ms)
    nf = [s.totlen for s in systems]
    out = {"workload": f"{len(systems)} random molecules, 4-80 functions, mixed path, one CUDA graph per step",
           "value": world * len(systems) / (t * 1e-3), "unit": "molecule energy+grad evals/s",
           "ms_per_step": t, "kernels_per_graph_launch": b.launches, "molecules_with_singular_pairs": singular,
           "weights_total": int(sum(nf))}
    if cpu_s > 0:
        out["cpu_baseline"] = {"value": len(sample) / cpu_s, "unit": "molecule energy evals/s",
                               "cores": os.cpu_count() or 1, "kind": "port",
                               "sample": f"the CPU oracle's full energy of every 16th molecule ({len(sample)} of "
                                         f"{len(systems)}), one at a time on all host cores; energy only"}
    b.close()
    for s in systems:
        s.close()
    return out


def main():
    a = _args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl" if a.impl == "ours" else "gloo")
    if a.impl == "reference":
        run_reference(a, rank, world)
    else:
        run_ours(a, rank, world)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
