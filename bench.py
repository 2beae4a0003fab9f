#!/usr/bin/env python3
"""Benchmark: ALS-sweep nonzeros/s of the sparse Tucker sweep on one GB300.

Workload (the headline configuration): a 4-order 100,000^4 tensor with 100M
distinct nonzeros, each mode's index Zipf(s=1.1) over a seeded permutation of
the axis, values uniform [0,1) FP32, Tucker rank 10, partition P_n = 4 on every
mode (256 blocks), plain FP32 sweep.  Synthetic data from the project's seeded
generator (the reference's published datasets are not available).

A step is one ALS sweep: the factor update of modes 0..3 (delta, Gram/RHS,
row solves) and the reconstruction fit, i.e. UpdateFactorMatrices +
Reconstruction of the reference.  Unit of work: one nonzero visited in one mode
update, so value = N * nnz * K / t (nnz/s per sweep).

  value ........ device time (CUDA events on the library's stream) of K sweeps on
                 the HBM-resident tensor; inputs (8 GB of views) are far larger
                 than the 129 MB L2.
  e2e .......... the whole job through the C ABI with host buffers: upload the
                 pinned host COO, partition and segment it on the GPU, initialise,
                 run the configuration's sweeps with a fit each, and read the
                 factors back -- N * nnz * sweeps / wall time.
  roofline ..... the dominant kernel (fused delta + Gram/RHS): SURVEY's compulsory
                 delta bytes (4N + 4J per nonzero and mode) per launch over its
                 event-timed duration, against the measured HBM copy bandwidth.
  cpu_baseline . the CPU restatement of the reference (its OpenMP delta/B,C/Eigen
                 path, oracle/gtk_oracle.cpp) on a bounded sample of the same
                 tensor, all host threads.

--impl reference times that CPU path alone (the reference's own code is CPU +
an sm_70 SIMT kernel with no Blackwell build; the restatement is its path).
Under torchrun every rank runs an independent replica ("replicas only": the
sweep has no data-path exchange on one GPU per process).
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(
    workload="zipf4d_100M_rank10_P4", order=4, dims=[100_000] * 4, nnz=100_000_000, zipf_s=1.1,
    rank=10, partition=[4, 4, 4, 4], dtype="f32", sweeps=10, seed=0,
)


def args_parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--nnz", type=int, default=None, help="override nnz (smaller runs)")
    p.add_argument("--e2e-runs", type=int, default=1)
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--cpu-sample", type=int, default=500_000, help="nonzeros in the CPU baseline sample")
    p.add_argument("--ref-sample", type=int, default=200_000, help="nonzeros per reference-arm step")
    p.add_argument("--precision", choices=["plain", "bf16", "tf32"], default="plain")
    return p.parse_args()


# ------------------------------------------------------------------ distributed (replicas)
class Dist:
    def __init__(self, impl):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = "nccl" if impl == "ours" and torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.dist, self.torch, self.backend = dist, torch, backend

    def barrier(self):
        if self.world > 1:
            self.dist.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        dev = f"cuda:{self.local}" if self.backend == "nccl" else "cpu"
        t = self.torch.tensor([x], dtype=self.torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.world > 1:
            self.dist.destroy_process_group()


# ------------------------------------------------------------------ clocks
class Clocks:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.p = None
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(device)], stdout=subprocess.PIPE,
                                      stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        try:
            out, _ = self.p.communicate(timeout=10)
        except Exception:
            self.p.kill()
            return None
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ CPU baseline (oracle)
def cpu_baseline(coo, cfg, sample: int, steps: int = 1):
    """The reference's CPU path (restated in oracle/) on the first `sample` nonzeros."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np

    from oracle_util import Oracle, ora_lib
    idx, vals = coo.arrays()
    s = min(sample, coo.nnz)
    sidx = [np.ascontiguousarray(i[:s]) for i in idx]
    svals = np.ascontiguousarray(vals[:s])
    ora = Oracle(0, sidx, svals, coo.dims, cfg["partition"], cfg["rank"])
    if ora.status:
        raise RuntimeError("oracle rejected the sample")
    ora.init_random(1, 0)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        ora.sweep()
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    return {
        "value": cfg["order"] * s / t, "unit": "nnz/s", "cores": int(ora_lib().ora_num_threads()), "kind": "port",
        "sample": f"first {s} nonzeros of the workload tensor (same dims, P, rank), {steps} full sweep(s), "
                  f"median {t:.2f} s per sweep",
    }


def gen_workload(cfg, nnz):
    import gputucker_gb300 as gtk
    t0 = time.perf_counter()
    coo = gtk.generate(cfg["order"], cfg["dims"], nnz, "zipf", cfg["zipf_s"], "uniform", cfg["dtype"], seed=cfg["seed"])
    return coo, time.perf_counter() - t0


def run_reference(args, cfg, dist):
    if dist.rank != 0:
        return
    nnz = args.nnz or cfg["nnz"]
    coo, _ = gen_workload(cfg, min(nnz, args.ref_sample * 4))
    steps = max(1, args.steps)
    import numpy as np  # noqa: F401
    res = None
    vals = []
    for _ in range(args.warmup and 1):
        cpu_baseline(coo, cfg, args.ref_sample, 1)
    for _ in range(steps):
        res = cpu_baseline(coo, cfg, args.ref_sample, 1)
        vals.append(res["value"])
    v = statistics.median(vals)
    res["value"] = v
    line = {
        "impl": "reference", "metric": "ALS-sweep nnz/s (plain FP32, 1 device)", "value": v, "unit": "nnz/s",
        "n_gpus": dist.world, "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * cfg["order"] * args.ref_sample / v,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {k: cfg[k] for k in ("workload", "order", "dims", "zipf_s", "rank", "partition", "dtype")}
        | {"nnz": nnz, "sample_nnz": min(args.ref_sample, coo.nnz)},
        "cpu_baseline": res,
        "e2e": {"value": v, "unit": "nnz/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = args_parse()
    cfg = dict(WORKLOAD)
    dist = Dist(args.impl)
    if args.impl == "reference":
        run_reference(args, cfg, dist)
        dist.close()
        return
    import gputucker_gb300 as gtk
    from gputucker_gb300 import _native
    _native.load()
    nnz = args.nnz or cfg["nnz"]
    N, J = cfg["order"], cfg["rank"]
    coo, gen_s = gen_workload(cfg, nnz)
    coo.pin()
    device = dist.local
    # ---- device-resident sweeps
    t = gtk.create_tensor_blocks(coo, cfg["partition"], J, device=device)
    t.init_random(1, 0)
    t.set_precision(args.precision)
    for _ in range(max(3, args.warmup)):
        t.update_factor_matrices()
        t.reconstruction()
    t.profile(True)
    t.profile_reset()
    clocks = Clocks(device)
    dist.barrier()
    t.synchronize()
    t.timer_begin()
    fits = []
    for _ in range(args.steps):
        t.update_factor_matrices()
        fits.append(t.reconstruction())
    ms = t.timer_end()
    t.synchronize()
    dist.barrier()
    clk = clocks.stop()
    ms = dist.max(ms)
    k_ms, k_n = t.profile_read(0)
    s_ms, s_n = t.profile_read(1)
    f_ms, f_n = t.profile_read(2)
    launches = int(t.profile_read(4)[1])  # kernels the library launched in the timed region
    t.profile(False)
    ms_step = ms / args.steps
    value = dist.world * N * nnz * args.steps / (ms / 1e3)
    # ---- roofline of the dominant kernel (fused delta + Gram/RHS)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    per_launch_s = (k_ms / max(1, k_n)) / 1e3
    bytes_per_launch = nnz * (4 * N + 4 * J)
    flops_delta = 2 * sum(J ** m for m in range(2, N + 1)) + 2 * (J * J + J)
    achieved = bytes_per_launch / per_launch_s / 1e9
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            tr = json.load(f)
        if "fused_delta_gram_bytes_per_nnz" in tr:
            traffic = tr["fused_delta_gram_bytes_per_nnz"] * nnz
    except Exception:
        pass
    roofline = {
        "bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak,
        "traffic": traffic,
        "kernel": ("k_mode_spec<float,4,10,2,kUpdate>" if args.precision == "plain"
                   else f"k_mode_tc<10,3,{args.precision},update>") + " (fused delta + Gram/RHS)",
        "bytes_per_launch": bytes_per_launch, "launch_ms": per_launch_s * 1e3,
        "fp32_tflops": nnz * flops_delta / per_launch_s / 1e12, "fp32_peak_tflops_nominal": 80.6,
        "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
    }
    kernels = {
        "delta_gram": {"launches": k_n, "ms_per_launch": k_ms / max(1, k_n)},
        "row_solve": {"launches": s_n, "ms_per_launch": s_ms / max(1, s_n)},
        "fit": {"launches": f_n, "ms_per_launch": f_ms / max(1, f_n)},
    }
    t.close()
    # ---- end to end through the C ABI with host buffers
    e2e = None
    if not args.no_e2e:
        import numpy as np
        walls = []
        sweeps = cfg["sweeps"]
        h2d = sum(4 * nnz for _ in range(N)) + 4 * nnz
        for _ in range(max(1, args.e2e_runs)):
            dist.barrier()
            t0 = time.perf_counter()
            tt = gtk.create_tensor_blocks(coo, cfg["partition"], J, device=device)
            tt.init_random(1, 0)
            tt.set_precision(args.precision)
            for _ in range(sweeps):
                tt.update_factor_matrices()
                tt.reconstruction()
            facs = [tt.get_factor(n) for n in range(N)]
            walls.append(time.perf_counter() - t0)
            fbytes = sum(f.nbytes for f in facs)
            tt.close()
        wall = dist.max(min(walls))
        e2e = {
            "value": dist.world * N * nnz * sweeps / wall, "unit": "nnz/s",
            "h2d_bytes_per_step": int(h2d + fbytes + 4 * J ** N), "d2h_bytes_per_step": int(fbytes + 8 * sweeps),
            "step": f"create_blocks from pinned host COO + init + {sweeps} sweeps with fit + factor readback",
            "wall_s": wall,
        }
        del np
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu:
        cpu = cpu_baseline(coo, cfg, args.cpu_sample)
    if dist.rank == 0:
        line = {
            "metric": f"ALS-sweep nnz/s ({args.precision}, FP32 values, 1 GB300)", "value": value, "unit": "nnz/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {k: cfg[k] for k in ("workload", "order", "dims", "zipf_s", "rank", "partition", "dtype")}
            | {"nnz": nnz, "parallelism": f"replicas{dist.world}", "l2": "inputs (8 GB views) exceed the 129 MB L2",
               "generator_s": gen_s},
            "fit_last": fits[-1] if fits else None,
            "fits": [round(f, 6) for f in fits],
            "gpu_launches": launches,
            "kernels": kernels,
            "roofline": roofline,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        print(json.dumps(line), flush=True)
    dist.close()


if __name__ == "__main__":
    main()
