"""Benchmark of the eigensubstitution hot path: Counts columns/s on one GB300.

Workload (default): A=4 HKY85 (kappa=2, pi ~ Dir(1^4)), random binary tree
with 128 leaves (R=255), branch lengths Exp(mean 0.05), C=2^20 columns
simulated down the tree with 10% gaps.  One step = one Counts call (general
eigensubstitution path, Steiner branch mask "auto" = the subby default) over
all 2^20 columns.  The 1.07 GB token matrix is larger than L2 (129 MB), so
no flush is needed between steps.  The F81 fast path is timed on the same
tokens and tree with the F81 model and reported beside it.

Output: one JSON line (rank 0).  ``value`` is device throughput with inputs
resident in HBM; ``e2e`` is the same metric through the public API with host
(pinned) buffers, copies included; ``roofline`` is the Counts kernel against
the measured HBM copy bandwidth, with ``fp32_issue`` (its issue-slot and
FP32 FLOP fractions) beside it; ``cpu_baseline`` is the FP64 oracle port on
the host cores on a bounded sample.  On one GPU the line also carries the
other workloads of the metric, each with its own clock record:

* ``precision64``: A=64 random reversible model with near-degenerate
  eigenvalue pairs, R=127, C=65536 — Counts + LogLike on the split-BF16
  tensor-core walk and on the plain FP32 CUDA-core walk, their ratio, errors
  against the FP64 oracle and each arm's fraction of its own peak;
* ``grad20``: A=20, R=399, C=10^5 — LogLike + adjoint gradient columns/s
  through host buffers;
* ``serving``: 10000 jobs (Poisson 200/s, uneven R, C, A) through the
  continuous-batching server, each job's alignment uploaded from pinned host
  memory and its results read back inside its latency — p50 / p99 latency,
  queue and service percentiles.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank processes its own 2^20 columns (weak
scaling, no data-path collective); the step time is the max over ranks.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Counts columns/s (A=4 HKY85, R=255, C=2^20, FP32, general eigensub path)"
UNIT = "columns/s"


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def _fp32_peak_tflops():
    """Nominal FP32 CUDA-core peak: SMs x 128 FP32 lanes x 2 FLOP x max SM
    clock (no FP32 peak is measured on this machine)."""
    import torch
    nsm = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = 2070.0
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            mhz = float(json.load(f).get("sm_max_mhz", mhz))
    return nsm * 128 * 2 * mhz * 1e6 / 1e12, nsm, mhz


def _profile_entry(kernel):
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f).get(kernel, {})


def fp32_issue_block(cols_per_s, R, A, clocks):
    """Issue-slot and FP32 fractions of the A=4 Counts kernel beside its HBM
    roofline: the kernel is issue-bound, so these are the fractions that
    move.  Warp instructions per column come from the committed ncu summary
    (profiles/traffic.json); FP32 FLOP per column is the algorithmic count
    11 A^2 (R-1) + 4 A^3 (inside / outside products, projections,
    accumulation, back-transform)."""
    peak, nsm, mhz = _fp32_peak_tflops()
    flop_col = 11 * A * A * (R - 1) + 4 * A ** 3
    out = {"flop_per_column": flop_col, "achieved_tflops": flop_col * cols_per_s / 1e12,
           "fp32_peak_tflops": peak, "fp32_frac": flop_col * cols_per_s / 1e12 / peak,
           "fp32_peak_kind": f"nominal: {nsm} SMs x 128 lanes x 2 FLOP x {mhz:.0f} MHz"}
    e = _profile_entry("counts_eigen_a4")
    ipc = e.get("thread_instructions_per_column")
    if ipc:
        clk = (clocks or {}).get("sm_mhz") or mhz
        slots = nsm * 4 * clk * 1e6          # warp-instruction issue slots per second
        out["issue_frac"] = (ipc / 32.0) * cols_per_s / slots
        out["thread_instructions_per_column"] = ipc
        out["issue_source"] = ("ncu smsp__inst_executed.sum of the same kernel (profiles/traffic.json) x "
                               "columns/s / (SMs x 4 schedulers x median SM clock of the timed region)")
    return out


def _traffic_per_column(kernel):
    """DRAM bytes per column of `kernel` from the committed ncu summary, or None."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    if not os.path.exists(p):
        return None
    with open(p) as f:
        d = json.load(f)
    v = d.get(kernel)
    return None if v is None else float(v["bytes_per_column"])


class ClockSampler:
    """nvidia-smi clocks/throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.f, stderr=subprocess.DEVNULL)
            # the sampler's start-up (driver queries) must not fall inside a
            # short timed region: wait for its first sample (at most 2 s)
            t0 = time.perf_counter()
            while (self.proc.poll() is None and os.path.getsize(self.path) == 0
                   and time.perf_counter() - t0 < 2.0):
                time.sleep(0.02)
        except Exception:  # noqa: BLE001
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:  # noqa: BLE001
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU baseline: the FP64 oracle port over column shards (spawned workers)
# ---------------------------------------------------------------------------

def _oracle_counts_shard(args):
    aln, parent, dist, ev, V, pi = args
    import oracle
    t = oracle.Tree(parent, dist)
    oracle.Counts(aln, t, {'eigenvalues': ev, 'eigenvectors': V, 'pi': pi})
    return aln.shape[1]


def cpu_oracle_throughput(aln, tree, model, target_s=12.0, pool=None, cores=None):
    """Columns/s of the oracle on a bounded sample sized to ~target_s of work."""
    cores = cores or (os.cpu_count() or 1)
    ev, V, pi = (np.asarray(x, dtype=np.float64) for x in (model.eigenvalues, model.eigenvectors, model.pi))
    parent, dist = np.asarray(tree.parentIndex), np.asarray(tree.distanceToParent)
    # calibrate on one shard in-process
    cal = 1024
    t0 = time.perf_counter()
    _oracle_counts_shard((aln[:, :cal], parent, dist, ev, V, pi))
    per_col = (time.perf_counter() - t0) / cal
    shard = 2048
    n_shards = max(cores, int(target_s * cores / max(per_col * shard, 1e-9)))
    n_shards = min(n_shards, max(1, aln.shape[1] // shard))
    sample = n_shards * shard
    work = [(np.ascontiguousarray(aln[:, i * shard:(i + 1) * shard]), parent, dist, ev, V, pi)
            for i in range(n_shards)]
    t0 = time.perf_counter()
    if pool is not None and cores > 1:
        done = sum(pool.map(_oracle_counts_shard, work))
    else:
        done = sum(map(_oracle_counts_shard, work))
    dt = time.perf_counter() - t0
    return done / dt, cores, f"{sample} of {aln.shape[1]} columns ({n_shards} shards of {shard}), {dt:.1f} s"


# ---------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200 for this implementation, whose steps take ~3 ms, so that "
                         "the clock sampler sees the timed region; 10 for --impl reference)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--columns", type=int, default=1 << 20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", choices=["plain_large", "precision64", "f81_64", "grad20", "serving",
                                           "posteriors", "irreversible", "gamma4"],
                    default="plain_large",
                    help="plain_large is the headline line; the others print their own line")
    ap.add_argument("--headline-only", action="store_true",
                    help="plain_large: skip the precision64 / grad20 / serving blocks")
    ap.add_argument("--jobs", type=int, default=10000, help="serving: number of jobs")
    ap.add_argument("--rate", type=float, default=200.0, help="serving: Poisson arrival rate (jobs/s)")
    ap.add_argument("--trace", default=None,
                    help="serving: write one JSON line per job (kind, R, C, estimated cost, arrival, start, "
                         "finish) to this file")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    if args.steps is None:
        args.steps = 10 if args.impl == "reference" else (200 if args.workload == "plain_large" else 20)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    from subby_gb300 import synth

    if args.impl == "reference":
        if rank != 0:
            return 0
        return reference_arm(args, world)
    if args.workload == "serving":
        return serving_bench(args)
    if args.workload == "precision64":
        return precision64_bench(args)
    if args.workload == "grad20":
        return grad20_bench(args)
    if args.workload == "f81_64":
        return f81_64_bench(args)
    if args.workload in ("posteriors", "irreversible", "gamma4"):
        return widened_bench(args)

    # spawn pool for the CPU baseline before any GPU work
    pool = None
    cores = os.cpu_count() or 1
    if rank == 0 and not args.no_cpu_baseline and cores > 1:
        pool = mp.get_context("spawn").Pool(cores)

    import torch
    import subby_gb300 as sg
    from subby_gb300 import _lib

    torch.cuda.set_device(local_rank)
    dist_on = world > 1
    if dist_on:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))

    C = args.columns
    w = synth.plain_large(seed=2 + rank, C=C)
    wf = synth.plain_large(seed=2 + rank, C=C, f81=True)
    aln, tree, model = w['alignment'], w['tree'], w['model']
    R, A = aln.shape[0], 4
    plan = sg.Plan(tree, model)
    plan_f81 = sg.Plan(wf['tree'], wf['model'])
    d_aln = torch.as_tensor(aln).cuda()
    d_aln_f = torch.as_tensor(wf['alignment']).cuda()
    out = {'counts': torch.empty((A, A, C), dtype=torch.float32, device="cuda")}
    out_f = {'counts': torch.empty((A, A, C), dtype=torch.float32, device="cuda")}
    stream = torch.cuda.current_stream()

    def step():
        plan.run(d_aln, loglike=False, counts=True, branch_mask="auto", out=out)

    def step_f81():
        plan_f81.run(d_aln_f, loglike=False, counts=True, f81=True, branch_mask="auto", out=out_f)

    def barrier():
        if dist_on:
            torch.distributed.barrier()

    def timed(fn, K):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(K):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1) / K
        if dist_on:
            t = torch.tensor([ms], device="cuda")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    # general path: headline value (clocks sampled during this region)
    with ClockSampler(local_rank) as clk:
        ms = timed(step, args.steps)
    clocks = clk.summary()
    launches_per_step = _lib.last_launch_count()
    ms_f81 = timed(step_f81, args.steps)

    # e2e through the public API with pinned host buffers (copies in the timed region)
    h_aln = torch.empty((R, C), dtype=torch.int32, pin_memory=True)
    h_aln.numpy()[:] = aln
    h_out = torch.empty((A, A, C), dtype=torch.float32, pin_memory=True)
    hbuf = {'counts': h_out.numpy()}
    for _ in range(2):
        plan.run(h_aln.numpy(), loglike=False, counts=True, branch_mask="auto", out=hbuf)
    barrier()
    # the mean over at least 10 calls: single calls run ~6.2 ms with rare
    # ~2x outliers (host scheduling), which a 5-call mean over-weights
    n_e2e = max(10, args.steps)
    t0 = time.perf_counter()
    for _ in range(n_e2e):
        plan.run(h_aln.numpy(), loglike=False, counts=True, branch_mask="auto", out=hbuf)
    e2e_ms = (time.perf_counter() - t0) * 1000 / n_e2e
    if dist_on:
        t = torch.tensor([e2e_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())

    # correctness spot check of this run against the oracle (64 columns)
    import oracle
    md = {'eigenvalues': np.asarray(model.eigenvalues), 'eigenvectors': np.asarray(model.eigenvectors),
          'pi': np.asarray(model.pi)}
    ref = oracle.Counts(aln[:, :64], oracle.Tree(tree.parentIndex, tree.distanceToParent), md)
    got = out['counts'][:, :, :64].cpu().numpy()
    from tests._tol import colwise_err
    err = colwise_err(got, ref)

    if rank != 0:
        if dist_on:
            torch.distributed.destroy_process_group()
        return 0

    blocks = {}
    if world == 1 and not args.headline_only:
        del d_aln, d_aln_f, out, out_f, h_aln, h_out, hbuf
        plan.close()
        plan_f81.close()
        torch.cuda.empty_cache()
        blocks["precision64"] = precision64_block(args)
        blocks["grad20"] = grad20_block(args)
        blocks["serving"] = serving_block(args)

    hbm, _, peak_kind = _peaks()
    b_col = 4 * R + 4 * A * A           # int32 tokens in, FP32 counts out
    achieved = b_col * C / (ms / 1000) / 1e9
    tr = _traffic_per_column("counts_eigen_a4")
    cpu = None
    if not args.no_cpu_baseline:
        v, ncores, sample = cpu_oracle_throughput(aln, tree, model, pool=pool, cores=cores)
        cpu = {"value": v, "unit": UNIT, "cores": ncores, "kind": "port",
               "sample": "FP64 numpy oracle restatement, Counts (mask auto) on " + sample}
    if pool is not None:
        pool.close()
    n = world
    line = {
        "metric": METRIC, "value": n * C / (ms / 1000), "unit": UNIT, "n_gpus": n,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded simulation)",
        "config": {"workload": "plain_large: A=4 HKY85 kappa=2, R=255 (128 leaves), C=2^20 per GPU, "
                               "10% gaps, branch_mask=auto", "columns_per_gpu": C, "R": R, "A": A,
                   "l2": "inputs (1.07 GB tokens) larger than L2, no flush",
                   "parallelism": f"column shards x{n}" if n > 1 else "single GPU"},
        "f81_fast_path": {"value": n * C / (ms_f81 / 1000), "unit": UNIT, "ms_per_step": ms_f81},
        "e2e": {"value": n * C / (e2e_ms / 1000), "unit": UNIT, "ms_per_step": e2e_ms, "calls": n_e2e,
                "h2d_bytes_per_step": R * C * 4, "d2h_bytes_per_step": A * A * C * 4},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "peak_kind": peak_kind,
                     "traffic": None if tr is None else tr * C,
                     "algorithmic_bytes_per_column": b_col},
        "fp32_issue": fp32_issue_block(C / (ms / 1000), R, A, clocks),
        "cpu_baseline": cpu,
        "clocks": clocks,
        "gpu_launches": launches_per_step * args.steps,
        "max_colwise_err_vs_oracle_64cols": err,
    }
    line.update(blocks)
    print(json.dumps(line))
    if dist_on:
        torch.distributed.destroy_process_group()
    return 0


def _time_fn(fn, steps, warmup):
    import torch
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / steps


def precision64_block(args):
    """A=64 random reversible model with near-degenerate eigenvalue pairs,
    R=127, C=65536 (inputs resident, CUDA events): Counts + LogLike on the
    split-BF16 tensor-core walk and on the plain FP32 CUDA-core walk, errors
    against the FP64 oracle on 64 seeded columns, each arm's fraction of its
    own peak."""
    import torch
    import oracle
    import subby_gb300 as sg
    from subby_gb300 import synth, _lib
    from tests._tol import colwise_err, loglike_err
    C = args.columns if args.columns != (1 << 20) else 65536
    w = synth.precision64(seed=3, C=C)
    R = len(w['tree'].parentIndex)
    A = 64
    plan = sg.Plan(w['tree'], w['model'])
    d_aln = torch.as_tensor(w['alignment']).cuda()
    idx = np.sort(np.random.default_rng(64).choice(C, 64, replace=False))
    sub = np.ascontiguousarray(w['alignment'][:, idx])
    md = w['model']._asdict()
    t = oracle.Tree(w['tree'].parentIndex, w['tree'].distanceToParent)
    ref_c = oracle.Counts(sub, t, md, branch_mask=None)
    ref_l = oracle.LogLike(sub, t, md)
    lib = _lib.load()
    _, bf16, peak_kind = _peaks()
    fp32_peak, _, _ = _fp32_peak_tflops()
    # FLOP per column (FMA = 2): tensor-core-eligible products of the walk,
    # 8 A^2 per branch (inside M, outside M^T, Vd and Vu projections), and
    # the back-transform 4 A^3; the whole step adds the J-weighted
    # accumulation, 3 A^2 per branch, on CUDA cores
    tc_flop = 8 * A * A * (R - 1) + 4 * A ** 3
    all_flop = 11 * A * A * (R - 1) + 4 * A ** 3
    ii = torch.as_tensor(idx).cuda()
    res = {}
    steps = max(3, args.steps)
    for name, sel in (("split_bf16_tensor_core", 0), ("fp32_cuda_core", 2)):
        lib.subby_debug_set_kernel(sel)
        try:
            out = {'counts': torch.empty((A, A, C), dtype=torch.float32, device="cuda"),
                   'logLike': torch.empty(C, dtype=torch.float32, device="cuda")}
            with ClockSampler(torch.cuda.current_device()) as clk:
                ms = _time_fn(lambda: plan.run(d_aln, loglike=True, counts=True, branch_mask=None, out=out),
                              steps, args.warmup)
            launches = _lib.last_launch_count()
            ll = {'logLike': out['logLike']}
            ms_ll = _time_fn(lambda: plan.run(d_aln, loglike=True, out=ll), steps, args.warmup)
            plan.status()
            r = {"columns_per_s": C / (ms / 1e3), "ms_per_step": ms, "gpu_launches_per_step": launches,
                 "loglike_only_columns_per_s": C / (ms_ll / 1e3),
                 "err_vs_oracle": {"loglike_rel": loglike_err(out['logLike'][ii].cpu().numpy(), ref_l),
                                   "counts_colwise": colwise_err(out['counts'][:, :, ii].cpu().numpy(), ref_c),
                                   "columns": len(idx), "branch_mask": None},
                 "clocks": clk.summary()}
        finally:
            lib.subby_debug_set_kernel(0)
        if sel == 0:
            ach = tc_flop * r["columns_per_s"] / 1e12
            r["peak"] = {"unit": "TFLOP/s", "flop_per_column": tc_flop, "achieved": ach, "peak": bf16,
                         "peak_kind": f"{peak_kind} bf16 burst", "frac": ach / bf16,
                         "frac_of_split_bf16_ceiling": 6 * ach / bf16,
                         "note": "useful tensor-core-eligible FLOP over the whole Counts step; split-BF16 "
                                 "issues 6 BF16 MMAs per product, so its ceiling is 1/6 of the BF16 peak"}
        else:
            ach = all_flop * r["columns_per_s"] / 1e12
            r["peak"] = {"unit": "TFLOP/s", "flop_per_column": all_flop, "achieved": ach, "peak": fp32_peak,
                         "peak_kind": "nominal FP32 CUDA-core peak", "frac": ach / fp32_peak}
        res[name] = r
        del out, ll
    plan.close()
    tc, fp = res["split_bf16_tensor_core"], res["fp32_cuda_core"]
    return {"workload": "precision64: A=64 random reversible (exchangeabilities LogNormal(0,1), "
                        "pi ~ Dir(1^64), ~5% of eigenvalue pairs within 1e-7), R=127 (64 leaves), "
                        f"C={C} simulated columns, Counts (unmasked) + LogLike",
            "unit": UNIT, "steps": steps, "warmup": args.warmup,
            "forced_near_degenerate_pairs": w['forced_pairs'],
            "tensor_core_vs_fp32_speedup": tc["columns_per_s"] / fp["columns_per_s"],
            "loglike_tensor_core_vs_fp32_speedup": tc["loglike_only_columns_per_s"] / fp["loglike_only_columns_per_s"],
            "precision": {"propagation": "split-BF16 (3 terms, 6 products, FP32 accumulation in TMEM) on the "
                                         "tensor-core arm; FP32 on the CUDA-core arm",
                          "J(t)": "FP64 for near-degenerate pairs (|dmu| t < 1e-3), FP32 expm1 form otherwise",
                          "back_transform": "FP32 (tensor-core arm: split-BF16 products) — the reference "
                                            "keeps FP64; the measured Counts error above is its effect"},
            "variants": res}


def precision64_bench(args):
    """Prints the precision64 block as its own line."""
    b = precision64_block(args)
    C = args.columns if args.columns != (1 << 20) else 65536
    b.update({"metric": f"Counts columns/s (A=64 reversible, R=127, C={C})",
              "value": b["variants"]["split_bf16_tensor_core"]["columns_per_s"], "higher_is_better": True,
              "dtype": "fp32 (split-bf16 tensor-core products)"})
    print(json.dumps(b))
    return 0


def f81_64_bench(args):
    """A=64 F81 model (pi ~ Dirichlet(1^64)), the precision64 tree (R=127),
    C=65536 simulated columns: F81 fast-path Counts (closed-form walk and
    tensor-core accumulation) and eigen-path Counts of the same model."""
    import torch
    import oracle
    import subby_gb300 as sg
    from subby_gb300 import synth, models
    from tests._tol import colwise_err
    C = args.columns if args.columns != (1 << 20) else 65536
    rng = np.random.default_rng(11)
    model = models.f81_model(rng.dirichlet(np.ones(64)))
    tree = synth.random_tree(64, 0.1, rng)
    aln = synth.simulated_alignment(tree, model, C, 0.05, rng)
    plan = sg.Plan(tree, model)
    d_aln = torch.as_tensor(aln).cuda()
    out = {'counts': torch.empty((64, 64, C), dtype=torch.float32, device="cuda")}
    ms_f81 = _time_fn(lambda: plan.run(d_aln, loglike=False, counts=True, f81=True, out=out), args.steps, args.warmup)
    t = oracle.Tree(tree.parentIndex, tree.distanceToParent)
    err = colwise_err(out['counts'][:, :, :16].cpu().numpy(),
                      oracle.Counts(aln[:, :16], t, model._asdict(), f81_fast=True))
    ms_eig = _time_fn(lambda: plan.run(d_aln, loglike=False, counts=True, out=out), args.steps, args.warmup)
    print(json.dumps({"metric": "F81 fast-path Counts columns/s (A=64 F81, R=127, C=65536)", "value": C / (ms_f81 / 1e3),
                      "unit": UNIT, "ms_per_step": ms_f81, "steps": args.steps, "warmup": args.warmup,
                      "higher_is_better": True, "dtype": "fp32 (split-bf16 tensor-core G accumulation)",
                      "err_vs_oracle_colwise_16cols": err,
                      "eigen_path_same_model": {"value": C / (ms_eig / 1e3), "ms_per_step": ms_eig}}))
    return 0


def widened_bench(args):
    """Device throughput of the rows beyond Counts (inputs resident, CUDA
    events): InsideOutside posteriors (A=4 plain_large tree, node and branch;
    A=64 precision64 tree), irreversible-model Counts (cyclic random rate
    matrices, A=4 / 20 / 64), and a 4-category discrete-gamma *H batch plus
    MixturePosterior (A=4).  One JSON line, one entry per case."""
    import torch
    import subby_gb300 as sg
    from subby_gb300 import synth, models
    rng = np.random.default_rng(7)
    res = {}

    def case(name, C, fn):
        ms = _time_fn(fn, args.steps, args.warmup)
        res[name] = {"ms_per_step": round(ms, 3), "columns_per_s": C / (ms / 1e3)}

    if args.workload == "posteriors":
        w = synth.plain_large(seed=2, C=1 << 20)
        plan = sg.Plan(w['tree'], w['model'])
        d = torch.as_tensor(w['alignment']).cuda()
        case("node_posteriors A=4 R=255 C=2^20", 1 << 20, lambda: plan.posteriors(d))
        case("branch_posteriors A=4 R=255 C=2^20", 1 << 20,
             lambda: plan.posteriors(d, want_node=False, want_branch=True))
        w = synth.precision64(seed=3, C=65536)
        plan = sg.Plan(w['tree'], w['model'])
        d = torch.as_tensor(w['alignment']).cuda()
        case("node_posteriors A=64 R=127 C=65536", 65536, lambda: plan.posteriors(d))
        case("branch_posteriors A=64 R=127 C=4096", 4096,
             lambda: plan.posteriors(d[:, :4096].contiguous(), want_node=False, want_branch=True))
    elif args.workload == "irreversible":
        for A, leaves, C in ((4, 128, 1 << 20), (20, 200, 100000), (64, 64, 65536)):
            m = models.random_irreversible(A, rng)
            tree = synth.random_tree(leaves, 0.05 if A == 4 else 0.1, rng)
            aln = synth.simulated_alignment(tree, m, C, 0.1, rng) if A == 4 else \
                rng.integers(0, A + 2, size=(len(tree.parentIndex), C)).astype(np.int32)
            plan = sg.Plan(tree, m)
            d = torch.as_tensor(aln).cuda()
            case(f"irreversible Counts A={A} R={plan.R} C={C}", C, lambda: plan.run(d, loglike=False, counts=True))
            case(f"irreversible LogLike A={A} R={plan.R} C={C}", C, lambda: plan.run(d, loglike=True))
    else:
        w = synth.plain_large(seed=2, C=1 << 20)
        d = torch.as_tensor(w['alignment']).cuda()
        rates, weights = models.gamma_rate_categories(0.5, 4)
        mb = models.scale_model(w['model'], rates)
        case("LogLike, 4 gamma categories (*H batch), A=4 R=255 C=2^20", 1 << 20,
             lambda: sg.LogLike(d, w['tree'], mb))
        ms = [models.scale_model(w['model'], r) for r in rates]
        case("MixturePosterior over 4 gamma categories, A=4 R=255 C=2^20", 1 << 20,
             lambda: sg.MixturePosterior(d, w['tree'], ms, np.log(weights)))
    print(json.dumps({"workload": args.workload, "steps": args.steps, "warmup": args.warmup,
                      "data": "synthetic, inputs resident on the device", "cases": res}))
    return 0


def grad20_block(args):
    """A=20 reversible model, R=399, C=100000: forward + adjoint gradient
    (d sum logL / d branch lengths and / d log-exchangeabilities) through
    host buffers (each step uploads the alignment and reads the gradients)."""
    import torch
    import subby_gb300 as sg
    from subby_gb300 import synth, autograd
    C = 100000
    w = synth.grad20(seed=4, C=C)
    plan = sg.Plan(w['tree'], w['model'])
    aln = w['alignment']
    for _ in range(args.warmup):
        plan.grad(aln)
    steps = max(3, args.steps)
    with ClockSampler(torch.cuda.current_device()) as clk:
        t0 = time.perf_counter()
        for _ in range(steps):
            _, dldt, G = plan.grad(aln)
        ms = (time.perf_counter() - t0) * 1e3 / steps
    dle = autograd.exchangeability_grad(G, w['log_exch'], w['pi'])
    dev_bytes = plan.device_bytes()
    plan.close()
    return {"workload": "grad20: A=20 reversible (exchangeabilities LogNormal(0,0.5), pi ~ Dir(2^20)), R=399 "
                        "(200 leaves), C=100000 simulated columns, 15% gaps",
            "value": C / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": steps,
            "what": "LogLike + d/d(branch lengths) + d/dS~ per step, host buffers (1.6e8 B in), synchronous",
            "h2d_bytes_per_step": aln.nbytes, "plan_device_bytes": dev_bytes,
            "grad_norms": {"d_dt": float(np.linalg.norm(dldt)), "d_dlogs": float(np.linalg.norm(dle))},
            "clocks": clk.summary()}


def grad20_bench(args):
    b = grad20_block(args)
    b["metric"] = "LogLike + adjoint gradient columns/s (A=20, R=399, C=100000, host buffers)"
    b["higher_is_better"] = True
    print(json.dumps(b))
    return 0


def serving_block(args):
    """Poisson job stream (uneven R, C, A) through the continuous-batching
    server.  Each job's alignment is a window of a pinned host buffer that
    the server uploads on the job's stream (the SMs gather it over the host
    link), and its results are copied back to pinned host memory: per-job
    latency runs from arrival to results in host memory and includes both."""
    # keep freed plan memory cached in the library pool between jobs
    os.environ.setdefault("SUBBY_POOL_KEEP_MB", str(32 << 10))
    import torch
    from subby_gb300 import synth, serve, models
    desc = synth.serving_jobs(n_jobs=args.jobs, rate=args.rate, seed=5)
    # warm-up stream (other seed, not timed): loads every kernel once and
    # grows the slot arenas and host/device pools to their working sizes
    wdesc = synth.serving_jobs(n_jobs=max(100, 50 * args.warmup), rate=args.rate, seed=6)
    # token pools in pinned host memory, one per alphabet: rows of leaf
    # states uniform with 5% gaps (A+1) and a last row of A (unobserved) for
    # the internal nodes; a job reads its leaves' rows and that row over a
    # window of columns
    POOL_C = max(d['C'] for d in desc + wdesc)
    max_leaves = max(d['leaves'] for d in desc + wdesc)
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    pools = {}
    for A_ in sorted({d['A'] for d in desc + wdesc}):
        v = torch.randint(0, 20 * A_, (max_leaves + 1, POOL_C), dtype=torch.int32, device="cuda", generator=g)
        v = torch.where(v < 19 * A_, v % A_, A_ + 1)
        v[max_leaves].fill_(A_)
        h = torch.empty((max_leaves + 1, POOL_C), dtype=torch.int32, pin_memory=True)
        h.copy_(v)
        pools[A_] = h
        del v
    torch.cuda.synchronize()

    def build(descs):
        out = []
        for d in descs:
            rng = np.random.default_rng(d['seed'])
            A = d['A']
            if d['kind'] == 'hky85':
                model = models.hky85_diag(2.0, rng.dirichlet(np.ones(4)))
            elif d['kind'] == 'f81':
                model = models.f81_model(rng.dirichlet(np.ones(A)))
            else:
                model, _, _ = models.random_reversible(A, rng)
            tree = synth.random_tree(d['leaves'], 0.1, rng)
            R, C = len(tree.parentIndex), d['C']
            leaf = synth.leaf_mask(tree)
            # pool row of every tree row: leaves take distinct rows, internal
            # rows the pool's row of A (unobserved)
            rowmap = np.full(R, max_leaves, dtype=np.int32)
            rowmap[leaf] = np.arange(int(leaf.sum()), dtype=np.int32)
            off = int(np.random.default_rng(d['seed']).integers(0, POOL_C - C + 1))
            aln = serve.HostRows(base=pools[A], col0=off, rowmap=rowmap, R=R, C=C)
            out.append(serve.Job(id=d['id'], alignment=aln, tree=tree, model=model,
                                 f81=(d['kind'] == 'f81'), want=("counts",), arrival=d['arrival']))
        return out

    jobs, warm = build(desc), build(wdesc)
    # work-item shape of the packed A = 4 kernel, tuned on this device
    fd, tune_path = tempfile.mkstemp(suffix=".json")
    os.close(fd)
    t_tune = time.perf_counter()
    tuned = serve.autotune_packed(cache=tune_path)
    t_tune = time.perf_counter() - t_tune
    with open(tune_path) as f:
        tune_record = json.load(f)
    # the library's engine (C++ thread): Python only submits and collects
    srv = serve.NativeServer(max_inflight=8, device_budget=64 << 30, pinned_prewarm=4 << 30,
                             autotune_cache=tune_path)
    os.unlink(tune_path)
    # the consumer takes each result as it lands and hands its buffers back
    srv.run(warm, realtime=False, on_done=lambda j: j.release())
    eng0 = srv.stats()
    with ClockSampler(torch.cuda.current_device()) as clk:
        t_run = time.perf_counter()
        done = srv.run(jobs, realtime=True, on_done=lambda j: j.release())
        t_run = time.perf_counter() - t_run
    engine = srv.stats()
    for k in ("engine_busy_s", "packed_jobs", "packed_launches"):
        engine[k] -= eng0[k]
    st = serve.latency_stats(done)
    kind_of = {d['id']: f"A={d['A']} {d['kind']}" for d in desc}
    by_kind = {}
    for k in sorted(set(kind_of.values())):
        sub = [j for j in done if kind_of[j.id] == k]
        if sub:
            s2 = serve.latency_stats(sub)
            by_kind[k] = {"jobs": s2['jobs'], "p50_ms": s2['p50_ms'], "p99_ms": s2['p99_ms'],
                          "queue_p99_ms": s2['queue_p99_ms'], "service_p99_ms": s2['service_p99_ms'],
                          "columns": s2['columns']}
    if getattr(args, "trace", None):
        dmap = {d['id']: d for d in desc}
        with open(args.trace, "w") as f:
            for j in done:
                d = dmap[j.id]
                R, C = j.RC
                f.write(json.dumps({"id": j.id, "A": d['A'], "kind": d['kind'], "R": R, "C": C,
                                    "cost_ms": serve.job_cost_ms(R, C, d['A'], d['kind'] == 'f81'),
                                    "arrival": j.arrival, "start": j.start, "finish": j.finish}) + "\n")
    failed = sum(1 for j in done if j.error)
    h2d = sum(j.alignment.nbytes for j in done)
    d2h = sum(4 * j.RC[1] * len(j.model.pi) ** 2 for j in done)
    srv.close()
    return {"workload": f"{st['jobs']} jobs, Poisson arrivals at {args.rate:g}/s; leaves log-uniform 8..512, "
                        "C log-uniform 100..2e5, A in {4 HKY85, 16 random reversible, 64 F81 or random "
                        "reversible}; Counts (mask auto) per job",
            "value": st['p99_ms'], "unit": "ms (p99)", "higher_is_better": False,
            "p50_ms": st['p50_ms'], "p99_ms": st['p99_ms'], "max_ms": st['max_ms'], "jobs": st['jobs'],
            "failed_jobs": failed,
            "queue_p50_ms": st['queue_p50_ms'], "queue_p99_ms": st['queue_p99_ms'],
            "service_p50_ms": st['service_p50_ms'], "service_p99_ms": st['service_p99_ms'],
            "columns_per_s": st['columns_per_s'], "span_s": st['span_s'], "rate_jobs_per_s": args.rate,
            "h2d_bytes": h2d, "d2h_bytes": d2h, "by_kind": by_kind,
            "autotune": {"settings": tuned, "wall_ms": tune_record.get("wall_ms"), "seconds": round(t_tune, 2)},
            "host": {"engine_busy_s": round(engine["engine_busy_s"], 3), "wall_s": round(t_run, 3),
                     "plans_cached": engine["plans_cached"], "packed_jobs": engine["packed_jobs"],
                     "packed_launches": engine["packed_launches"],
                     "engine": "library serving engine (subby_server_*, one C++ thread); Python submits "
                               "each job at its arrival time and collects results"},
            "latency": "arrival -> counts in pinned host memory; includes the upload of the job's alignment "
                       "from pinned host memory and the result copy",
            "data": "synthetic: per-job random tree and model; leaf tokens uniform with 5% gaps from a pinned "
                    "host pool, internal rows unobserved",
            "clocks": clk.summary()}


def serving_bench(args):
    b = serving_block(args)
    b["metric"] = "serving latency (Poisson arrivals, uneven R/C/A)"
    print(json.dumps(b))
    return 0


def reference_arm(args, world):
    """The reference's CPU algorithm (FP64 oracle port: the reference itself is
    Python and does not travel) on the host cores, same workload and metric."""
    from subby_gb300 import synth
    C = args.columns
    w = synth.plain_large(seed=2, C=C)
    cores = os.cpu_count() or 1
    pool = mp.get_context("spawn").Pool(cores) if cores > 1 else None
    vals = []
    sample = ""
    for i in range(args.warmup + args.steps):
        v, ncores, sample = cpu_oracle_throughput(w['alignment'], w['tree'], w['model'],
                                                  target_s=4.0, pool=pool, cores=cores)
        if i >= args.warmup:
            vals.append(v)
    if pool is not None:
        pool.close()
    v = float(statistics.median(vals))
    line = {
        "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": C / v * 1000, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded simulation)",
        "config": {"workload": "plain_large: A=4 HKY85 kappa=2, R=255 (128 leaves), C=2^20, "
                               "10% gaps, branch_mask=auto", "columns_per_gpu": C},
        "impl": "reference",
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": "per step: " + sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


if __name__ == "__main__":
    sys.exit(main())
