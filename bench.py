"""Benchmark of the DynLP per-batch update path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (default): the reference's default run — n = 50,000 vertices,
average degree 5, 10 batches, delta 1e-4, maxIter 1e5, tau = mean edge weight,
seed 42 — generated with the reference generator's exact decisions
(synthetic; the reference ships no dataset). One step = one replay of the 10
batches from an empty graph on the plain per-batch path, in the reference's
semantics. Unit of work: one affected edge, i.e. one (frontier vertex, live
row entry) visit in propagation, summed over passes and batches — the count is
fixed by the workload (the oracle produces the same count).

GPU arm: `value` times the batch kernels with the batches already resident in
HBM (CUDA events on the session stream, L2 flushed by a 512 MiB memset before
each step); `e2e` replays through the C ABI from host arrays (pinned staging,
H2D, one kernel per batch, D2H of every batch's statistics and of the final
labels), wall clock with the stream synchronised on both sides.
Reference arm (--impl reference): the reference's path is CUDA only, so its
CPU counterpart is the oracle's restatement of it (oracle/, a port), run with
all host threads on the same workload.

Served vs plain (the `served` object of the same line; --no-served skips it):
the multi-instance configuration, 512 resident graphs (n log-uniform on
[1e3, 5e5], degree {3,5,7}, generator seed i, 10 batches each: 5,120
requests). `batched` runs one engine launch per batch index over all graphs;
`served_saturated` replays every request through the continuous-batching
server with all of them queued at t = 0; `served_poisson_sweep` replays a
size-stratified subset with Poisson arrivals at fractions of its saturated
request rate (latency = finish - arrival); `plain` is the server in serial
mode (one request at a time, run to its end — the plain per-batch path) on a
stratified sample of whole graphs, scaled to the whole trace. All count the
same affected edges per request; the served paths include the host-to-device
copy of every request. --gpus N (without WORLD_SIZE set) starts N ranks; the
graphs are then split across them with no collective on the data path.

Also on the line: the FP64 oracle's error on the headline workload, and the
reference's own CUDA build (oracle/_ref/ref_kernels, built from a guarded copy
of its sources when that copy is present) timed on the same GPU.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "affected-edges/sec and p50/p99 batch-update latency, served vs plain, same GPU"
UNIT = "affected-edges/s"
WORKLOADS = {
    "config2": dict(n=50000, degree=5, batches=10, seed=42),
    "config1": dict(n=5000, degree=5, batches=10, seed=42),
    "config3": dict(n=20000000, degree=7, batches=100, seed=42),
    # a state of about 0.5 GB, beyond the 129 MB L2: the profiling shape of
    # the full-grid passes (the same generator at a tenth of config3)
    "large2m": dict(n=2000000, degree=7, batches=100, seed=42),
}


def workload_desc(name: str, limit: int = 0) -> str:
    w = WORKLOADS[name]
    nb = f"first {limit} of {w['batches']}" if 0 < limit < w["batches"] else str(w["batches"])
    return (f"{name}: plain per-batch replay, n={w['n']}, avg degree {w['degree']}, {nb} batches "
            f"(90/1/9 insert/GT/delete), delta 1e-4, maxIter 1e5, tau = mean edge weight, seed {w['seed']}")


# ------------------------------------------------------------------ helpers --

def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def dist_init(world: int):
    if world <= 1:
        return None
    import torch.distributed as td
    os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
    td.init_process_group("gloo")
    return td


def dist_max(td, x: float) -> float:
    if td is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def dist_sum(td, x: float) -> float:
    if td is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    td.all_reduce(t, op=td.ReduceOp.SUM)
    return float(t.item())


def dist_barrier(td):
    if td is not None:
        td.barrier()


class ClockSampler:
    """nvidia-smi clock / throttle-reason samples during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, val in zip(names, f[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_gbs() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def algorithmic_bytes(st: dict, num_edges: int, num_inserted: int) -> int:
    """Bytes one batch kernel must move at minimum (see the roofline notes):
    propagation 12 B per affected edge (entry 8 + neighbour label 4) and 20 B
    per frontier visit (row start/length 8, own old label 4, new label 4,
    stamp 4); live-row rebuild 16 B per full-graph entry read (read 8, write
    8); tau filter 28 B per raw edge (src/dst/weight 12, two position lookups
    8, two position writes 8); label init 16 B per inserted vertex."""
    return (12 * st["affected_edges"] + 20 * st["frontier_visits"] + 16 * st["dirty_entries"]
            + 28 * num_edges + 16 * num_inserted)


def mode_delta(before: dict, after: dict, steps: int) -> dict:
    """Propagation passes and device time per pass mode between two
    readings, per step, with the time per pass."""
    out = {}
    for m, a in after.items():
        p = a["passes"] - before[m]["passes"]
        t = a["seconds"] - before[m]["seconds"]
        if m == "team":  # a subset of the one-block passes; its time is counted there
            out[m] = {"passes": p / max(steps, 1), "ms": "in one_block"}
            continue
        out[m] = {"passes": p / max(steps, 1), "ms": 1e3 * t / max(steps, 1),
                  "us_per_pass": 1e6 * t / p if p else None}
    return out


def percentile(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = (len(xs) - 1) * q
    lo = int(k)
    hi = min(lo + 1, len(xs) - 1)
    return xs[lo] + (xs[hi] - xs[lo]) * (k - lo)


# -------------------------------------------------------------- CPU (oracle) --

def host_cpu() -> dict:
    """CPU model and core count of this host (the CPU baselines' hardware)."""
    model = None
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            k, _, v = ln.partition(":")
            if k.strip() in ("model name", "Model"):
                model = v.strip()
                break
    except OSError:
        pass
    if model is None:
        try:
            out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
            for ln in out.splitlines():
                if ln.startswith("Model name:"):
                    model = ln.split(":", 1)[1].strip()
                    break
        except (OSError, subprocess.SubprocessError):
            pass
    return {"model": model or "unknown", "nproc": os.cpu_count() or 1}


def oracle_problem(w: dict, batches: int = 0):
    """The workload's inputs from the oracle's own generator (no product code)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    p = pyoracle.OracleProblem(w["n"], w["degree"], w["batches"], w["seed"])
    if batches > 0:
        p.batches = p.batches[:batches]
    return p


def cpu_run(problem, threads: int, budget_s: float):
    """Oracle replay in batch order until the budget is used; returns
    (affected edges, seconds, batches done)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    orc = pyoracle.OracleRun.from_problem(problem, threads=threads)
    edges, t0, done = 0, time.perf_counter(), 0
    for b, bt in enumerate(problem.batches):
        edges += orc.apply(b, bt)["affected_edges"]
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    return edges, time.perf_counter() - t0, done


def fp64_error(problem, gpu_labels, threads: int) -> dict:
    """The FP32 path against the FP64 oracle on the same workload: the
    oracle's fp32 run (which the GPU's final labels must equal bit for bit)
    with each batch's propagation repeated in double from the same state."""
    import numpy as np
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    run = pyoracle.OracleRun.from_problem(problem, threads=threads, fp64=2)
    per = []
    for b, bt in enumerate(problem.batches):
        st = run.apply(b, bt)
        l32, l64 = run.labels().astype(np.float64), run.labels64()
        err = np.abs(l32 - l64)
        per.append({"batch": b, "max_abs": float(err.max()), "p999_abs": float(np.percentile(err, 99.9)),
                    "prediction_flips": int(np.sum((l32 >= 0.5) != (l64 >= 0.5))),
                    "fp32_passes": st["iterations"], "fp64_passes": run.shadow_iterations()})
    return {"max_abs": max(r["max_abs"] for r in per), "prediction_flips_max": max(r["prediction_flips"] for r in per),
            "gpu_labels_equal_oracle_fp32": bool(np.array_equal(gpu_labels, run.labels())),
            "per_batch": per,
            "how": "oracle fp32 schedule vs the same batch's propagation in double from the same state"}


def irlp_block(p, batch_ms: list, threads: int, budget_s: float, device: int) -> dict:
    """IrLP full recompute after every batch of the workload, on the snapshot
    the reference's driver builds for it (src/main.cu:127-176): on the GPU
    (dlp_irlp, one cooperative launch per snapshot, the whole run) and on the
    host cores (the oracle's restatement of src/validation.cu:47-139, all
    threads; per snapshot a bounded number of iterations, scaled to the GPU's
    iteration count when the budget does not cover the whole run), beside the
    incremental path's per-batch device time."""
    import numpy as np
    import labelpropcuda_gb300 as dlp
    sys.path.insert(0, str(ROOT / "oracle"))
    import pyoracle
    snaps = [dlp.irlp_snapshot(p, b) for b in range(len(p.batches))]
    dlp.irlp(snaps[-1], max_iterations=10, device=device)  # first launch: module load
    rows, per_snap_s = [], budget_s / max(1, len(snaps))
    for b, snap in enumerate(snaps):
        t = {}
        lab, it = dlp.irlp(snap, device=device, timing=t)
        visits = it * int(np.diff(snap.row_ptr)[snap.status == 0].sum())
        # CPU: a probe of a few iterations sets how many fit this snapshot's share
        t0 = time.perf_counter()
        _, k0, _ = pyoracle.irlp(snap.num_nodes, snap.row_ptr, snap.col_ind, snap.values, snap.status,
                                 snap.gt_class, snap.labels, max_iterations=min(it, 5) or 1, threads=threads)
        per_it = (time.perf_counter() - t0) / max(k0, 1)
        k = max(1, min(it, int(per_snap_s / max(per_it, 1e-9))))
        t0 = time.perf_counter()
        cl, kc, _ = pyoracle.irlp(snap.num_nodes, snap.row_ptr, snap.col_ind, snap.values, snap.status,
                                     snap.gt_class, snap.labels, max_iterations=k, threads=threads)
        cpu_s = time.perf_counter() - t0
        whole = kc >= it
        rows.append({"batch": b, "iterations": it, "edge_visits": visits, "gpu_ms": t["ms"],
                     "cpu_ms": 1e3 * (cpu_s if whole else cpu_s / max(kc, 1) * it),
                     "cpu_iterations_timed": kc, "cpu_estimated": not whole,
                     "labels_equal_cpu": bool(np.array_equal(cl, lab)) if whole else None,
                     "incremental_ms": batch_ms[b]})
    gpu_ms = sum(r["gpu_ms"] for r in rows)
    inc_ms = sum(batch_ms)
    return {"snapshot": "the IrLP input src/main.cu:127-176 builds, after each batch",
            "gpu_ms_all_batches": gpu_ms, "cpu_ms_all_batches": sum(r["cpu_ms"] for r in rows),
            "incremental_ms_all_batches": inc_ms,
            "gpu_irlp_over_incremental": gpu_ms / inc_ms if inc_ms > 0 else None,
            "gpu_edge_visits_per_s": sum(r["edge_visits"] for r in rows) / (gpu_ms / 1e3) if gpu_ms > 0 else None,
            "cpu_threads": threads, "cpu_kind": "oracle port",
            "timing": "GPU: wall time of one dlp_irlp launch, device synchronised on both sides, inputs resident; "
                      "CPU: wall time", "per_batch": rows}


def reference_cuda(w: dict, batches: int, our_stats: list) -> dict | None:
    """The reference's own CUDA build (its runDynLP, launchers and kernels,
    -O3 --use_fast_math, from the guarded source copy) timed on this GPU on
    the same workload; None when oracle/_ref/ref_kernels is absent."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import tempfile
    import pyoracle
    if not pyoracle.REF_KERNELS.exists():
        return None
    nb = batches or w["batches"]
    with tempfile.TemporaryDirectory() as td:
        t0 = time.perf_counter()
        r = pyoracle.run_ref_kernels(w["n"], w["degree"], nb, w["seed"], 100000, Path(td) / "ref.bin",
                                     record=False)
        wall = time.perf_counter() - t0
    ms = [float(x) for x in r["batch_ms"]]
    its = [b["iterations"] for b in r["batches"]]
    same = its == [s["iterations"] for s in our_stats]
    out = {"batch_ms": ms, "ms_per_replay": sum(ms), "batch_ms_p50": percentile(ms, 0.5),
           "batch_ms_p99": percentile(ms, 0.99), "iterations": its, "iterations_match": same,
           "process_wall_s": wall,
           "timing": "the reference's own per-batch CUDA events (src/dynLP.cu:285,547-552: host CSR rebuild, "
                     "uploads, kernels, label read-back and host accuracy), sm_103a build of its sources"}
    if same:
        out["value"] = sum(s["affected_edges"] for s in our_stats) / (sum(ms) / 1e3)
        out["unit"] = UNIT + " (affected edges counted by the oracle: identical pass counts)"
    return out


def reference_arm(args, td, rank):
    """The reference has no CPU implementation of its path (it is CUDA only),
    so this arm times the oracle's restatement of it on every host thread, on
    inputs from the oracle's own generator: nothing of the product is loaded."""
    if rank != 0:
        return 0
    w = WORKLOADS[args.workload]
    p = oracle_problem(w, args.batches)
    cpu = host_cpu()
    threads = cpu["nproc"]
    for _ in range(args.warmup):
        cpu_run(p, threads, args.ref_budget_s)
    tot_e, tot_t, per = 0, 0.0, []
    batches_done = 0
    for _ in range(args.steps):
        e, t, done = cpu_run(p, threads, args.ref_budget_s)
        tot_e += e
        tot_t += t
        per.append(t)
        batches_done = done
    value = tot_e / tot_t if tot_t > 0 else 0.0
    sample = (f"oracle port (CPU restatement of the reference's per-batch path), {threads} threads on "
              f"{cpu['model']} ({cpu['nproc']} cores), first {batches_done} of {w['batches']} batches per step "
              f"(budget {args.ref_budget_s:.0f} s)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / max(args.steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
            "data": "synthetic (reference generator decisions, seed 42)",
            "config": {"workload": workload_desc(args.workload, args.batches), "semantics": "ref"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample,
                             "cpu_model": cpu["model"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------- GPU arm -----

def gpu_arm(args, td, rank, world, local_rank):
    import labelpropcuda_gb300 as dlp
    from labelpropcuda_gb300 import DeviceArray, DeviceBatch
    L = dlp._n.lib()
    dlp._n.check(L.dlp_set_device(local_rank))
    w = WORKLOADS[args.workload]
    p = dlp.Problem(w["n"], w["degree"], w["batches"], w["seed"])
    if args.batches > 0:  # bounded sample: the first --batches batches of the workload
        p.batches = p.batches[:args.batches]
    nb = len(p.batches)
    sess = dlp.Session.from_problem(p, device=local_rank, narrow_lanes=args.lanes, blocks_per_sm=args.blocks_per_sm)
    dev_batches = [DeviceBatch(bt) for bt in p.batches]
    flush = DeviceArray(nbytes=512 << 20)

    def flush_l2():
        dlp._n.check(L.dlp_memset(flush.ptr, 1, flush.nbytes))
        dlp._n.check(L.dlp_device_synchronize())

    def device_step():
        sess.reset()
        flush_l2()
        for b in range(nb):
            sess.apply_device(b, dev_batches[b])
        try:
            sess.synchronize()
        except dlp.DlpError:
            print("device diagnostics:", sess.debug(), file=sys.stderr, flush=True)
            raise
        stats = [sess.stats(b) for b in range(nb)]
        return sess.elapsed_ms(0, nb - 1), stats

    for _ in range(args.warmup):
        device_step()
    modes0 = sess.pass_modes()
    sampler = ClockSampler(local_rank)
    sampler.start()
    dist_barrier(td)
    step_ms, batch_ms, all_stats = [], [], []
    edges = 0
    for _ in range(args.steps):
        ms, stats = device_step()
        step_ms.append(ms)
        batch_ms += [s["device_ms"] for s in stats]
        all_stats.append(stats)
        edges += sum(s["affected_edges"] for s in stats)
    dist_barrier(td)
    clocks = sampler.stop()
    modes = mode_delta(modes0, sess.pass_modes(), args.steps)
    t_dev = sum(step_ms) / 1e3
    t_max = dist_max(td, t_dev)
    edges_all = dist_sum(td, edges)
    value = edges_all / t_max if t_max > 0 else 0.0

    # end to end: host arrays through the C ABI, statistics read back per batch
    h2d = sum(bt.nbytes() for bt in p.batches)
    d2h = nb * 96 + 4 * p.num_nodes
    for _ in range(max(1, args.warmup // 2)):
        sess.reset()
        for b, bt in enumerate(p.batches):
            sess.apply(b, bt)
        sess.labels()
    e2e_s, e2e_edges, e2e_batch_ms = 0.0, 0, []
    for _ in range(args.steps):
        sess.reset()
        flush_l2()
        t0 = time.perf_counter()
        for b, bt in enumerate(p.batches):
            tb = time.perf_counter()
            st = sess.apply(b, bt)
            e2e_batch_ms.append(1e3 * (time.perf_counter() - tb))
            e2e_edges += st["affected_edges"]
        sess.labels()
        e2e_s += time.perf_counter() - t0
    e2e_max = dist_max(td, e2e_s)
    e2e_value = dist_sum(td, e2e_edges) / e2e_max if e2e_max > 0 else 0.0
    # every rank serves its shard of the mixed stream (the aggregation inside
    # is collective, so it runs before the other ranks leave)
    served = None if args.no_served else served_block(args, local_rank, rank, world, td)

    if rank != 0:
        return 0
    # roofline of the batch kernel (the only kernel of the timed region)
    peak, peak_kind = measured_peak_gbs()
    stats0 = all_stats[-1]
    bytes_step = sum(algorithmic_bytes(s, bt.edge_src.size, bt.inserted.size) for s, bt in zip(stats0, p.batches))
    kern_s = sum(s["device_ms"] for s in stats0) / 1e3
    achieved = bytes_step / kern_s / 1e9 if kern_s > 0 else 0.0
    traffic = None
    # DRAM traffic comes from an ncu capture of the same workload, when one exists
    tf = ROOT / "profiles" / f"traffic_engine_kernel_{args.workload}.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get("dram_bytes_per_launch")
        except Exception:
            traffic = None
    # CPU baseline: the oracle, single thread, bounded sample of the same workload
    cpu_edges, cpu_t, cpu_done = cpu_run(p, 1, args.cpu_budget_s)
    cpu = host_cpu()
    # FP64 oracle error on this workload, and the reference's own CUDA build
    fp64 = None
    if not args.no_fp64:
        progress("fp64 oracle")
        fp64 = fp64_error(p, sess.labels(), cpu["nproc"])
    irlp_full = None
    if not args.no_irlp:
        progress("IrLP full recompute")
        try:
            irlp_full = irlp_block(p, [s["device_ms"] for s in stats0], cpu["nproc"], args.irlp_budget_s,
                                   local_rank)
        except Exception as exc:  # reported, not fatal: it is a baseline
            irlp_full = {"error": repr(exc)[:300]}
    ref_cuda = None
    if not args.no_reference_cuda:
        progress("reference CUDA build")
        try:
            ref_cuda = reference_cuda(w, args.batches, stats0)
        except Exception as exc:  # reported, not fatal: it is a baseline
            ref_cuda = {"error": repr(exc)[:300]}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "fp32",
        "data": "synthetic (reference generator decisions, seed 42), inputs resident in HBM",
        "config": {"workload": workload_desc(args.workload, args.batches), "semantics": "ref", "parallelism": "replicas",
                   "l2": "flushed before every step (512 MiB memset)", "narrow_lanes": args.lanes or 8,
                   "blocks_per_sm": args.blocks_per_sm or "occupancy",
                   "affected_edges_per_step": edges // max(args.steps, 1)},
        "latency_ms": {"per": "batch", "p50": percentile(batch_ms, 0.5), "p99": percentile(batch_ms, 0.99),
                       "max": max(batch_ms) if batch_ms else None,
                       "e2e_p50": percentile(e2e_batch_ms, 0.5), "e2e_p99": percentile(e2e_batch_ms, 0.99)},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "timing": "wall clock, stream synchronised on both sides"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak if peak else None, "traffic": traffic,
                     "kernel": f"dlp::engine_kernel<{args.lanes or 8}>", "peak_source": peak_kind,
                     "algorithmic_bytes_per_step": bytes_step},
        "cpu_baseline": {"value": cpu_edges / cpu_t if cpu_t > 0 else 0.0, "unit": UNIT, "cores": 1, "kind": "port",
                         "sample": f"oracle port, 1 thread, first {cpu_done} of {nb} batches of the same workload",
                         "cpu_model": cpu["model"], "host_cores": cpu["nproc"]},
        "fp64_oracle_error": fp64,
        "irlp_full_recompute": irlp_full,
        "reference_cuda": ref_cuda,
        "clocks": clocks,
        "pass_modes_per_step": modes,
        "gpu_launches": args.steps * nb * 2,
    }
    if args.per_batch:
        line["per_batch"] = [{k: s[k] for k in ("batch", "iterations", "affected_edges", "frontier_visits",
                                                 "dirty_entries", "device_ms")} for s in stats0]
    if served is not None:
        line["served"] = served
    print(json.dumps(line), flush=True)
    return 0


# ------------------------------------------------------ served vs plain -----

def mix_sizes(count: int, lo: float, hi: float, seed: int):
    """Graph sizes log-uniform on [lo, hi] (numpy PCG64, fixed seed), average
    degree {3,5,7}[i mod 3], generator seed i."""
    import numpy as np
    rng = np.random.default_rng(seed)
    n = np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), count))).astype(int)
    return [(int(n[i]), (3, 5, 7)[i % 3], 10, i) for i in range(count)]


def shard_graphs(specs, rank: int, world: int) -> list[int]:
    """Indices of the graphs rank `rank` of `world` serves: graphs are
    independent, so they are split across GPUs with no collective on the data
    path. Greedy by expected edges (n x degree), largest first, to the least
    loaded rank; ties go to the lower rank, so every rank computes the same
    split."""
    load = [0] * world
    mine = []
    for i in sorted(range(len(specs)), key=lambda i: (-specs[i][0] * specs[i][1], i)):
        r = min(range(world), key=lambda r: (load[r], r))
        load[r] += specs[i][0] * specs[i][1]
        if r == rank:
            mine.append(i)
    return sorted(mine)


def make_problems(specs, threads: int):
    import concurrent.futures as cf
    import labelpropcuda_gb300 as dlp
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        return list(ex.map(lambda s: dlp.Problem(*s), specs))


def progress(msg: str) -> None:
    """Progress of a long run on stderr (stdout carries only the JSON line)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {msg}", file=sys.stderr, flush=True)


def stratified_plain(sizes_n, plain_time, per_stratum: int, bins: int, seed: int):
    """Stratified sample of whole graphs for the plain path: graphs binned by
    log(vertex count) into `bins` equal-width strata, `per_stratum` graphs
    drawn per stratum (seeded), each replayed serially by plain_time(index) ->
    seconds. Returns (estimated total seconds for all graphs, its standard
    error, graphs sampled): the stratified estimator sum_h N_h * mean_h with
    the finite-population correction."""
    import numpy as np
    logs = np.log(np.asarray(sizes_n, dtype=np.float64))
    edges = np.linspace(logs.min(), logs.max() + 1e-9, bins + 1)
    strata = np.clip(np.digitize(logs, edges) - 1, 0, bins - 1)
    rng = np.random.default_rng(seed)
    total, var, sampled = 0.0, 0.0, []
    for h in range(bins):
        members = np.flatnonzero(strata == h)
        if members.size == 0:
            continue
        k = min(per_stratum, members.size)
        pick = rng.choice(members, size=k, replace=False)
        t = np.array([plain_time(int(i)) for i in pick])
        sampled += [int(i) for i in pick]
        total += members.size * t.mean()
        if k > 1:
            var += members.size ** 2 * (1.0 - k / members.size) * t.var(ddof=1) / k
    return total, float(np.sqrt(var)), sampled


def served_block(args, local_rank, rank=0, world=1, td=None) -> dict:
    """Served vs plain over the mixed-graph stream. Default: the multi-instance
    configuration, 512 graphs with n log-uniform on [1e3, 5e5] (numpy PCG64
    seed 1000003), degree {3,5,7}[i mod 3], generator seed i, every graph's
    10 batches as 5,120 requests in batch-major order.
      batched          one engine launch per batch index over every graph
      served_saturated the continuous-batching server with every request
                       queued at t = 0 (host-to-device copies included)
      served_poisson   the same server with Poisson arrivals at fractions of
                       the saturated request rate, over a size-stratified
                       subset of the graphs (every k-th by vertex count, all
                       its requests); latency = finish - arrival
      plain            the server in serial mode (one request at a time, run
                       to its end: the plain per-batch path) replaying the same
                       requests graph by graph, on a stratified sample of whole
                       graphs (strata by log size), scaled to all graphs
    With several ranks each serves its shard of the graphs (shard_graphs);
    rates are summed over ranks and times take the slowest rank."""
    import numpy as np
    import labelpropcuda_gb300 as dlp
    from labelpropcuda_gb300 import PackedBatches
    t_setup = time.perf_counter()
    if args.served_shape == "stream":
        # serving-stream shape: larger graphs, requests of about 2% of a graph
        # (40 batches per graph); every graph first takes its first `skip`
        # batches (untimed), then --served-batches more are served
        lo, hi, count, gen_batches, nb = 1e4, 5e6, args.served_graphs or 256, 40, args.served_batches
        skip = 20 if args.served_skip < 0 else args.served_skip
    else:
        lo, hi, count, gen_batches, nb = 1e3, 5e5, args.served_graphs or 512, 10, 10
        skip = 0
    all_specs = [(n, d, gen_batches, sd) for n, d, _, sd in mix_sizes(count, lo, hi, 1000003)]
    mine = shard_graphs(all_specs, rank, world)
    specs = [all_specs[i] for i in mine]
    probs = make_problems(specs, min(16, os.cpu_count() or 1))
    lanes, bps, tune = args.served_lanes, 0, None
    if lanes == 0:  # the tuned launch shape for this GPU (cached per GPU model)
        sample = specs[:: max(1, len(specs) // 8)][:8]
        tune = dlp.autotune_cached([s[0] for s in sample], [s[1] for s in sample], batches=10, max_iterations=300,
                                   device=local_rank)
        lanes, bps = tune["narrow_lanes"], tune["blocks_per_sm"]
    eng = dlp.Engine(len(probs), 150 << 30, device=local_rank, narrow_lanes=lanes, blocks_per_sm=bps,
                     **(tune or {}).get("engine_kw", {}))
    gids = [eng.add_problem(p) for p in probs]
    warm = [p.batches[:skip] for p in probs]  # applied untimed before every measured phase
    for p in probs:  # the requests of this run: batches skip .. skip+nb-1 of each graph
        p.batches = p.batches[skip:skip + nb]
    packed = [PackedBatches([p.batches[b] for p in probs]) for b in range(nb)]
    setup_s = time.perf_counter() - t_setup
    progress(f"served setup {setup_s:.1f} s: {len(probs)} graphs, lanes {lanes}, blocks/SM {bps or 'occupancy'}")
    vertices = sum(p.num_nodes for p in probs)
    edges_full = sum(p.num_edges for p in probs)

    snaps = None  # the graphs' state after the warm-up batches, in host memory

    def reserve_all():
        for g, p, w in zip(gids, probs, warm):  # scratch sized up front: no allocation inside the timed runs
            eng.reserve(g, max(bt.edge_src.size for bt in p.batches + w), max(bt.deleted.size for bt in p.batches + w))

    def reset_all():
        nonlocal snaps
        if snaps is not None:  # back to the warmed-up state without replaying the warm-up
            for g, sn in zip(gids, snaps):
                eng.remove_graph(g)
                eng.restore_as(sn, g)
            reserve_all()
            eng.synchronize()
            return
        for g in gids:
            eng.reset_graph(g)
        for b in range(skip):  # the graphs' state before the served batches (untimed)
            eng.step([(g, b, w[b]) for g, w in zip(gids, warm)], wait=False)
        eng.synchronize()
        if skip > 0:
            snaps = [eng.snapshot(g) for g in gids]
            progress(f"warm state: {sum(len(x) for x in snaps) / 1e9:.1f} GB snapshotted to host memory")

    reserve_all()

    # batched: one launch per step over every graph
    def batched_run():
        reset_all()
        m0 = eng.pass_modes()
        first = eng.steps
        for b in range(nb):
            eng.step_device([(g, skip + b, packed[b].view(i)) for i, g in enumerate(gids)])
        eng.synchronize()
        ms = [eng.elapsed_ms(first + b, first + b) for b in range(nb)]
        ae = sum(eng.stats(g, skip + b)["affected_edges"] for g in gids for b in range(nb))
        return ms, ae, mode_delta(m0, eng.pass_modes(), 1)
    b_ms, b_ae, b_modes = batched_run()
    b_t = dist_max(td, sum(b_ms) / 1e3)
    b_ae = int(dist_sum(td, b_ae))
    batched = {"value": b_ae / b_t, "ms_per_step": 1e3 * b_t / nb,
               "step_ms_p50": percentile(b_ms, 0.5), "step_ms_max": max(b_ms),
               "affected_edges": b_ae, "launches": 2 * nb, "pass_modes": b_modes,
               "timing": "CUDA events around each step, batches resident in HBM"}
    progress(f"batched {batched['value'] / 1e9:.3f} G/s, step max {max(b_ms):.0f} ms")

    reqs = [(0.0, g, skip + b, probs[i].batches[b]) for b in range(nb) for i, g in enumerate(gids)]
    srv = dlp.Server(eng, memory_budget_bytes=150 << 30, slice_us=args.slice_us)
    for g, p in zip(gids, probs):
        srv.reserve(g, p.batches)

    def replay(trace):
        reset_all()
        res, span = srv.replay(trace)
        bad = [r for r in res if r["status"] != 0]
        if bad:
            raise RuntimeError(f"{len(bad)} requests failed: {bad[0]}")
        return res, span

    # saturation: everything queued at t = 0
    res, span = replay(reqs)
    req_edges = [r["stats"]["affected_edges"] for r in res]
    total_edges = sum(req_edges)
    sat_ae = dist_sum(td, total_edges)
    sat_rate = len(res) / span  # this rank's, for its own Poisson traces
    span = dist_max(td, span)
    svc = [1e3 * (r["finish_s"] - r["admit_s"]) for r in res]
    served_sat = {"value": sat_ae / span, "makespan_s": span, "requests": int(dist_sum(td, len(res))),
                  "requests_per_s": dist_sum(td, sat_rate), "service_ms_p50": dist_max(td, percentile(svc, 0.5)),
                  "service_ms_p99": dist_max(td, percentile(svc, 0.99))}
    progress(f"served saturated {served_sat['value'] / 1e9:.3f} G/s, makespan {span:.1f} s")

    # Poisson sweep over a size-stratified subset (every --sweep-stride-th
    # graph by vertex count, all its batches): its own saturated run first,
    # then Poisson arrivals at fractions of that request rate, every request
    # of the subset in each run (batch-major order: every graph's batches keep
    # their order)
    by_size = sorted(range(len(gids)), key=lambda i: (probs[i].num_nodes, i))
    sub = sorted(by_size[::max(1, args.sweep_stride)])
    sub_reqs = [(0.0, gids[i], skip + b, probs[i].batches[b]) for b in range(nb) for i in sub]
    res, sub_span = replay(sub_reqs)
    sub_rate = len(res) / sub_span
    sweep = [{"fraction_of_saturated": "saturated (all queued at t = 0)", "requests": int(dist_sum(td, len(res))),
              "value": dist_sum(td, sum(r["stats"]["affected_edges"] for r in res)) / dist_max(td, sub_span),
              "makespan_s": dist_max(td, sub_span),
              "latency_ms_p50": dist_max(td, percentile([1e3 * (r["finish_s"] - r["arrival_s"]) for r in res], 0.5)),
              "latency_ms_p99": dist_max(td, percentile([1e3 * (r["finish_s"] - r["arrival_s"]) for r in res],
                                                        0.99))}]
    progress(f"sweep subset: {len(sub)} graphs, {len(res)} requests, saturated {sub_rate:.1f} req/s")
    for frac in args.poisson_fractions:
        rate = frac * sub_rate
        rng = np.random.default_rng(7)
        times = np.cumsum(rng.exponential(1.0 / rate, len(sub_reqs)))
        trace = [(float(t), g, b, bt) for t, (_, g, b, bt) in zip(times, sub_reqs)]
        res, span = replay(trace)
        lat = [1e3 * (r["finish_s"] - r["arrival_s"]) for r in res]
        p_ae = dist_sum(td, sum(r["stats"]["affected_edges"] for r in res))
        span = dist_max(td, span)
        row = {"fraction_of_saturated": frac, "offered_requests_per_s": dist_sum(td, rate),
               "requests": int(dist_sum(td, len(res))), "value": p_ae / span, "makespan_s": span,
               "latency_ms_p50": dist_max(td, percentile(lat, 0.5)),
               "latency_ms_p99": dist_max(td, percentile(lat, 0.99)), "latency_ms_max": dist_max(td, max(lat))}
        sweep.append(row)
        progress(f"poisson x{frac}: {row['requests']} requests, {row['value'] / 1e9:.3f} G/s, "
                 f"p50 {row['latency_ms_p50']:.1f} ms, p99 {row['latency_ms_p99']:.1f} ms")
    srv.close()

    # plain: the same requests, one at a time, graph by graph (stratified sample)
    reset_all()
    srv = dlp.Server(eng, serial=True)
    for g, p in zip(gids, probs):
        srv.reserve(g, p.batches)
    pl_svc, pl_edges, pl_graph_s = [], 0, {}

    def plain_time(i: int) -> float:
        nonlocal pl_edges
        res, span = srv.replay([(0.0, gids[i], skip + b, probs[i].batches[b]) for b in range(nb)])
        pl_svc.extend(1e3 * (r["finish_s"] - r["admit_s"]) for r in res)
        pl_edges += sum(r["stats"]["affected_edges"] for r in res)
        pl_graph_s[i] = span
        return span
    est_s, est_se, sampled = stratified_plain([p.num_nodes for p in probs], plain_time, args.plain_per_stratum,
                                              args.plain_strata, 11)
    srv.close()
    plain_v = dist_sum(td, total_edges / est_s if est_s > 0 else 0.0)  # every GPU runs its own plain path
    lo_v = dist_sum(td, total_edges / (est_s + 2 * est_se) if est_s > 0 else 0.0)
    hi_v = dist_sum(td, total_edges / max(est_s - 2 * est_se, 1e-9) if est_s > 0 else 0.0)
    progress(f"plain {plain_v / 1e6:.1f} M/s (estimated {est_s:.1f} +- {est_se:.1f} s for all graphs, "
             f"{len(sampled)} sampled)")
    plain = {"value": plain_v, "value_2se_interval": [lo_v, hi_v],
             "estimated_seconds_all_graphs": est_s, "standard_error_s": est_se,
             "sampled_graphs": len(sampled), "sampled_requests": len(sampled) * nb,
             "sampled_seconds": sum(pl_graph_s.values()),
             "service_ms_p50": percentile(pl_svc, 0.5), "service_ms_p99": percentile(pl_svc, 0.99),
             "sample": (f"stratified: {args.plain_strata} strata by log vertex count, {args.plain_per_stratum} whole "
                        f"graphs per stratum (seed 11), all {nb} requests of each replayed one at a time; total "
                        f"time estimated as sum over strata of stratum size x mean graph time; value = the "
                        f"trace's affected edges / that estimate")}
    sat_sweep = [r for r in sweep if r["fraction_of_saturated"] == 1.0]
    out = {"workload": (f"mixed-graph stream ({args.served_shape}): {len(all_specs)} graphs ({len(probs)} on this "
                        f"rank of {world}), n log-uniform on [{lo:.0e}, {hi:.0e}], {gen_batches} batches generated per "
                        f"graph, batches {skip}-{skip + nb - 1} served after the first {skip} (numpy seed "
                        f"1000003), degree {{3,5,7}}[i mod 3], generator seed i, batches 90/1/9 insert/GT/delete, "
                        f"delta 1e-4, maxIter 1e5, ref semantics; {vertices} vertices, {edges_full} directed "
                        f"edges in all; {len(reqs)} requests"),
           "config": "multi-instance batching (512 graphs)" if args.served_shape == "mixed" and count == 512
           else f"{count} graphs",
           "setup_s": setup_s, "batched": batched, "served_saturated": served_sat,
           "served_poisson_sweep": sweep,
           "sweep_subset": f"{len(sub)} of {len(gids)} graphs (every {args.sweep_stride}th by vertex count), "
                           f"{len(sub_reqs)} requests per run; Poisson arrivals (numpy seed 7) at fractions of the "
                           f"subset's saturated request rate; latency = finish - arrival",
           "plain": plain,
           "served_over_plain": served_sat["value"] / plain_v if plain_v else None,
           "batched_over_plain": batched["value"] / plain_v if plain_v else None,
           "p99_latency_ms_at_saturated_offer": sat_sweep[0]["latency_ms_p99"] if sat_sweep else None,
           "slice_us": args.slice_us, "narrow_lanes": lanes, "blocks_per_sm": bps or "occupancy",
           "autotune": tune}
    eng.close()
    return out


def launch_ranks(argv: list[str], n: int) -> int:
    """Runs this script as n ranks on this node (one per GPU: RANK, LOCAL_RANK,
    WORLD_SIZE, MASTER_ADDR/PORT in each one's environment), the way
    torch.distributed.run would, and waits for all of them. Rank 0 prints the
    JSON line. Returns the first nonzero exit code, else 0."""
    import socket
    with socket.socket() as sk:  # a free port for the gloo rendezvous
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    procs = []
    for r in range(n):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE=str(n), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, str(Path(__file__).resolve())] + argv, env=env))
    codes = [p.wait() for p in procs]
    return next((c for c in codes if c != 0), 0)


def shard_check(args, td, rank, world) -> int:
    """Host-only check of the multi-rank plumbing (no GPU work): every rank
    takes its shard of the mixed stream and the per-rank counts are reduced
    with the same collectives the served block uses."""
    specs = [(n, d, 10, sd) for n, d, _, sd in mix_sizes(args.served_graphs or 512, 1e3, 5e5, 1000003)]
    mine = shard_graphs(specs, rank, world)
    load = sum(specs[i][0] * specs[i][1] for i in mine)
    graphs = int(dist_sum(td, len(mine)))
    total_load = int(dist_sum(td, load))
    max_load = int(dist_max(td, load))
    if td is not None:
        import torch
        t = torch.zeros(len(specs), dtype=torch.int64)
        t[mine] = rank + 1
        td.all_reduce(t)
        owners = t.tolist()
    else:
        owners = [1] * len(specs)
    if rank == 0:
        print(json.dumps({"impl": "shard-check", "n_gpus": world, "graphs": graphs, "total_load": total_load,
                          "max_load": max_load, "owners": owners}), flush=True)
    return 0


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference", "shard-check"], default="gb300")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="config2")
    ap.add_argument("--lanes", type=int, default=0)
    ap.add_argument("--batches", type=int, default=0, help="replay only the first N batches (0: all)")
    ap.add_argument("--blocks-per-sm", type=int, default=0)
    ap.add_argument("--cpu-budget-s", type=float, default=15.0)
    ap.add_argument("--ref-budget-s", type=float, default=20.0)
    ap.add_argument("--served-graphs", type=int, default=0, help="0: 512 (mixed shape) / 256 (stream shape)")
    ap.add_argument("--served-shape", choices=["mixed", "stream"], default="mixed",
                    help="mixed: sizes 1e3-5e5, 10 batches; stream: sizes 1e4-5e6, 40 batches (about 2%% of a graph "
                         "per request), the first --served-batches of each served")
    ap.add_argument("--served-batches", type=int, default=5)
    ap.add_argument("--served-skip", type=int, default=-1, help="stream shape: batches applied before serving "
                    "(default 20)")
    ap.add_argument("--served-lanes", type=int, default=0, help="0: the tuned shape")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--slice-us", type=float, default=2000.0)
    ap.add_argument("--poisson-fractions", type=lambda x: [float(v) for v in x.split(",")],
                    default=[0.25, 0.5, 0.75, 1.0], help="offered rates as fractions of the saturated rate")
    ap.add_argument("--sweep-stride", type=int, default=4, help="Poisson sweep over every k-th graph by size")
    ap.add_argument("--plain-per-stratum", type=int, default=3)
    ap.add_argument("--plain-strata", type=int, default=8)
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 oracle error of the headline workload")
    ap.add_argument("--no-irlp", action="store_true", help="skip the IrLP full-recompute comparison")
    ap.add_argument("--irlp-budget-s", type=float, default=10.0, help="host time for the CPU IrLP leg")
    ap.add_argument("--per-batch", action="store_true", help="add every batch's statistics to the line")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="skip timing the reference's own CUDA build (oracle/_ref/ref_kernels)")
    ap.add_argument("--input-cache", default=None,
                    help="directory of the binary input cache (DLP_INPUT_CACHE): generated problems are kept there "
                         "and read back on later runs")
    args = ap.parse_args(argv)
    if args.input_cache:
        os.environ["DLP_INPUT_CACHE"] = args.input_cache
    if args.warmup < 3 and args.impl == "gb300":
        args.warmup = 3
    if "WORLD_SIZE" not in os.environ and args.gpus > 1:
        return launch_ranks(argv, args.gpus)
    rank, world, local_rank = dist_env()
    td = dist_init(world)
    try:
        if args.impl == "reference":
            return reference_arm(args, td, rank)
        if args.impl == "shard-check":
            return shard_check(args, td, rank, world)
        from labelpropcuda_gb300 import build
        build.build()
        return gpu_arm(args, td, rank, world, local_rank)
    finally:
        if td is not None:
            td.destroy_process_group()


if __name__ == "__main__":
    sys.exit(main())
