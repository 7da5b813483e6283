"""Benchmark: trials recovered per second on the dense phase-transition sweep.

Workload: the sweep of independent dense Gaussian trials (n in {1024,...,16384},
delta in {0.1,...,0.9}, rho on a 0.02 grid up to 0.5; gaga_gb300/sweep.py), NIHT with
||y - A x|| <= 1e-4 ||y||, maxiter 5000; a trial is recovered when its relative l2
error is <= 1e-3.  A step is one wave of the sweep (the 4096-trial sweep split into 16
interleaved waves of 256 trials).  Each trial's A and x are drawn on the device from
(seed + trial id) inside the timed region; every trial's A is a separate matrix.

  value : recovered trials / device time of the batched (tuned) form's kernels
  e2e   : recovered trials / wall time of gb_cs_solve_batch called with host arrays
          (trial table in, per-trial iterations/errors/verdicts out)
  plain : the single-trial drop-in (gb_cs_generate_and_solve per trial) on a sample of
          the same wave, for the tuned-vs-plain ratio
  cpu_baseline / --impl reference : the CPU oracle (oracle/gbo.c, OpenMP inside each
          trial) on a bounded sample of the wave

Multi-GPU: each rank solves its own waves (weak scaling, no data-path collective).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "trials recovered/s (rel err<=1e-3), tuned vs plain on 1 GB300; matvec % HBM peak"
TOTAL, WAVES, SEED, TOL_REL, MAXITER = 4096, 16, 20240607, 1e-4, 5000


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu, self.rows, self.proc = gpu, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
                for nm, v in zip(names, r[5:9]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                pass
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def wave_arrays(w):
    from gaga_gb300 import sweep

    n, m, k, tid = sweep.sweep_trials(TOTAL)
    idx = sweep.wave(TOTAL, WAVES, w % WAVES)
    return n[idx], m[idx], k[idx], tid[idx]


def cpu_sample(w, count):
    n, m, k, tid = wave_arrays(w)
    step = max(1, len(n) // count)
    sel = np.arange(0, len(n), step)[:count]
    return n[sel], m[sel], k[sel], tid[sel]


def run_cpu(w, count):
    from oracle import gbo

    n, m, k, tid = cpu_sample(w, count)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    ok, iters, err = gbo.solve_dense_trials(n, m, k, SEED, tid, alg="NIHT", tol_rel=TOL_REL, maxiter=MAXITER,
                                            threads=cores)
    dt = time.perf_counter() - t0
    return {"value": ok / dt, "unit": "trials/s", "cores": cores, "kind": "port",
            "sample": "%d trials of wave %d (every %d-th; n=%s), NIHT, CPU oracle oracle/gbo.c with OpenMP inside each "
                      "trial, generation included; %d recovered in %.1f s" % (len(n), w, len(wave_arrays(w)[0]) // count,
                                                                               sorted(set(n.tolist())), ok, dt)}


def bench_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    t_steps = []
    last = None
    for s in range(args.warmup + args.steps):
        r = run_cpu(s, args.cpu_trials)
        if s >= args.warmup:
            t_steps.append(r)
        last = r
    value = float(np.mean([r["value"] for r in t_steps]))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "trials/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded Philox trials)",
            "config": {"workload": "dense phase-transition sweep, NIHT, bounded CPU sample per wave",
                       "trials_per_sample": args.cpu_trials},
            "cpu_baseline": dict(last, value=value),
            "e2e": {"value": value, "unit": "trials/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def bench_ours(args):
    import torch

    import gaga_gb300 as gb

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    gb._lib.load()
    peak, peak_kind = peaks()

    def solve_wave(w):
        n, m, k, tid = wave_arrays(w)
        t0 = time.perf_counter()
        ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg="NIHT", tol_rel=TOL_REL, maxiter=MAXITER)
        wall = time.perf_counter() - t0
        nbytes, kms = gb.batch_last_stats()
        return ns, wall, kms, nbytes, len(n), iters

    # warm-up waves
    from gaga_gb300 import sweep

    for s in range(args.warmup):
        solve_wave(sweep.rank_wave(rank, world, s))
    sampler = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler.start()
    t_start = time.perf_counter()
    tot_ok = tot_trials = 0
    tot_wall = tot_kms = tot_bytes = 0.0
    launches = 0
    for s in range(args.steps):
        w = sweep.rank_wave(rank, world, args.warmup + s)
        ns, wall, kms, nbytes, cnt, _ = solve_wave(w)
        tot_ok += ns
        tot_trials += cnt
        tot_wall += wall
        tot_kms += kms
        tot_bytes += nbytes
        # one persistent launch per cluster-size class present in the wave
        launches += len({1 if nn <= 2048 else 2 if nn <= 4096 else 4 if nn <= 8192 else 8 for nn in wave_arrays(w)[0]})
    torch.cuda.synchronize()
    elapsed = time.perf_counter() - t_start
    clocks = sampler.stop()
    if world > 1:
        t = torch.tensor([elapsed, tot_kms, tot_wall], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        c = torch.tensor([tot_ok, tot_trials, tot_bytes], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(c)
        elapsed, tot_kms, tot_wall = t.tolist()
        tot_ok, tot_trials, tot_bytes = c.tolist()
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    value = tot_ok / (tot_kms / 1e3)
    e2e = tot_ok / tot_wall
    achieved = tot_bytes / (tot_kms / 1e3) / 1e9 / max(1, world)
    line = {"metric": METRIC, "value": value, "unit": "trials/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_kms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded Philox Gaussian trials drawn on device)",
            "config": {"workload": "dense phase-transition sweep (4096 trials, n 1024-16384, delta 0.1-0.9, "
                                   "rho 0.02-0.5), NIHT tol 1e-4*||y||, one 256-trial wave per step per GPU",
                       "form": "tuned: batched slot graphs (device trial queue, device generation)",
                       "trials_per_step": int(tot_trials // max(1, args.steps)), "l2": "working set >> L2 (A up to "
                                                                                         "966 MB per trial)"},
            "recovered": int(tot_ok), "trials": int(tot_trials),
            "e2e": {"value": e2e, "unit": "trials/s", "h2d_bytes_per_step": 16 * 256, "d2h_bytes_per_step": 12 * 256},
            "batched_matvec_bytes_per_s": {"achieved": achieved, "unit": "GB/s", "frac": achieved / peak,
                                           "what": "algorithmic dense operator bytes of all trials / device time of "
                                                   "the whole batched form (generation and control included)"},
            "gpu_launches": launches, "clocks": clocks}
    mv = matvec_roofline(peak, peak_kind)
    line["roofline"] = mv["at"]
    line["matvec"] = mv
    if args.plain_trials > 0 and world == 1:
        line["plain"] = bench_plain(args)
        line["tuned_vs_plain"] = value / line["plain"]["value"] if line["plain"]["value"] else None
    if not args.no_cpu and world == 1:
        line["cpu_baseline"] = run_cpu(args.warmup, args.cpu_trials)
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def matvec_roofline(peak, peak_kind, m=14746, n=16384, k=5000, reps=20):
    """Dense A^T r (k_dense_at, the dominant kernel) and A x_S (k_dense_av) on the sweep's
    largest trial shape, timed with CUDA events on the stream they run on."""
    import ctypes as C

    import torch

    import gaga_gb300 as gb

    L = gb._lib.load()
    g = torch.Generator(device="cuda").manual_seed(1)
    lda = (m + 31) // 32 * 32  # the library's own layout: 128-byte aligned columns
    A = torch.randn(n * lda, device="cuda", generator=g) / np.sqrt(m)  # column-major
    r = torch.randn(m, device="cuda", generator=g)
    x = torch.zeros(n, device="cuda")
    x[torch.randperm(n, device="cuda", generator=g)[:k]] = 1.0
    g_out, y_out = torch.empty(n, device="cuda"), torch.empty(m, device="cuda")
    s = torch.cuda.Stream()
    res = {}
    for name, tr, vin, vout, nbytes in (("at", 1, r, g_out, 4.0 * m * n + 4 * m + 4 * n),
                                        ("av", 0, x, y_out, 4.0 * m * k + 8 * k + 4 * m)):
        with torch.cuda.stream(s):
            for _ in range(3):
                L.gb_cs_dense_apply_noalloc(A.data_ptr(), lda, m, n, tr, vin.data_ptr(), vout.data_ptr(),
                                            C.c_void_p(s.cuda_stream))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.synchronize()
            e0.record(s)
            for _ in range(reps):
                L.gb_cs_dense_apply_noalloc(A.data_ptr(), lda, m, n, tr, vin.data_ptr(), vout.data_ptr(),
                                            C.c_void_p(s.cuda_stream))
            e1.record(s)
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / reps
        ach = nbytes / t / 1e9
        res[name] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                     "traffic": None, "kernel": "k_dense_at" if name == "at" else "k_dense_av (+ support compaction)",
                     "shape": "m=%d n=%d lda=%d%s, A %.0f MB > L2" % (m, n, lda, "" if name == "at" else
                                                                      " |S|=%d" % k, 4.0 * m * n / 1e6),
                     "us_per_launch": t * 1e6, "peak_source": peak_kind}
    del A
    torch.cuda.empty_cache()
    return res


def bench_plain(args):
    """Single-trial drop-in on a sample of one wave: gb_cs_generate_and_solve per trial."""
    import gaga_gb300 as gb

    n, m, k, tid = wave_arrays(args.warmup)
    step = max(1, len(n) // args.plain_trials)
    sel = np.arange(0, len(n), step)[: args.plain_trials]
    ok = 0
    t0 = time.perf_counter()
    for i in sel:
        opts = gb.gaga_options("tol", TOL_REL, "tol_is_relative", 1, "maxiter", MAXITER, "seed", int(SEED + tid[i]))
        x, xt, r = gb.generate_and_solve("NIHT", "gen", int(k[i]), int(m[i]), int(n[i]), 0, opts)
        ok += int(r.norms[1] <= 1e-3)
    dt = time.perf_counter() - t0
    return {"value": ok / dt, "unit": "trials/s", "trials": int(len(sel)), "recovered": ok, "seconds": dt,
            "sample": "every %d-th trial of wave %d" % (step, args.warmup)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-trials", type=int, default=32)
    ap.add_argument("--cpu-trials", type=int, default=8)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
