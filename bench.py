"""Benchmark: trials recovered per second on the dense phase-transition sweep, the tuned
form (batched + BF16 tensor cores + learned warm start) against the plain single-trial
FP32 form.

Workload: 4096 dense Gaussian CGIHT trials with ||y - A x|| <= 1e-4 ||y||, maxiter 5000;
a trial is recovered when its relative l2 error is <= 1e-3 (gaga_gb300/sweep.py):
  - 3072 independent trials (n in {1024,...,16384}, delta in {0.1,...,0.9}, rho on a
    0.02 grid up to 0.5), each with its own A and x drawn on the device from
    (seed + trial id): the batched form (gb_cs_solve_batch: cluster-resident kernel for
    n <= 8192, slot graphs for the rest), learned warm start;
  - 1024 trials sharing one A (n = 8192, m = 4096, rho cycling the same grid): the
    shared-matrix form (gb_cs_solve_shared_batch; split-BF16 tcgen05 GEMMs in lockstep,
    least-squares debias), learned warm start.
A step is one quarter of the sweep: 768 independent trials plus 256 shared-matrix trials.
Problem generation runs inside the timed region.

  value : recovered trials / device time of both forms
  e2e   : recovered trials / wall time of the two calls made with host arrays (trial
          tables in, per-trial iterations/errors/verdicts out)
  plain : the single-trial FP32 drop-in, zero-initialised CGIHT, on every trial of the
          first timed step (gb_cs_generate_and_solve for the independent trials with the
          same seeds, gb_cs_solve on the shared A and each y), each call timed with CUDA
          events; scaled to the 3072 + 1024 mix for tuned_vs_plain; the verdicts of the same
          trials give the agreement between the two forms, split by direction
  faithful : the same sweep from the zero start with the 24-bit A^T r operand (the form whose
          verdicts are meant to equal plain's), its rate over plain and its agreement with
          the plain leg's verdicts
  niht_sweep : the same sweep with NIHT (batched + shared-matrix forms, no warm start)
  learned_warm_start : the trained MLP warm start against zero-initialised CGIHT on 2048
          fresh trials of its own workload (n = 8192, delta 0.1-0.6, rho 0.05-0.45)
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
TOTAL, SHARED, PARTS, SEED, TOL_REL, MAXITER = 4096, 1024, 4, 20240607, 1e-4, 5000
ALG = "CGIHT"
WORKLOAD = ("dense phase-transition sweep: 4096 CGIHT trials = 3072 independent (n 1024-16384, delta 0.1-0.9, "
            "rho 0.02-0.5) + 1024 sharing one A (n 8192, m 4096, rho 0.02-0.5); tol 1e-4*||y||; one quarter of "
            "the sweep per step per GPU")
SHARED_SEED = SEED + 1000003  # keys of the shared subset stay clear of the independent trials' seed + id


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
    """Independent trials of step w: one of PARTS interleaved waves of the 3072 (waves beyond
    PARTS repeat the grid points with new trial ids, so no two steps share a trial)."""
    from gaga_gb300 import sweep

    return sweep.wave_trials(TOTAL - SHARED, PARTS, w)


def shared_part(w):
    """Shared-matrix trials of step w: (k array, first trial index)."""
    from gaga_gb300 import sweep

    ks = sweep.shared_subset(SHARED)
    q = w % PARTS
    return np.ascontiguousarray(ks[q::PARTS]), q * (SHARED // PARTS)


def cpu_sample(w, count):
    n, m, k, tid = wave_arrays(w)
    step = max(1, len(n) // count)
    sel = np.arange(0, len(n), step)[:count]
    return n[sel], m[sel], k[sel], tid[sel]


def run_cpu(w, count):
    """The CPU oracle on the step's mix: 3/4 of `count` independent trials (every few of the
    wave, generated from the same keys) and 1/4 shared-matrix trials (the step's shared A and
    signals, regenerated by the oracle's generators), so the rate covers the same 3:1 mix as
    the GPU's value."""
    from gaga_gb300 import sweep
    from oracle import gbo

    n_sh = max(1, count // 4)
    n, m, k, tid = cpu_sample(w, count - n_sh)
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    ok, iters, err = gbo.solve_dense_trials(n, m, k, SEED, tid, alg=ALG, tol_rel=TOL_REL, maxiter=MAXITER,
                                            threads=cores)
    t1 = time.perf_counter()
    # shared-matrix trials: A from SHARED_SEED, x0_t from SHARED_SEED + 1 + trial (the GPU form's keys)
    ks, first = shared_part(w)
    sel = np.linspace(0, len(ks) - 1, n_sh).astype(int)
    sm, sn = sweep.SHARED_M, sweep.SHARED_N
    A = gbo.gen_dense(sm, sn, SHARED_SEED, 0, 1)
    op = gbo.Op.dense(A, sm, sn)
    ok_sh = 0
    for t in sel:
        x0, kt = gbo.gen_vector(sn, int(ks[t]), 1, SHARED_SEED + 1 + first + int(t), 0)
        y = gbo.A(op, x0)
        x, info = gbo.solve(ALG, op, y, kt, TOL_REL * float(np.linalg.norm(y)), maxiter=MAXITER, threads=cores)
        ok_sh += int(np.linalg.norm(x - x0) <= 1e-3 * np.linalg.norm(x0))
    t2 = time.perf_counter()
    dt = t2 - t0
    tot_ok = ok + ok_sh
    return {"value": tot_ok / dt, "unit": "trials/s", "cores": cores, "kind": "port", "seconds": dt,
            "sample": ("%d independent trials of wave %d (every %d-th; n=%s) and %d shared-matrix trials "
                       "(n=%d, m=%d) of the step, %s, CPU oracle oracle/gbo.c with OpenMP inside each trial, "
                       "generation included; %d + %d recovered in %.1f + %.1f s" % (
                           len(n), w, len(wave_arrays(w)[0]) // max(1, count - n_sh), sorted(set(n.tolist())),
                           len(sel), sn, sm, ALG, ok, ok_sh, t1 - t0, t2 - t1, ))}


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
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean([r["seconds"] for r in t_steps])) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": "synthetic (seeded Philox trials)",
            "config": {"workload": WORKLOAD, "form": "reference: the CPU restatement of the algorithm (oracle), a "
                                                     "bounded sample of each step's trials",
                       "trials_per_step": TOTAL // PARTS,
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
    tpeak, tpeak_kind = tensor_peak()

    # schedule of the batched form, measured on a probe of the first step (untimed)
    from gaga_gb300 import autotune

    n0, m0, k0, t0_ = wave_arrays(sweep_rank_first(rank, world))
    params = gb.learned.load_weights()
    sched = autotune.tune_batch(n0, m0, k0, SEED, t0_, alg=ALG, tol_rel=TOL_REL, maxiter=MAXITER,
                                use_cache=not args.retune, learned_params=params, grad_format=args.grad_format,
                                residual_refresh=args.residual_refresh)

    def solve_step(w, alg=ALG, lp=params, schedule=sched, gfmt=args.grad_format):
        """One quarter of the sweep: independent trials, then the shared-matrix trials."""
        n, m, k, tid = wave_arrays(w)
        t0 = time.perf_counter()
        per_trial = None
        if gfmt == "transition":  # 24-bit operand near the phase transition, BF16 elsewhere
            from gaga_gb300 import transition

            per_trial = transition.operand_formats(n, m, k)
        ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg=alg, tol_rel=TOL_REL, maxiter=MAXITER,
                                            slots=schedule["slots"], sm_share=schedule["sm_share"],
                                            cluster=schedule.get("cluster", 0), av_rows=schedule.get("av_rows", 0),
                                            learned_params=lp,
                                            grad_format="a24" if per_trial is not None else gfmt,
                                            grad_formats=per_trial, residual_refresh=args.residual_refresh)
        t1 = time.perf_counter()
        nbytes, kms = gb.batch_last_stats()
        ks, first = shared_part(w)
        ns2, it2, err2, ok2 = gb.solve_shared_batch(gb.sweep.SHARED_M, gb.sweep.SHARED_N, ks, SHARED_SEED,
                                                    tol_rel=TOL_REL, maxiter=MAXITER, first_trial=first, alg=alg,
                                                    learned_params=lp)
        t2 = time.perf_counter()
        flops, kms2 = gb.shared_last_stats()
        fb = gb.shared_last_fallbacks() if lp is not None else 0
        return dict(ok=ns + ns2, trials=len(n) + len(ks), wall=t2 - t0, kms=kms + kms2, bytes=nbytes, flops=flops,
                    kms_batch=kms, kms_shared=kms2, ok_batch=ns, ok_shared=ns2, n_batch=len(n), n_shared=len(ks),
                    verdict_batch=ok, verdict_shared=ok2, iters_batch=iters, iters_shared=it2, wall_batch=t1 - t0,
                    wall_shared=t2 - t1, fallbacks_shared=fb,
                    h2d=12 * len(n) + 4 * len(ks), d2h=12 * (len(n) + len(ks)))

    from gaga_gb300 import sweep

    for s in range(args.warmup):
        solve_step(sweep.rank_wave(rank, world, s))
    sampler = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    sampler.start()
    acc = {}
    first_step = None
    launches = 0
    for s in range(args.steps):
        w = sweep.rank_wave(rank, world, args.warmup + s)
        r = solve_step(w)
        if first_step is None:
            first_step = (w, r)
        for key in ("ok", "trials", "wall", "kms", "bytes", "flops", "kms_batch", "kms_shared", "ok_batch", "ok_shared",
                    "n_batch", "n_shared", "wall_batch", "wall_shared", "h2d", "d2h", "fallbacks_shared"):
            acc[key] = acc.get(key, 0) + r[key]
        # host-issued launches: one graph per slot stream and the cluster-resident kernel of
        # the batched form (twice with the warm start's fallback pass); the shared form's 9
        # setup kernels and GEMMs, its graph and its verdict kernel
        launches += 2 * (sched["slots"] + 1) + 11
    torch.cuda.synchronize()
    clocks = sampler.stop()
    if world > 1:
        t = torch.tensor([acc["kms"], acc["wall"]], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        c = torch.tensor([acc["ok"], acc["trials"], acc["bytes"]], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(c)
        acc["kms"], acc["wall"] = t.tolist()
        acc["ok"], acc["trials"], acc["bytes"] = c.tolist()
    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()
        return
    value = acc["ok"] / (acc["kms"] / 1e3)
    e2e = acc["ok"] / acc["wall"]
    achieved = acc["bytes"] / (acc["kms_batch"] / 1e3) / 1e9 / max(1, world)
    gemm_tf = acc["flops"] / (acc["kms_shared"] / 1e3) / 1e12
    line = {"metric": METRIC, "value": value, "unit": "trials/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": acc["kms"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32 (shared-matrix part: bf16 GEMM, fp32 accumulate)",
            "data": "synthetic (seeded Philox Gaussian trials drawn on device)",
            "config": {"workload": WORKLOAD,
                       "form": "tuned: batched form (n <= 8192: cluster-resident learned-CGIHT kernel, one "
                               "thread-block cluster per trial; larger: slot graphs; device trial queues, device "
                               "generation) + shared-matrix form (CGIHT in lockstep, split-BF16 tcgen05 GEMMs, FP64-"
                               "scalar CG debias), both starting from the learned warm start with the plain fallback",
                       "independent_grad_operand": {"fp32": "FP32 A", "a24": "A rounded to 24 bits (3 bytes per "
                                                    "entry)", "bf16": "A rounded to BF16 (2 bytes per entry)"}[
                           args.grad_format] + " for A^T r; A x, residual and stopping test on FP32 A",
                       "independent_residual": ("y - A x every %d-th restricted step on an unchanged support, "
                                                "r - alpha A p between" % args.residual_refresh)
                       if args.residual_refresh > 0 else "y - A x at every step",
                       "schedule": {"slots": sched["slots"], "sm_share": sched["sm_share"],
                                    "cluster": sched.get("cluster", 0), "av_rows": sched.get("av_rows", 128),
                                    "picked_by": "autotune over %d candidates on %d probe trials%s" % (
                                        len(sched["candidates"]), sched["probe_trials"],
                                        " (cached)" if sched.get("cached") else "")},
                       "trials_per_step": int(acc["trials"] // max(1, args.steps)),
                       "l2": "working set >> L2 (A up to 966 MB per trial; shared form 600 MB of BF16 operands)"},
            "recovered": int(acc["ok"]), "trials": int(acc["trials"]),
            "parts": {"independent": {"trials": int(acc["n_batch"]), "recovered": int(acc["ok_batch"]),
                                      "kernel_ms": acc["kms_batch"],
                                      "recovered_per_s": acc["ok_batch"] / (acc["kms_batch"] / 1e3)},
                      "shared_matrix": {"trials": int(acc["n_shared"]), "recovered": int(acc["ok_shared"]),
                                        "kernel_ms": acc["kms_shared"],
                                        "warm_start_fallbacks": int(acc["fallbacks_shared"]),
                                        "recovered_per_s": acc["ok_shared"] / (acc["kms_shared"] / 1e3),
                                        "gemm_tflops": gemm_tf,
                                        "gemm_frac": gemm_tf / tpeak if tpeak else None}},
            "e2e": {"value": e2e, "unit": "trials/s", "h2d_bytes_per_step": int(acc["h2d"] // args.steps),
                    "d2h_bytes_per_step": int(acc["d2h"] // args.steps)},
            "batched_matvec_bytes_per_s": {"achieved": achieved, "unit": "GB/s", "frac": achieved / peak,
                                           "what": "algorithmic dense operator bytes of the independent trials / "
                                                   "device time of the whole batched form (generation and control "
                                                   "included)"},
            "gpu_launches": launches,
            "gpu_launches_note": "host-issued launches (kernels and graphs); the graphs run the solver kernels in "
                                 "device-side WHILE loops",
            "clocks": clocks}
    # the roofline of the tuned form's A^T r at the sweep's largest trial (the compact operand
    # when the tuned form uses one; the FP32 kernels stay in "matvec")
    mv = matvec_roofline(peak, peak_kind, grad_format=args.grad_format)
    line["roofline"] = mv.get("at_c", mv["at"])
    line["matvec"] = mv
    line["resident"] = resident_roofline(peak, peak_kind, cluster=sched.get("cluster", 0))
    line["resident_tuned"] = resident_roofline(peak, peak_kind, cluster=sched.get("cluster", 0), alg=ALG,
                                               learned_params=params, grad_format=args.grad_format,
                                               residual_refresh=args.residual_refresh)
    if not args.no_configs:
        line["single_trial_configs"] = bench_configs(cpu=not args.no_cpu)
    line["gemm"] = gemm_roofline(tpeak, tpeak_kind)
    line["operators"] = operators_roofline(peak, peak_kind)
    if args.plain_trials > 0 and world == 1:
        pverd = {}
        line["plain"] = bench_plain(args, first_step, pverd)
        line["tuned_vs_plain"] = value / line["plain"]["value"] if line["plain"]["value"] else None
        line["tuned_vs_plain_e2e"] = e2e / line["plain"]["value"] if line["plain"]["value"] else None
        if args.faithful_steps > 0:
            line["faithful"] = bench_faithful(args, solve_step, pverd, line["plain"]["value"], n0, m0, k0, t0_)
    if args.niht_steps > 0 and world == 1:
        line["niht_sweep"] = bench_niht(args, solve_step)
    if args.learned_trials > 0 and world == 1:
        line["learned_warm_start"] = bench_learned(args)
    if not args.no_cpu and world == 1:
        line["cpu_baseline"] = run_cpu(args.warmup, args.cpu_trials)
    print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def bench_faithful(args, solve_step, pverd, plain_value, n0, m0, k0, t0_):
    """The same sweep in the form whose verdicts are meant to match the plain drop-in's:
    batched + shared-matrix as in the headline, but from the zero start (no learned warm
    start) and with the 24-bit A^T r operand (rounding at 2^-16 leaves the trajectories'
    verdicts unchanged, where BF16's 2^-9 moves a few near the phase transition), residual
    recurrence as the headline.  Device time over the timed steps' waves; verdicts of the
    first timed step against the plain leg's on the same sampled trials."""
    from gaga_gb300 import autotune, sweep

    sched = autotune.tune_batch(n0, m0, k0, SEED, t0_, alg=ALG, tol_rel=TOL_REL, maxiter=MAXITER,
                                use_cache=not args.retune, grad_format="a24", residual_refresh=args.residual_refresh)
    kw = dict(lp=None, schedule=sched, gfmt=args.faithful_format)
    solve_step(sweep.rank_wave(0, 1, 0), **kw)  # warm-up: engines and graphs of this form
    ok = trials = 0
    kms = 0.0
    first = None
    for s_ in range(args.faithful_steps):
        w = sweep.rank_wave(0, 1, args.warmup + s_)
        r = solve_step(w, **kw)
        ok += r["ok"]
        trials += r["trials"]
        kms += r["kms"]
        if first is None:
            first = (w, r)
    value = ok / (kms / 1e3)
    out = {"value": value, "unit": "trials/s", "steps": args.faithful_steps, "recovered": int(ok), "trials": int(trials),
           "ms_per_step": kms / args.faithful_steps, "vs_plain": value / plain_value if plain_value else None,
           "form": "batched + shared-matrix forms, zero start, %s A^T r operand, residual recurrence every %d"
                   % ({"a24": "24-bit", "transition": "24-bit near the phase transition (|rho - rho*(delta)| <= "
                       "0.08 (1024/n)^0.3) and BF16 elsewhere"}[args.faithful_format], args.residual_refresh),
           "schedule": {"slots": sched["slots"], "sm_share": sched["sm_share"], "cluster": sched.get("cluster", 0)}}
    if pverd and first is not None and first[0] == pverd["w"]:
        tv = np.asarray(first[1]["verdict_batch"], bool)[pverd["sel"]]
        tv2 = np.asarray(first[1]["verdict_shared"], bool)[pverd["sel2"]]
        pv, pv2 = pverd["pv"], pverd["pv2"]
        agree = int(np.sum(pv == tv) + np.sum(pv2 == tv2))
        tot = len(pv) + len(pv2)
        out["verdict_agreement"] = agree / tot
        out["verdicts"] = {"trials": tot, "agree": agree,
                           "only_plain_recovers": int(np.sum(pv & ~tv) + np.sum(pv2 & ~tv2)),
                           "only_faithful_recovers": int(np.sum(tv & ~pv) + np.sum(tv2 & ~pv2))}
    return out


def bench_niht(args, solve_step):
    """The same sweep with NIHT (batched + shared-matrix forms, no warm start): the steps
    after the headline's, device time of both forms."""
    from gaga_gb300 import autotune

    n0, m0, k0, t0_ = wave_arrays(0)
    sched = autotune.tune_batch(n0, m0, k0, SEED, t0_, alg="NIHT", tol_rel=TOL_REL, maxiter=MAXITER,
                                use_cache=not args.retune)
    solve_step(PARTS - 1, alg="NIHT", lp=None, schedule=sched, gfmt="fp32")  # warm-up
    ok = trials = 0
    kms = kb = ks = 0.0
    for s in range(args.niht_steps):
        r = solve_step(s, alg="NIHT", lp=None, schedule=sched, gfmt="fp32")
        ok += r["ok"]
        trials += r["trials"]
        kms += r["kms"]
        kb += r["kms_batch"]
        ks += r["kms_shared"]
    return {"value": ok / (kms / 1e3), "unit": "trials/s", "steps": args.niht_steps, "recovered": int(ok),
            "trials": int(trials), "ms_per_step": kms / args.niht_steps,
            "independent_ms_per_step": kb / args.niht_steps, "shared_ms_per_step": ks / args.niht_steps,
            "schedule": {"slots": sched["slots"], "sm_share": sched["sm_share"], "cluster": sched.get("cluster", 0)}}


def bench_learned(args):
    """The learned warm start on its own workload: fresh dense Gaussian CGIHT trials with
    n = 8192, delta in [0.1, 0.6], rho in [0.05, 0.45], warm-started from the trained MLP
    (with the plain fallback) against zero-initialised CGIHT, both through the batched form."""
    from gaga_gb300 import learned

    res = learned.evaluate(learned.load_weights(), count=args.learned_trials)
    res["workload"] = "%d fresh CGIHT trials, n=8192, delta U[0.1,0.6], rho U[0.05,0.45], tol 1e-4*||y||" % (
        args.learned_trials)
    return res


def sweep_rank_first(rank, world):
    from gaga_gb300 import sweep

    return sweep.rank_wave(rank, world, 0)


def tensor_peak():
    """Dense BF16 tensor peak (TFLOP/s) for a kernel timed inside a long run."""
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        for key in ("bf16_tflops_sustained", "bf16_tflops"):
            if d.get(key):
                return float(d[key]), "measured (%s)" % key
    except (OSError, ValueError):
        pass
    return 1700.0, "fallback (sustained bf16 on an earlier GB300)"


def gemm_roofline(tpeak, tpeak_kind, M=4096, N=1024, K=3 * 8192, reps=10):
    """The shared-matrix form's residual GEMM ([A_hi|A_lo|A_hi] . X^T, the tcgen05 kernel
    unless GB_CS_GEMM=mma) on its full 1024-trial shape, timed with CUDA events on its stream."""
    import torch

    import gaga_gb300 as gb

    g = torch.Generator(device="cuda").manual_seed(2)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    Y = torch.randn(N, M, device="cuda", generator=g)
    s = torch.cuda.Stream()
    torch.cuda.synchronize()  # the operands come from torch's stream; s does not wait for it
    with torch.cuda.stream(s):
        for _ in range(3):
            gb.gemm_bf16_tn(A, B, Y=Y, want_bf16=True)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        for _ in range(reps):
            gb.gemm_bf16_tn(A, B, Y=Y, want_bf16=True)
        e1.record(s)
    e1.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / reps
    ach = 2.0 * M * N * K / t / 1e12
    del A, B, Y
    torch.cuda.empty_cache()
    mma = os.environ.get("GB_CS_GEMM") == "mma"
    single = os.environ.get("GB_CS_GEMM_PAIR") == "0" or M % 256 != 0
    kern = "k_gemm_tn_mma (mma.sync)" if mma else (
        "k_gemm_tn_tc<0> (tcgen05 cta_group::1 + TMA, 128x256 tiles)" if single else
        "k_gemm_tn_tc<1> (tcgen05 cta_group::2 on CTA pairs + TMA, 256x256 tiles)")
    out = {"bound": "tensor", "achieved": ach, "peak": tpeak, "unit": "TFLOP/s", "frac": ach / tpeak,
           "kernel": kern, "shape": "M=%d N=%d K=%d (bf16 in, fp32 accumulate, Y - AB^T epilogue)" % (
               M, N, K), "us_per_launch": t * 1e6, "peak_source": tpeak_kind, "traffic": None}
    key = "%s M=%d N=%d K=%d" % ("k_gemm_tn_mma" if mma else "k_gemm_tn_tc", M, N, K)
    tr = ncu_traffic()
    if key in tr:
        out["traffic"] = tr[key]["read"] + tr[key]["write"]
        out["traffic_unit"] = "bytes"
        out["traffic_source"] = "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, same shape " \
                                "(profiles/dram_traffic.json)"
    return out


def operators_roofline(peak, peak_kind, reps=20):
    """Every operator kernel at its workload's size with a cold L2 (a 256 MB buffer is
    overwritten before each application, outside the CUDA events), and again back to back
    with a warm L2 (`us_per_launch_warm_l2`): the dense operator at the
    single-trial NIHT size (n=4096, m=1024) and the sweep's largest trial, the subsampled DCT at
    n=2^20, m=2^18 and the expander at n=2^18, m=2^16, d=7, and each of the last two also at
    n=2^22 (working set well above L2).  Algorithmic bytes per
    application: dense A^T r 4mn+4m+4n, A x 4mn+4n+4m; DCT A or A^T 4n+8m; expander A^T r
    b nd+4m+4n (b = 2-byte row indices when m <= 65536, else 4; the values are all equal and
    not streamed), A x 4nd+4(m+1)+4n+4m (column indices, row pointers, x, y); the int32 +
    fp32 layout's 8nd-based figures are kept beside them."""
    import ctypes as C

    import torch

    import gaga_gb300 as gb
    from gaga_gb300 import _lib

    L = gb._lib.load()
    g = torch.Generator(device="cuda").manual_seed(3)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    out = {}

    def one(name, p, m, n, tr, nbytes, what):
        vin = torch.randn(m if tr else n, device="cuda", generator=g)
        vout = torch.empty(n if tr else m, device="cuda")
        torch.cuda.synchronize()  # the inputs come from torch's stream; s does not wait for it
        p.stream = C.c_void_p(s.cuda_stream)
        ms = C.c_float(0)
        _lib.check(L.gb_cs_operator_time(C.byref(p), tr, vin.data_ptr(), vout.data_ptr(), 3, reps, flush.data_ptr(),
                                         flush.numel(), C.byref(ms)))
        t = ms.value / 1e3
        ach = nbytes / t / 1e9
        # the same applications back to back without the flush: a working set that fits in L2
        # (the DCT's and the expander's at these sizes) stays there, as it does inside a solve
        msw = C.c_float(0)
        _lib.check(L.gb_cs_operator_time(C.byref(p), tr, vin.data_ptr(), vout.data_ptr(), 3, reps, None, 0,
                                         C.byref(msw)))
        out[name] = {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "us_per_launch": t * 1e6,
                     "us_per_launch_warm_l2": msw.value * 1e3,
                     "shape": what, "bytes": nbytes, "l2": "cold (flushed before each application)",
                     "peak_source": peak_kind}

    for (m, n) in ((1024, 4096), (14746, 16384)):
        lda = (m + 31) // 32 * 32  # the library's own layout: 128-byte aligned columns
        A = torch.randn(n * lda, device="cuda", generator=g) / np.sqrt(m)
        p = _lib.Problem(_lib.GB_OP_DENSE, m, n, 0, None, A.data_ptr(), lda, None, None, None, 0, 0, _lib.GB_DEVICE,
                         None)
        one("dense_at_n%d" % n, p, m, n, 1, 4.0 * m * n + 4 * m + 4 * n, "k_dense_at m=%d n=%d" % (m, n))
        one("dense_ax_n%d" % n, p, m, n, 0, 4.0 * m * n + 4 * n + 4 * m, "k_dense_av m=%d n=%d, full x" % (m, n))
        if n == 16384:  # the batched form's compact A^T r operands (3 and 2 bytes per entry)
            one("dense_at_a24_n%d" % n, p, m, n, 2, 3.0 * m * n + 4 * m + 4 * n,
                "k_dense_at_c<1> m=%d n=%d, A rounded to 24 bits" % (m, n))
            one("dense_at_bf16_n%d" % n, p, m, n, 3, 2.0 * m * n + 4 * m + 4 * n,
                "k_dense_at_c<0> m=%d n=%d, A rounded to BF16" % (m, n))
        del A
    for ln in (20, 22):
        n, m = 2 ** ln, 2 ** (ln - 2)
        rows = torch.randperm(n, device="cuda", generator=g)[:m].to(torch.int32)
        p = _lib.Problem(_lib.GB_OP_DCT, m, n, 0, None, None, 0, rows.data_ptr(), None, None, 0, 0, _lib.GB_DEVICE,
                         None)
        one("dct_at_n2^%d" % ln, p, m, n, 1, 4.0 * n + 8 * m,
            "k_dct_scatter + 2 k_dct_pass (n/2-point transform), n=2^%d m=n/4" % ln)
        one("dct_a_n2^%d" % ln, p, m, n, 0, 4.0 * n + 8 * m,
            "2 k_dct_pass (n/2-point transform) + k_dct_select_half, n=2^%d m=n/4" % ln)
    for ln in (18, 22):
        n, m, d = 2 ** ln, 2 ** (ln - 2), 7
        rows = torch.randint(0, m, (n * d,), device="cuda", generator=g, dtype=torch.int32)
        vals = torch.full((n * d,), 1.0 / np.sqrt(d), device="cuda")
        p = _lib.Problem(_lib.GB_OP_SMV, m, n, 0, None, None, 0, rows.data_ptr(), None, vals.data_ptr(), d, 0,
                         _lib.GB_DEVICE, None)
        # the kernels' own layout: one value for all entries (none streamed), row indices of
        # 2 bytes when m <= 65536 (A^T), column indices of 4 bytes plus the row pointers (A)
        ib = 2 if m <= 65536 else 4
        one("smv_at_n2^%d" % ln, p, m, n, 1, float(ib * n * d + 4 * m + 4 * n),
            "k_smv_AT n=2^%d m=n/4 d=7, values 1/sqrt(d), %d-byte row indices" % (ln, ib))
        out["smv_at_n2^%d" % ln]["bytes_int32_fp32_layout"] = 8.0 * n * d + 4 * m + 4 * n
        one("smv_a_n2^%d" % ln, p, m, n, 0, float(4 * n * d + 4 * (m + 1) + 4 * n + 4 * m),
            "k_smv_A n=2^%d m=n/4 d=7, values 1/sqrt(d), full x" % ln)
        out["smv_a_n2^%d" % ln]["bytes_int32_fp32_layout"] = 8.0 * n * d + 4 * n + 4 * m
    del flush
    torch.cuda.empty_cache()
    return out


def matvec_roofline(peak, peak_kind, m=14746, n=16384, k=5000, reps=20, grad_format="fp32"):
    """Dense A^T r (k_dense_at) and A x_S (k_dense_av) on the sweep's largest trial shape,
    timed with CUDA events on the stream they run on; with a compact A^T r operand also
    k_dense_at_c (the tuned form's A^T r, "at_c": CUDA events inside gb_cs_operator_time)."""
    import ctypes as C

    import torch

    import gaga_gb300 as gb
    from gaga_gb300 import _lib

    L = gb._lib.load()
    g = torch.Generator(device="cuda").manual_seed(1)
    lda = (m + 31) // 32 * 32  # the library's own layout: 128-byte aligned columns
    A = torch.randn(n * lda, device="cuda", generator=g) / np.sqrt(m)  # column-major
    r = torch.randn(m, device="cuda", generator=g)
    x = torch.zeros(n, device="cuda")
    x[torch.randperm(n, device="cuda", generator=g)[:k]] = 1.0
    g_out, y_out = torch.empty(n, device="cuda"), torch.empty(m, device="cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()  # the inputs come from torch's stream; s does not wait for it
    res = {}
    # A x_S is timed on a fixed support (transpose 2: the support scan of the first call is
    # reused), so the events bracket the k_dense_av launches alone
    for name, tr, vin, vout, nbytes in (("at", 1, r, g_out, 4.0 * m * n + 4 * m + 4 * n),
                                        ("av", 2, x, y_out, 4.0 * m * k + 8 * k + 4 * m)):
        with torch.cuda.stream(s):
            if tr == 2:
                _lib.check(L.gb_cs_dense_apply_noalloc(A.data_ptr(), lda, m, n, 0, vin.data_ptr(), vout.data_ptr(),
                                                       C.c_void_p(s.cuda_stream)))
            for _ in range(3):
                _lib.check(L.gb_cs_dense_apply_noalloc(A.data_ptr(), lda, m, n, tr, vin.data_ptr(), vout.data_ptr(),
                                                       C.c_void_p(s.cuda_stream)))
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.synchronize()
            e0.record(s)
            for _ in range(reps):
                _lib.check(L.gb_cs_dense_apply_noalloc(A.data_ptr(), lda, m, n, tr, vin.data_ptr(), vout.data_ptr(),
                                                       C.c_void_p(s.cuda_stream)))
            e1.record(s)
        e1.synchronize()
        t = e0.elapsed_time(e1) / 1e3 / reps
        ach = nbytes / t / 1e9
        res[name] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                     "traffic": None, "kernel": "k_dense_at" if name == "at" else "k_dense_av",
                     "shape": "m=%d n=%d lda=%d%s, A %.0f MB > L2" % (m, n, lda, "" if name == "at" else
                                                                      " |S|=%d" % k, 4.0 * m * n / 1e6),
                     "us_per_launch": t * 1e6, "peak_source": peak_kind}
    if grad_format != "fp32":
        code = {"a24": 2, "bf16": 3}[grad_format]
        b = {"a24": 3.0, "bf16": 2.0}[grad_format]
        p = _lib.Problem(_lib.GB_OP_DENSE, m, n, 0, None, A.data_ptr(), lda, None, None, None, 0, 0, _lib.GB_DEVICE,
                         None)
        p.stream = C.c_void_p(s.cuda_stream)
        ms = C.c_float(0)
        _lib.check(L.gb_cs_operator_time(C.byref(p), code, r.data_ptr(), g_out.data_ptr(), 3, reps, None, 0,
                                         C.byref(ms)))
        t = ms.value / 1e3
        ach = (b * m * n + 4 * m + 4 * n) / t / 1e9
        res["at_c"] = {"bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak,
                       "traffic": None, "kernel": "k_dense_at_c<%d>" % (1 if grad_format == "a24" else 0),
                       "shape": "m=%d n=%d lda=%d, %s A^T r operand %.0f MB > L2" % (
                           m, n, lda, grad_format, b * m * n / 1e6),
                       "us_per_launch": t * 1e6, "peak_source": peak_kind}
    del A
    torch.cuda.empty_cache()
    tr = ncu_traffic()
    if "at_c" in res:
        key = ("k_dense_at_c<0> (BF16 operand) m=14746 n=16384 lda=14752" if grad_format == "bf16" else
               "k_dense_at_c<1> (24-bit operand) m=14746 n=16384 lda=14752")
        if key in tr and (m, n) == (14746, 16384):
            res["at_c"]["traffic"] = tr[key]["read"] + tr[key]["write"]
            res["at_c"]["traffic_source"] = "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, same " \
                                            "shape (profiles/dram_traffic.json)"
    for name, key in (("at", "k_dense_at m=14746 n=16384 lda=14752"), ("av", "k_dense_av m=14746 n=16384 lda=14752 |S|=5000")):
        if key in tr and (m, n, k) == (14746, 16384, 5000):
            res[name]["traffic"] = tr[key]["read"] + tr[key]["write"]
            res[name]["traffic_source"] = "ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, same shape " \
                                          "(profiles/dram_traffic.json)"
    return res


def resident_roofline(peak, peak_kind, max_n=8192, sample=0, cluster=0, alg="NIHT", learned_params=None,
                      grad_format="fp32", residual_refresh=0):
    """The cluster-resident kernel alone (k_resident, one launch; NIHT, or the tuned form's
    instance: CGIHT from the learned start with its A^T r operand and residual recurrence)
    on the first wave's trials with n <= max_n (every one, or `sample` evenly spaced), timed
    with CUDA events around the batched call; algorithmic operator bytes of its iterations
    per second.  Trials whose slab of A fits in L2 re-read it from there, so the DRAM
    traffic can be below the algorithmic bytes."""
    import gaga_gb300 as gb

    n, m, k, tid = wave_arrays(0)
    sel = np.flatnonzero(n <= max_n)
    if sample:
        sel = sel[np.linspace(0, len(sel) - 1, min(sample, len(sel))).astype(int)]
    n, m, k, tid = n[sel], m[sel], k[sel], tid[sel]
    for _ in range(2):  # the first call sizes the kernel's buffers
        ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg=alg, tol_rel=TOL_REL, maxiter=MAXITER,
                                            resident_n=max_n, cluster=cluster, learned_params=learned_params,
                                            grad_format=grad_format, residual_refresh=residual_refresh)
    nbytes, ms = gb.batch_last_stats()
    achieved = nbytes / (ms / 1e3) / 1e9
    what = "k_resident<%s%s%s>" % (alg, ", learned start" if learned_params is not None else "",
                                   "" if grad_format == "fp32" else ", %s A^T r operand" % grad_format)
    out = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
           "kernel": what, "trials": int(len(n)), "recovered": int(ns), "iterations": int(iters.sum()),
           "sizes": "n=%s" % sorted(set(n.tolist())), "ms": ms, "algorithmic_bytes": nbytes,
           "cluster": gb._lib.load().gb_cs_batch_last_cluster(), "peak_source": peak_kind}
    tr = ncu_traffic().get("k_resident<NIHT> sweep wave 0, 655 trials n=1024..8192, 4 CTAs per cluster")
    if tr and not sample and max_n == 8192 and out["cluster"] == 4 and alg == "NIHT":
        out["traffic"] = tr["read"] + tr["write"]
        out["traffic_unit"] = "bytes"
        out["traffic_source"] = "ncu dram__bytes_read.sum + dram__bytes_write.sum of the same launch " \
                                "(profiles/dram_traffic.json)"
    return out


# The reference's single-trial configurations (dense, DCT, expander), each through the drop-in
# generate-and-solve call: (name, algorithm, operator, k, m, n, d, options, seed)
SINGLE_CONFIGS = (
    ("dense NIHT n=4096 m=1024 k=102", "NIHT", "gen", 102, 1024, 4096, 0, (), 101),
    ("DCT CGIHT n=2^20 m=2^18 k=26214", "CGIHT", "dct", 26214, 2 ** 18, 2 ** 20, 0, ("vecDistribution", "gaussian"), 202),
    ("DCT HTP n=2^20 m=2^18 k=26214", "HTP", "dct", 26214, 2 ** 18, 2 ** 20, 0, ("vecDistribution", "gaussian"), 203),
    ("expander NIHT n=2^18 m=2^16 d=7 k=3276", "NIHT", "smv", 3276, 2 ** 16, 2 ** 18, 7, ("matrixEnsemble", "ones"), 303),
    ("expander parallel_l0 n=2^18 m=2^16 d=7 k=3276", "parallel_l0", "smv", 3276, 2 ** 16, 2 ** 18, 7,
     ("matrixEnsemble", "expander"), 304),
)


def bench_configs(cpu=True, cpu_iters=3, only=None):
    """Each single-trial configuration solved by the drop-in on the GPU (generation included
    in `ms_total`, the solve alone in `ms_algorithm`, the library's own events), and the CPU
    oracle's time per iteration on the same problem (regenerated from the same keys by the
    oracle's generators; at most `cpu_iters` iterations, all of them for the dense case,
    OpenMP over the host cores)."""
    import gaga_gb300 as gb

    out = {}
    for name, alg, ens, k, m, n, d, extra, seed in SINGLE_CONFIGS:
        if only and only not in name:
            continue
        opts = gb.gaga_options("tol", TOL_REL, "tol_is_relative", 1, "maxiter", MAXITER, "seed", seed, *extra)
        for _ in range(2):  # the first call loads the kernels
            t0 = time.perf_counter()
            x, xt, r = gb.generate_and_solve(alg, ens, k, m, n, d, opts)
            wall = time.perf_counter() - t0
        rec = {"algorithm": alg, "iterations": int(r.iter), "rel_l2": float(r.norms[1]),
               "recovered": bool(r.norms[1] <= 1e-3), "ms_algorithm": float(r.times[0]),
               "ms_per_iteration": float(r.times[0]) / max(1, int(r.iter)), "ms_total": float(r.times[2]),
               "wall_ms": wall * 1e3}
        if cpu:
            rec["cpu"] = _config_cpu(alg, ens, k, m, n, d, dict(zip(extra[::2], extra[1::2])), seed, int(r.iter),
                                     cpu_iters)
            rec["cpu_vs_gpu_per_iteration"] = rec["cpu"]["ms_per_iteration"] / rec["ms_per_iteration"]
        out[name] = rec
    return out


def _config_cpu(alg, ens, k, m, n, d, extra, seed, gpu_iters, cpu_iters):
    """CPU oracle timing of one single-trial configuration (the problem regenerated on the host)."""
    import os

    from oracle import gbo

    vec = {"uniform": 0, "binary": 1, "gaussian": 2}[extra.get("vecDistribution", "binary")]
    x0, ks = gbo.gen_vector(n, k, vec, seed)
    if ens == "gen":
        op = gbo.Op.dense(gbo.gen_dense(m, n, seed, 0, 1), m, n)
    elif ens == "dct":
        op = gbo.Op.dct(n, gbo.gen_dct_rows(n, m, seed))
    else:
        ensn = {"ones": 1, "binary": 2, "expander": 3}[extra.get("matrixEnsemble", "ones")]
        rows, vals = gbo.gen_smv(m, n, d, ensn, seed)
        op = gbo.Op.smv(m, n, d, rows, vals)
    y = gbo.A(op, x0)
    tol = TOL_REL * float(np.linalg.norm(y))
    iters = gpu_iters if ens == "gen" else max(1, min(cpu_iters, gpu_iters))
    t0 = time.perf_counter()
    if alg == "parallel_l0":
        _, _, _, info = gbo.parallel_l0(op, y, tol, iters)
    else:
        _, info = gbo.solve(alg, op, y, ks, tol, maxiter=iters)
    t = time.perf_counter() - t0
    return {"ms_per_iteration": t * 1e3 / max(1, int(info.iter)), "iterations_timed": int(info.iter),
            "cores": os.cpu_count(), "kind": "port"}


def ncu_traffic():
    """Per-launch DRAM bytes of the dense kernels from the committed ncu summary."""
    try:
        with open(os.path.join(ROOT, "profiles", "dram_traffic.json")) as f:
            return json.load(f)["per_launch_dram_bytes"]
    except (OSError, ValueError, KeyError):
        return {}


def bench_plain(args, first_step, verdicts_out=None):
    """Single-trial FP32 drop-in, zero-initialised CGIHT, on the first timed step's trials:
    the independent trials by gb_cs_generate_and_solve (same seeds, so the same problems),
    the shared-matrix trials by gb_cs_solve on the shared A and the trial's y.  Each call is
    timed with CUDA events on the stream it runs on (per-call setup included, as a caller of
    the drop-in sees it; its solver time alone is reported too).  The rate is scaled to the
    3072 + 1024 mix; verdicts are compared with the tuned form's on the same trials."""
    import torch

    import gaga_gb300 as gb

    w, r = first_step
    n, m, k, tid = wave_arrays(w)
    cnt = args.plain_trials
    sel = np.linspace(0, len(n) - 1, min(cnt, len(n))).astype(int)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        ev0.record()
        out = fn()
        ev1.record()
        ev1.synchronize()
        return out, ev0.elapsed_time(ev1)

    def count(pv, tv):
        pv, tv = np.asarray(pv, bool), np.asarray(tv, bool)
        return {"agree": int(np.sum(pv == tv)), "only_plain": int(np.sum(pv & ~tv)), "only_tuned": int(np.sum(tv & ~pv))}

    pv, tv, t_call, t_solver = [], [], 0.0, 0.0
    for i in sel:
        opts = gb.gaga_options("tol", TOL_REL, "tol_is_relative", 1, "maxiter", MAXITER, "seed", int(SEED + tid[i]))
        (x, xt, res), ms = timed(lambda: gb.generate_and_solve(ALG, "gen", int(k[i]), int(m[i]), int(n[i]), 0, opts))
        t_call += ms
        t_solver += res.times[0]
        pv.append(res.norms[1] <= 1e-3)
        tv.append(bool(r["verdict_batch"][i]))
    t_ind, ts_ind = t_call / 1e3 / len(sel), t_solver / 1e3 / len(sel)
    ok_ind = float(np.mean(pv))
    c_ind = count(pv, tv)
    # shared-matrix trials: regenerate the step's problems (same keys) to get A and y
    ks, first = shared_part(w)
    _, _, _, _, A, Y, X0 = gb.solve_shared_batch(gb.sweep.SHARED_M, gb.sweep.SHARED_N, ks, SHARED_SEED,
                                                 tol_rel=TOL_REL, maxiter=MAXITER, first_trial=first, outputs=True,
                                                 alg=ALG)
    torch.cuda.synchronize()
    X0h = X0.cpu().numpy()
    At = A.t()
    sel2 = np.linspace(0, len(ks) - 1, min(len(ks), max(4, cnt // 3))).astype(int)
    pv2, tv2, tt = [], [], 0.0
    for t in sel2:
        kt = int(np.count_nonzero(X0h[t]))
        opts = gb.gaga_options("tol", TOL_REL, "tol_is_relative", 1, "maxiter", MAXITER)
        yt = Y[t].contiguous()
        (x, it, _), ms = timed(lambda: gb.gaga_cs(ALG, "gen", yt, At, kt, opts))
        tt += ms
        pv2.append(np.linalg.norm(x.cpu().numpy() - X0h[t]) / np.linalg.norm(X0h[t]) <= 1e-3)
        tv2.append(bool(r["verdict_shared"][t]))
    t_sh = tt / 1e3 / len(sel2)
    ok_sh = float(np.mean(pv2))
    c_sh = count(pv2, tv2)
    n_ind, n_sh = TOTAL - SHARED, SHARED
    est_time = n_ind * t_ind + n_sh * t_sh
    est_ok = n_ind * ok_ind + n_sh * ok_sh
    tot = len(sel) + len(sel2)
    if verdicts_out is not None:
        verdicts_out.update(sel=sel, pv=np.asarray(pv, bool), sel2=sel2, pv2=np.asarray(pv2, bool), w=w)
    return {"value": est_ok / est_time, "unit": "trials/s", "algorithm": ALG + " (zero-initialised)",
            "timing": "CUDA events around each call on its stream",
            "independent": {"trials": int(len(sel)), "s_per_trial": t_ind, "solver_s_per_trial": ts_ind,
                            "recovered_frac": ok_ind, "verdicts": c_ind},
            "shared_matrix": {"trials": int(len(sel2)), "s_per_trial": t_sh, "recovered_frac": ok_sh,
                              "verdicts": c_sh},
            "verdict_agreement": (c_ind["agree"] + c_sh["agree"]) / tot,
            "verdicts": {"trials": tot, "agree": c_ind["agree"] + c_sh["agree"],
                         "only_plain_recovers": c_ind["only_plain"] + c_sh["only_plain"],
                         "only_tuned_recovers": c_ind["only_tuned"] + c_sh["only_tuned"]},
            "sample": "%d independent + %d shared-matrix trials of step %d; rate = estimated recovered / estimated "
                      "time of the 3072 + 1024 sweep" % (len(sel), len(sel2), w)}


def size_classes(args):
    """The independent trials of one step (step --warmup) by size class, in the tuned form
    (learned start, the --grad-format operand) and the faithful form (zero start,
    transition-aware operand), both with the residual recurrence: device time (best of two
    calls) and algorithmic operator bytes per second of each class alone and of the whole
    wave, at the tuned schedule of the bench (--slots / --sm-share / --cluster)."""
    import gaga_gb300 as gb
    from gaga_gb300 import transition

    lp = gb.learned.load_weights()
    n0, m0, k0, t0 = wave_arrays(args.warmup)
    sel = [("all", n0 > 0), ("n=16384", n0 == 16384), ("n<=8192", n0 <= 8192)]
    sel += [("n=%d" % v, n0 == v) for v in (1024, 2048, 4096, 8192)]
    out = {"step": args.warmup, "schedule": {"slots": args.slots, "sm_share": args.sm_share, "cluster": args.cluster}}
    for form in ("tuned", "faithful"):
        rows = {}
        for name, s in sel:
            n, m, k, tid = n0[s], m0[s], k0[s], t0[s]
            if form == "tuned":
                kw = dict(learned_params=lp, grad_format=args.grad_format)
            else:
                kw = dict(grad_format="a24", grad_formats=transition.operand_formats(n, m, k))
            best = None
            for _ in range(2):
                ns, it, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg=ALG, tol_rel=TOL_REL, maxiter=MAXITER,
                                                 slots=args.slots, sm_share=args.sm_share, cluster=args.cluster,
                                                 residual_refresh=args.residual_refresh, **kw)
                nb, ms = gb.batch_last_stats()
                best = (ms, nb) if best is None or ms < best[0] else best
            rows[name] = {"trials": int(len(n)), "recovered": int(ns), "iterations": int(np.sum(it)),
                          "max_iterations": int(np.max(it)), "ms": best[0], "gbs": best[1] / best[0] / 1e6}
        out[form] = rows
    return out


def shared_part_alone(args):
    """The shared-matrix trials of one step (step --warmup) alone, in the tuned form (learned
    start) or, with --shared-zero, from the zero start: device time of each of two calls."""
    import gaga_gb300 as gb

    lp = None if args.shared_zero else gb.learned.load_weights()
    ks, first = shared_part(args.warmup)
    runs = []
    for _ in range(2):
        ns, it, err, ok = gb.solve_shared_batch(gb.sweep.SHARED_M, gb.sweep.SHARED_N, ks, SHARED_SEED, tol_rel=TOL_REL,
                                                maxiter=MAXITER, first_trial=first, alg=ALG, learned_params=lp)
        runs.append(gb.shared_last_stats()[1])
    return {"trials": int(len(ks)), "recovered": int(ns), "iterations": int(np.sum(it)), "max_iterations": int(np.max(it)),
            "ms": runs, "start": "zero" if args.shared_zero else "learned"}


def bench_only(args):
    import torch

    import gaga_gb300 as gb

    gb._lib.load()
    torch.cuda.set_device(0)
    if args.only == "matvec":
        out = matvec_roofline(*peaks())
    elif args.only == "gemm":
        out = gemm_roofline(*tensor_peak())
    elif args.only == "operators":
        out = operators_roofline(*peaks())
    elif args.only == "learned":
        out = bench_learned(args)
    elif args.only == "configs":
        out = bench_configs(cpu=not args.no_cpu, only=args.config)
    elif args.only == "resident":
        out = resident_roofline(*peaks(), max_n=args.resident_max_n, sample=args.resident_sample)
    elif args.only == "shared":
        out = shared_part_alone(args)
    elif args.only == "classes":
        out = size_classes(args)
    else:
        w = args.warmup
        n, m, k, tid = wave_arrays(w)
        lp = gb.learned.load_weights()
        ns, iters, err, ok = gb.solve_batch(n, m, k, SEED, tid, alg=ALG, tol_rel=TOL_REL, maxiter=MAXITER,
                                            learned_params=lp, grad_format=args.grad_format,
                                            residual_refresh=args.residual_refresh)
        ks, first = shared_part(w)
        _, _, _, ok2 = gb.solve_shared_batch(gb.sweep.SHARED_M, gb.sweep.SHARED_N, ks, SHARED_SEED, tol_rel=TOL_REL,
                                             maxiter=MAXITER, first_trial=first, alg=ALG, learned_params=lp)
        out = bench_plain(args, (w, {"verdict_batch": ok, "verdict_shared": ok2}))
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--plain-trials", type=int, default=768,
                    help="independent trials of the first timed step solved by the plain form (768 = all); a third "
                         "as many shared-matrix trials (256 = all)")
    ap.add_argument("--niht-steps", type=int, default=2, help="steps of the NIHT sweep leg (0: skip)")
    ap.add_argument("--faithful-steps", type=int, default=3,
                    help="steps of the verdict-faithful leg (zero start, 24-bit A^T r operand; 0: skip)")
    ap.add_argument("--faithful-format", default="transition", choices=["a24", "transition"],
                    help="the verdict-faithful leg's A^T r operand: 24-bit for every trial, or 24-bit near the "
                         "phase transition and BF16 elsewhere (gaga_gb300/transition.py)")
    ap.add_argument("--cpu-trials", type=int, default=32)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--learned-trials", type=int, default=2048)
    ap.add_argument("--retune", action="store_true", help="ignore the autotuner's cache")
    ap.add_argument("--resident-max-n", type=int, default=8192, help="--only resident: largest trial n")
    ap.add_argument("--resident-sample", type=int, default=0, help="--only resident: trials (0: all)")
    ap.add_argument("--no-configs", action="store_true", help="skip the single-trial configurations")
    ap.add_argument("--grad-format", default="bf16", choices=["fp32", "a24", "bf16"],
                    help="the tuned form's A^T r operand for the independent trials: FP32 A, A rounded to 24 bits "
                         "(3 bytes per entry) or to BF16 (2 bytes); A x, the residual and the stopping test stay FP32")
    ap.add_argument("--residual-refresh", type=int, default=8,
                    help="the tuned form's CGIHT residual recurrence: y - A x every N-th restricted step on an "
                         "unchanged support, r - alpha A p between (0: y - A x at every step)")
    ap.add_argument("--config", default=None,
                    help="--only configs: run the configurations whose name contains this text")
    ap.add_argument("--shared-zero", action="store_true", help="--only shared: from the zero start")
    ap.add_argument("--slots", type=int, default=24, help="--only classes: slot graphs")
    ap.add_argument("--sm-share", type=int, default=76, help="--only classes: SMs per slot's kernels")
    ap.add_argument("--cluster", type=int, default=8, help="--only classes: CTAs per resident cluster")
    ap.add_argument("--only", choices=["matvec", "gemm", "operators", "plain", "learned", "resident", "configs", "shared",
                                       "classes"],
                    help="run one measurement alone and print its JSON (for profiling)")
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.only:
        bench_only(args)
    elif args.impl == "reference":
        bench_reference(args)
    else:
        bench_ours(args)


if __name__ == "__main__":
    main()
