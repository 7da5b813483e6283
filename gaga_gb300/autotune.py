"""Autotuner for the batched form's schedule.

The batched form (gb_cs_solve_batch) runs `slots` trials at a time in slot graphs, each
slot's kernels shaped for `sm_share` SMs (the dense A^T r grid is 4 CTAs per shared SM, the
reductions one CTA per shared SM, and the A x_S row tiles x support splits fill whole waves
of that many SMs), while trials with n <= 8192 go to the cluster-resident kernel with
`cluster` CTAs per trial.  The probe runs the form the caller will run (algorithm, learned
warm start, A^T r operand format).  Which combination is fastest depends on the GPU and on the mix of
trial sizes, so it is measured: every candidate solves the same probe subset of the workload
(every `stride`-th trial, all trial sizes represented), the second run of each is timed on
the device, and the fastest candidate wins.  Results are cached per GPU, algorithm and trial-size mix in a JSON
file (GB_CS_TUNE_CACHE, default ~/.cache/gaga_gb300/autotune.json).
"""
import json
import os

import numpy as np

SLOTS = (8, 16, 24)
SHARE_FRACTIONS = (0.25, 0.5)
# CTAs per cluster of the resident kernel.  Alone, its CGIHT trials run much faster with 8
# (n <= 8192 of one sweep wave on GB300: 673 vs 1072 ms) because 4 CTAs leave the n = 8192
# trials latency-bound; next to the slot graphs, where the whole GPU's HBM bandwidth is the
# limit, both take the same time (1998 ms per wave).  A probe holds a quarter of the trials,
# so the longest trial weighs more there than in a whole wave.
CLUSTERS = (4, 8)
# the slot graphs' A x_S row tile, tried at the best schedule (256-row tiles read 1 KB of a
# column per warp instead of 512 B, with half the tiles and half the resident CTAs)
AV_ROWS = (128, 256)


def _cache_path():
    return os.environ.get("GB_CS_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "gaga_gb300", "autotune.json"))


def _key(alg, n, m, form=""):
    import torch

    name = torch.cuda.get_device_name()
    sizes = sorted(set(zip(np.asarray(n).tolist(), np.asarray(m).tolist())))
    h = hash(tuple(sizes)) & 0xFFFFFFFF
    return "%s|%s%s|%d sizes|%08x" % (name, alg, form, len(sizes), h)


def tune_batch(n, m, k, seed, trial_ids=None, alg="NIHT", tol_rel=1e-4, maxiter=5000, stride=4, use_cache=True,
               slots=SLOTS, fractions=SHARE_FRACTIONS, clusters=CLUSTERS, log=None, learned_params=None,
               grad_format="fp32", residual_refresh=0, av_rows_candidates=AV_ROWS):
    """Pick (slots, sm_share, cluster), then the A x_S row tile, for solving trials like
    (n, m, k) with the given form; returns a dict with the choice and the measured device
    milliseconds of every candidate on the probe."""
    import torch

    import gaga_gb300 as gb

    n, m, k = (np.asarray(a, dtype=np.int32) for a in (n, m, k))
    tid = np.arange(len(n), dtype=np.uint32) if trial_ids is None else np.asarray(trial_ids, dtype=np.uint32)
    key = _key(alg, n, m, "%s|%s|r%d|v2" % ("learned" if learned_params is not None else "plain", grad_format,
                                             residual_refresh))
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            return dict(cache[key], cached=True)
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    # the probe: every stride-th trial in descending size order, so every size class appears
    order = np.argsort(-(n.astype(np.int64) * m), kind="stable")
    probe = np.sort(order[::stride])
    pn, pm, pk, pt = n[probe], m[probe], k[probe], tid[probe]
    table = []
    for c in clusters:
        for s in slots:
            for fr in fractions:
                share = max(1, int(round(sms * fr)))
                for rep in range(2):  # the first run builds the engine and its graphs
                    ns, it, err, ok = gb.solve_batch(pn, pm, pk, seed, pt, alg=alg, tol_rel=tol_rel,
                                                     maxiter=maxiter, slots=s, sm_share=share, cluster=c,
                                                     learned_params=learned_params, grad_format=grad_format,
                                                     residual_refresh=residual_refresh)
                _, ms = gb.batch_last_stats()
                table.append({"slots": s, "sm_share": share, "cluster": c, "ms": ms, "recovered": int(ns)})
                if log:
                    log(json.dumps(table[-1]))
    best = min(table, key=lambda r: r["ms"])
    # second stage, at the best schedule: the slot graphs' A x_S row tile (128 or 256 rows)
    best = dict(best, av_rows=128)
    if av_rows_candidates:
        for rows in av_rows_candidates:
            if rows == 128:
                continue
            for rep in range(2):
                ns, it, err, ok = gb.solve_batch(pn, pm, pk, seed, pt, alg=alg, tol_rel=tol_rel, maxiter=maxiter,
                                                 slots=best["slots"], sm_share=best["sm_share"],
                                                 cluster=best["cluster"], learned_params=learned_params,
                                                 grad_format=grad_format, residual_refresh=residual_refresh,
                                                 av_rows=rows)
            _, ms = gb.batch_last_stats()
            row = {"slots": best["slots"], "sm_share": best["sm_share"], "cluster": best["cluster"], "av_rows": rows,
                   "ms": ms, "recovered": int(ns)}
            table.append(row)
            if log:
                log(json.dumps(row))
            if ms < best["ms"]:
                best = row
    res = {"slots": best["slots"], "sm_share": best["sm_share"], "cluster": best["cluster"],
           "av_rows": best.get("av_rows", 128), "probe_trials": int(len(probe)), "candidates": table, "key": key}
    if use_cache:
        cache[key] = res
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return dict(res, cached=False)
