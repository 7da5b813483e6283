"""The batched form's autotuner as host logic: the candidate grid, the probe subset, the
second stage (the A x_S row tile) and the per-form cache, with the device calls replaced by
a fake whose timings the test chooses (no GPU)."""
import json

import numpy as np
import pytest


@pytest.fixture
def fake_device(monkeypatch, tmp_path):
    torch = pytest.importorskip("torch")
    import gaga_gb300 as gb

    calls = []
    state = {"ms": 0.0, "tile256": 0.95}

    def cost(slots, share, cluster, av_rows):
        # fastest at 16 slots, half the SMs, 8 CTAs per cluster; 256-row tiles scaled by
        # state["tile256"] (5% faster unless a test changes it)
        ms = 100.0 + abs(slots - 16) + abs(share - 76) * 0.1 + (0.0 if cluster == 8 else 3.0)
        return ms * (state["tile256"] if av_rows == 256 else 1.0)

    def solve_batch(n, m, k, seed, trial_ids=None, slots=0, sm_share=0, cluster=0, av_rows=0, **kw):
        calls.append({"n": np.asarray(n).tolist(), "m": np.asarray(m).tolist(), "slots": slots, "sm_share": sm_share,
                      "cluster": cluster, "av_rows": av_rows, "kw": sorted(kw)})
        state["ms"] = cost(slots, sm_share, cluster, av_rows or 128)
        ok = np.ones(len(n), dtype=np.int32)
        return len(n), np.ones(len(n), dtype=np.int32), np.zeros(len(n), dtype=np.float32), ok

    class Props:
        multi_processor_count = 152

    monkeypatch.setattr(gb, "solve_batch", solve_batch)
    monkeypatch.setattr(gb, "batch_last_stats", lambda: (1.0, state["ms"]))
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda *a: "FAKE GB300")
    monkeypatch.setattr(torch.cuda, "current_device", lambda: 0)
    monkeypatch.setattr(torch.cuda, "get_device_properties", lambda *a: Props())
    monkeypatch.setenv("GB_CS_TUNE_CACHE", str(tmp_path / "tune.json"))
    return calls, tmp_path / "tune.json", state


def _workload():
    n = np.repeat([1024, 2048, 4096, 8192, 16384], 12).astype(np.int32)
    m = (n // 2).astype(np.int32)
    k = (m // 10).astype(np.int32)
    return n, m, k


def test_autotune_picks_the_fastest_candidate_then_the_row_tile(fake_device):
    from gaga_gb300 import autotune

    calls, _, _ = fake_device
    n, m, k = _workload()
    res = autotune.tune_batch(n, m, k, 7, alg="CGIHT", stride=4, grad_format="bf16", residual_refresh=8)
    assert (res["slots"], res["sm_share"], res["cluster"], res["av_rows"]) == (16, 76, 8, 256)
    assert res["cached"] is False
    # every (cluster, slots, share) candidate twice (the first run builds the engine), then
    # the 256-row tile twice at the winner
    grid = len(autotune.CLUSTERS) * len(autotune.SLOTS) * len(autotune.SHARE_FRACTIONS)
    assert len(calls) == 2 * grid + 2
    assert len(res["candidates"]) == grid + 1
    assert {(c["slots"], c["sm_share"], c["cluster"]) for c in calls[-2:]} == {(16, 76, 8)}
    assert all(c["av_rows"] == 256 for c in calls[-2:])
    # the probe: every 4th trial in descending size order, every size class present
    assert res["probe_trials"] == len(n) // 4
    assert sorted(set(calls[0]["n"])) == [1024, 2048, 4096, 8192, 16384]
    # the caller's form reaches every probe call
    assert all("grad_format" in c["kw"] and "residual_refresh" in c["kw"] for c in calls)


def test_autotune_keeps_128_row_tiles_when_not_faster(fake_device):
    from gaga_gb300 import autotune

    _, _, state = fake_device
    state["tile256"] = 1.2
    n, m, k = _workload()
    res = autotune.tune_batch(n, m, k, 7, alg="NIHT", stride=3, use_cache=False)
    assert (res["slots"], res["sm_share"], res["cluster"], res["av_rows"]) == (16, 76, 8, 128)
    assert res["candidates"][-1]["av_rows"] == 256  # measured, and not taken
    assert res["probe_trials"] == len(n) // 3


def test_autotune_cache_is_per_form(fake_device):
    from gaga_gb300 import autotune

    calls, path, _ = fake_device
    n, m, k = _workload()
    first = autotune.tune_batch(n, m, k, 7, alg="CGIHT", grad_format="bf16", residual_refresh=8)
    ncalls = len(calls)
    again = autotune.tune_batch(n, m, k, 7, alg="CGIHT", grad_format="bf16", residual_refresh=8)
    assert again["cached"] is True and len(calls) == ncalls
    assert (again["slots"], again["sm_share"], again["cluster"], again["av_rows"]) == \
        (first["slots"], first["sm_share"], first["cluster"], first["av_rows"])
    # another operand, recurrence or start is another form: measured again, cached apart
    autotune.tune_batch(n, m, k, 7, alg="CGIHT", grad_format="a24", residual_refresh=8)
    assert len(calls) > ncalls
    ncalls = len(calls)
    autotune.tune_batch(n, m, k, 7, alg="CGIHT", grad_format="bf16", residual_refresh=0)
    assert len(calls) > ncalls
    keys = list(json.load(open(path)))
    assert len(keys) == 3 and len(set(keys)) == 3
    assert all(key.startswith("FAKE GB300|CGIHT") for key in keys)
