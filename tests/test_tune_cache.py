"""The autotuner's bookkeeping without a GPU: the cache is keyed by the
workload signature, a cached choice is returned without measuring, a retune
measures again, and the tuned parameters carry the chosen engine and launch
shape (measurement itself is covered by tests/test_tune.py on the GPU)."""
import json

from c2a_gb300 import api, tune


class _FakeTuner(tune.Tuner):
    def __init__(self, cache, record):
        super().__init__(ctx=None, cache=cache)
        self.record, self.calls = record, 0

    def measure(self, d_queries, n, params, contacts_per_query=64, stream=None):
        self.calls += 1
        return dict(self.record)


def test_choice_is_cached_per_signature(tmp_path, monkeypatch):
    cache = str(tmp_path / "t.json")
    key = {"k": "GB300|sm152|reference|contacts1x64|tris40000|n2^16"}
    monkeypatch.setattr(tune, "signature", lambda ctx, dq, n, params, cpq: key["k"])
    rec = {"choice": {"engine": api.ENGINE_SPEC, "warps_per_sm": 4, "name": "spec/4"},
           "ms": {"warp/max": 3.0, "spec/4": 2.0}, "sample_queries": 16, "batch_queries": 65536, "when": 0.0}
    t = _FakeTuner(cache, rec)
    params = {"tol_d": 1e-4, "tol_t": 1e-4, "toc_delta": 1e-4, "engine": api.ENGINE_AUTO}
    r = t.choose(None, 65536, params)
    assert t.calls == 1 and not r["record"]["cached"]
    assert r["params"]["engine"] == api.ENGINE_SPEC and r["params"]["warps_per_sm"] == 4
    assert params["engine"] == api.ENGINE_AUTO  # the caller's dict is left alone
    table = json.load(open(cache))
    assert list(table) == [key["k"]] and table[key["k"]]["choice"]["name"] == "spec/4"
    again = t.choose(None, 65536, params)
    assert t.calls == 1 and again["record"]["cached"] and again["params"] == r["params"]
    t.choose(None, 65536, params, retune=True)
    assert t.calls == 2
    key["k"] = "GB300|sm152|canonical|contacts1x64|tris40000|n2^16"  # another kind of batch: measured anew
    t.choose(None, 65536, params)
    assert t.calls == 3 and len(json.load(open(cache))) == 2


def test_candidates_by_mode():
    t = tune.Tuner(ctx=None, cache=None)
    ref = t.candidates({"mode": api.MODE_REFERENCE})
    can = t.candidates({"mode": api.MODE_CANONICAL})
    assert (api.ENGINE_WARP, 0) in ref and (api.ENGINE_SPEC, 0) in ref and (api.ENGINE_THREAD, 0) in ref
    assert all(e in (api.ENGINE_WARP, api.ENGINE_BATCHED) for e, _ in can)
    assert all(e != api.ENGINE_BATCHED for e, _ in ref)
