"""Autotuner: choice rules and the persistent cache (CPU, with injected
timings), and one real tuning pass on the device."""
import json

import numpy as np
import pytest

from tcstencil_gb300 import autotune


def test_sweep_choice_is_persisted_per_class(tmp_path):
    path = str(tmp_path / "tune.json")
    fake = {"tensor": 2e-5, "cudacore": 1e-5}
    cache = autotune.Cache(path, shipped=None)
    e = autotune.tune_sweep("star2d1r", "f16", 300, 300, cache=cache,
                            timer=lambda eng, depth, *a, **kw: fake[eng])
    assert e["engine"] == "cudacore" and e["temporal_depth"] == 1
    # a fresh reader sees it, for any grid of the same size class only
    c2 = autotune.Cache(path, shipped=None)
    assert autotune.best_engine("star2d1r", "f16", 350, 270, cache=c2) == "cudacore"
    assert autotune.best_engine("star2d1r", "f16", 400, 300, cache=c2) == "tensor"
    assert autotune.best_engine("box2d2r", "f16", 300, 300, cache=c2) == "tensor"
    assert autotune.best_engine("box2d2r", "f32", 300, 300, cache=c2) == "cudacore"
    data = json.load(open(path))
    assert list(data.values())[0]["sweep"]["star2d1r/f16/8.5x8.5"]["engine"] == "cudacore"


def test_shipped_results_back_up_an_empty_cache(tmp_path):
    shipped = tmp_path / "shipped.json"
    dev = autotune.device_key()
    shipped.write_text(json.dumps({dev: {"sweep": {"box2d1r/f16/8x8": {"engine": "cudacore"}},
                                         "serve": {"poisson/2000": {"round_steps": 4}}}}))
    c = autotune.Cache(str(tmp_path / "user.json"), shipped=str(shipped))
    assert autotune.best_engine("box2d1r", "f16", 200, 256, cache=c) == "cudacore"
    assert autotune.best_round_steps(2000.0, cache=c) == 4
    c.section("serve")["poisson/2000"] = {"round_steps": 8}  # the user's own result wins
    assert autotune.best_round_steps(2000.0, cache=c) == 8


def test_split_tries_both_temporal_depths_and_launch_forms(tmp_path):
    seen = []
    cache = autotune.Cache(str(tmp_path / "t.json"), shipped=None)
    e = autotune.tune_sweep("box2d1r", "split", 64, 64, cache=cache,
                            timer=lambda eng, depth, *a: seen.append((eng, depth, a[-1])) or 1.0 / depth)
    assert seen == [("tensor", 1, 0), ("tensor", 1, 1), ("tensor", 2, 0)]
    assert set(e["s_per_step"]) == {"tensor/1", "tensor/1/m", "tensor/2"}
    assert e["engine"] == "tensor" and e["temporal_depth"] == 2 and e["multistep"] == 0
    assert autotune.best_config("box2d1r", "split", 60, 50, cache=cache) == ("tensor", 2)
    assert autotune.best_config("box2d2r", "split", 60, 50, cache=cache) == ("tensor", 1)


def test_launch_form_is_tuned_and_looked_up(tmp_path):
    cache = autotune.Cache(str(tmp_path / "t.json"), shipped=None)
    times = {("tensor", 1, 0): 3.0, ("tensor", 1, 1): 2.0, ("cudacore", 1, 0): 9.0}
    e = autotune.tune_sweep("box2d2r", "f16", 5000, 5000, cache=cache,
                            timer=lambda eng, depth, *a, tile_w=128: times[(eng, depth, a[-1])]
                            + (tile_w != 128))
    assert e["engine"] == "tensor" and e["temporal_depth"] == 1 and e["multistep"] == 1
    assert e["tile_w"] == 128
    assert autotune.best_launch("box2d2r", "f16", 4500, 5500, cache=cache) == 1
    assert autotune.best_launch("box2d2r", "f16", 300, 300, cache=cache) == -1  # not tuned


def test_tile_width_is_tuned_and_looked_up(tmp_path):
    """Plain FP16 tensor candidates come in 128-, 96- and 64-column tiles;
    the fastest width is stored and Plan(engine="auto") takes it."""
    cache = autotune.Cache(str(tmp_path / "t.json"), shipped=None)
    seen = []

    def timer(eng, depth, *a, tile_w=128):
        seen.append((eng, a[-1], tile_w))
        return {128: 3.0, 96: 2.0, 64: 2.5}[tile_w] + (0.5 if a[-1] else 0) + (eng == "cudacore")

    e = autotune.tune_sweep("star2d1r", "f16", 1026, 1026, cache=cache, timer=timer)
    assert sorted(seen) == sorted([("tensor", m, w) for w in (128, 96, 64) for m in (0, 1)] +
                                  [("cudacore", 0, 128)])
    assert (e["engine"], e["multistep"], e["tile_w"]) == ("tensor", 0, 96)
    assert "tensor/1/w96" in e["s_per_step"] and "tensor/1/m/w64" in e["s_per_step"]
    assert autotune.best_tile_width("star2d1r", 1100, 1300, cache=cache) == 96
    assert autotune.best_tile_width("star2d1r", 3000, 3000, cache=cache) == 128  # not tuned
    assert autotune.parse_candidate("tensor/1/m/w64") == ("tensor", 1, 1, 64)
    assert autotune.parse_candidate("cudacore/1") == ("cudacore", 1, 0, 128)


def test_serve_choice_prefers_low_p99_among_those_keeping_up(tmp_path):
    runs = {0: {"gpts": 260.0, "p50_ms": 20.0, "p99_ms": 58.0},
            4: {"gpts": 265.0, "p50_ms": 6.0, "p99_ms": 66.0},
            16: {"gpts": 265.0, "p50_ms": 7.0, "p99_ms": 63.0},
            32: {"gpts": 200.0, "p50_ms": 5.0, "p99_ms": 10.0}}  # fell behind
    cache = autotune.Cache(str(tmp_path / "t.json"), shipped=None)
    e = autotune.tune_serve(2000.0, candidates=tuple(runs), cache=cache,
                            runner=lambda rate, sec, rs, b: runs[rs])
    assert e["round_steps"] == 0  # 260 is within 2 % of 265, and its p99 is lowest
    assert autotune.best_round_steps(2000.0, cache=autotune.Cache(cache.path, shipped=None)) == 0
    assert autotune.best_round_steps(1000.0, cache=cache) == autotune.DEFAULT_ROUND_STEPS


@pytest.mark.gpu
def test_real_tuning_pass_and_auto_engine(tcs, torch_cuda, tmp_path, monkeypatch):
    monkeypatch.setenv("TCS_AUTOTUNE_CACHE", str(tmp_path / "t.json"))
    e = autotune.tune_sweep("star2d2r", "f16", 512, 512, steps=5)
    assert e["engine"] in ("tensor", "cudacore")
    assert all(t > 0 for t in e["s_per_step"].values())
    s = autotune.tune_sweep("star2d2r", "split", 512, 512, steps=6)
    assert set(s["s_per_step"]) == {"tensor/1", "tensor/1/m", "tensor/2"}
    p = tcs.Plan(512, 512, "star2d2r", np.full((5, 5), 0.04, np.float32), engine="auto")
    g = np.random.default_rng(0).uniform(-1, 1, (512, 512)).astype(np.float32)
    p.upload(g)
    p.run(3)
    out = np.empty_like(g)
    p.download(out)
    torch_cuda.cuda.synchronize()
    ref = tcs.Plan(512, 512, "star2d2r", np.full((5, 5), 0.04, np.float32), engine=e["engine"])
    ref.upload(g)
    ref.run(3)
    out2 = np.empty_like(g)
    ref.download(out2)
    torch_cuda.cuda.synchronize()
    np.testing.assert_array_equal(out, out2)


def test_shipped_tuning_is_consistent():
    """Every shipped sweep entry names a candidate the tuner tries for its
    precision, and its choice is the fastest recorded time."""
    shipped = json.load(open(autotune.SHIPPED))
    assert shipped, "tuned.json is empty"
    for dev, sections in shipped.items():
        for key, e in sections.get("sweep", {}).items():
            stencil, precision, size = key.split("/")
            assert stencil in ("star2d1r", "star2d2r", "box2d1r", "box2d2r")
            valid = {autotune.candidate_key(*c) for c in autotune.CANDIDATES[precision]}
            assert set(e["s_per_step"]) <= valid, (dev, key)
            chosen = autotune.candidate_key(e["engine"], e["temporal_depth"], e.get("multistep", 0),
                                            e.get("tile_w", 128))
            assert chosen in e["s_per_step"], (dev, key)
            assert e["s_per_step"][chosen] == min(e["s_per_step"].values()), (dev, key)
        for key, e in sections.get("serve", {}).items():
            assert int(e["round_steps"]) >= 0 and str(e["round_steps"]) in e["candidates"]
