"""Autotuner of the batch march: candidate space, workload signature and
cache (CPU), and on the GPU that every candidate renders the same bytes."""

import json

import numpy as np
import pytest

from pyvr_gb300 import autotune as AT
from pyvr_gb300 import workloads as W
from pyvr_gb300.batch import Tuning


def _small_scenes(n=5):
    return W.config_batching(n, max_dim=40, resolutions=(32, 48, 64))


def test_candidates_are_valid_launch_settings():
    cands = AT.candidates()
    assert len(cands) == len(AT.TILES) * len(AT.BRICKS) * len(AT.STEPS) * len(AT.BLOCKS)
    for t in cands:
        assert t.tile_w * t.tile_h == 256 and t.tile_w % 8 == 0 and t.tile_h % 4 == 0
        assert t.steps_per_iter in (1, 4) and 2 <= t.brick_log2 <= 4 and 0 <= t.blocks_per_sm <= 16


def test_workload_signature_is_stable_and_sensitive():
    a = AT.workload_signature(_small_scenes())
    assert a == AT.workload_signature(_small_scenes())
    s = _small_scenes()
    s[2]["width"] += 1
    assert AT.workload_signature(s) != a


def test_cached_tuning_is_used(tmp_path, monkeypatch):
    scenes = _small_scenes(3)
    monkeypatch.setattr(AT, "device_key", lambda: "TESTGPU|sm1")
    path = tmp_path / "tuning.json"
    want = Tuning(tile_w=32, tile_h=8, steps_per_iter=4, blocks_per_sm=3, brick_log2=2)
    path.write_text(json.dumps({f"TESTGPU|sm1|{AT.workload_signature(scenes)}": want.__dict__}))
    got, results = AT.autotune(scenes, cache_path=str(path))
    assert got == want and results == []


@pytest.mark.gpu
def test_every_candidate_renders_the_same_bytes(tmp_path):
    pytest.importorskip("torch")
    scenes = _small_scenes(6)
    bench = AT._Bench(scenes)
    ref = None
    picks = [Tuning(), Tuning(tile_w=32, tile_h=8, steps_per_iter=4, blocks_per_sm=3, brick_log2=2),
             Tuning(tile_w=8, tile_h=32, steps_per_iter=1, blocks_per_sm=5, brick_log2=4),
             Tuning(tile_w=16, tile_h=16, steps_per_iter=4, blocks_per_sm=0, brick_log2=3)]
    for t in picks:
        for o in bench.outs:
            o.zero_()
        assert bench.time(t, repeats=1) > 0
        imgs = bench.images()
        assert any(i.any() for i in imgs)
        if ref is None:
            ref = imgs
        else:
            for a, b in zip(imgs, ref):
                assert np.array_equal(a, b), t
    best, results = AT.autotune(scenes, repeats=1, cands=picks, cache_path=str(tmp_path / "t.json"))
    assert best in picks and len(results) == len(picks)
    again, res2 = AT.autotune(scenes, cache_path=str(tmp_path / "t.json"))
    assert again == best and res2 == []
