"""The autotuner's host logic (lighthugger_gb300/autotune.py) on CPU: a fake
renderer whose frame time is a known function of the tuning, with the CUDA
timing replaced.  Coordinate descent must land on the fastest value of
every knob group, apply it, cache it under a key that tells scenes and
cameras apart, and reuse the cache without timing again."""
import json

import pytest

torch = pytest.importorskip("torch")


class _Tuning:
    def __init__(self, d):
        self.d = dict(d)

    def as_dict(self):
        return dict(self.d)


class _Desc:
    def __init__(self, seed):
        self.n_instances, self.total_triangles, self.seed = 4096, 54_500_000, seed


class _Scene:
    def __init__(self, seed):
        self.desc = _Desc(seed)


class _Config:
    width, height, shadow_size = 1920, 1080, 1024


class FakeRenderer:
    def __init__(self, seed=1):
        self.config = _Config()
        self.scene = _Scene(seed)
        self.state = {"small_px": 32, "medium_px": 32, "schedule": 0, "raster_batch": 0, "occlusion_px": 128,
                      "chunk_rows": [16, 32], "chunk_cols": [128, 64], "cull_blocks_per_sm": 3.0, "backward_rows": 8}
        self.applied = []

    def tuning(self):
        return _Tuning(self.state)

    def set_tuning(self, **kw):
        self.state.update({k: (list(v) if isinstance(v, (list, tuple)) else v) for k, v in kw.items()})
        self.applied.append(dict(kw))

    def frame_graph(self, *a, **kw):
        pass


# a separable frame time with one best value per knob group
BEST = {"occlusion_px": 32, "bins": (16, 64), "vis_chunk": (32, 128), "shadow_chunk": (16, 64), "raster_batch": 2,
        "schedule": 1}


def _cost(s):
    c = 1.0
    c += 0.0 if s["occlusion_px"] == BEST["occlusion_px"] else 0.05
    c += 0.0 if (s["small_px"], s["medium_px"]) == BEST["bins"] else 0.04
    c += 0.0 if (s["chunk_rows"][0], s["chunk_cols"][0]) == BEST["vis_chunk"] else 0.03
    c += 0.0 if (s["chunk_rows"][1], s["chunk_cols"][1]) == BEST["shadow_chunk"] else 0.02
    c += 0.0 if s["raster_batch"] == BEST["raster_batch"] else 0.01
    c += 0.0 if s["schedule"] == BEST["schedule"] else 0.005
    return c


@pytest.fixture
def fake_cuda(monkeypatch):
    from lighthugger_gb300 import autotune
    timed = []

    def fake_time(renderer, run, frames, stream):
        run()
        timed.append(dict(renderer.state))
        return _cost(renderer.state)

    class _Stream:
        cuda_stream = 0

    monkeypatch.setattr(autotune, "time_frames", fake_time)
    monkeypatch.setattr(torch.cuda, "Stream", _Stream)
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda *a: "fake-gpu")
    return timed


def test_descent_finds_every_groups_best_and_caches_it(fake_cuda, tmp_path):
    from lighthugger_gb300 import SCHEDULE_PER_STAGE, SCHEDULE_PERSISTENT, autotune
    assert BEST["schedule"] in (SCHEDULE_PER_STAGE, SCHEDULE_PERSISTENT)
    r = FakeRenderer()
    cache = str(tmp_path / "tuning.json")
    u = bytes(range(256)) * 2
    best, results = autotune.tune(r, u, probes=None, n_probes=3, batched=True, cache_path=cache)
    assert best["occlusion_px"] == BEST["occlusion_px"]
    assert (best["small_px"], best["medium_px"]) == BEST["bins"]
    assert (best["chunk_rows"][0], best["chunk_cols"][0]) == BEST["vis_chunk"]
    assert (best["chunk_rows"][1], best["chunk_cols"][1]) == BEST["shadow_chunk"]
    assert best["raster_batch"] == BEST["raster_batch"] and best["schedule"] == BEST["schedule"]
    assert best["ms"] == pytest.approx(1.0) == min(results.values())
    # the renderer is left on the kept tuning
    for k in autotune.KNOBS:
        assert r.state[k] == best[k], k
    # each candidate timed once
    assert len(fake_cuda) == len(results)
    saved = json.load(open(cache))
    assert list(saved.values())[0]["occlusion_px"] == BEST["occlusion_px"]
    # a second call reuses the cache without timing
    n = len(fake_cuda)
    r2 = FakeRenderer()
    best2, results2 = autotune.tune(r2, u, probes=None, n_probes=3, batched=True, cache_path=cache)
    assert results2 == {} and len(fake_cuda) == n
    assert {k: best2[k] for k in autotune.KNOBS} == {k: r2.state[k] for k in autotune.KNOBS}


def test_cache_key_tells_workloads_apart(fake_cuda):
    from lighthugger_gb300 import autotune
    u1, u2 = bytes(560), bytes([1]) + bytes(559)
    a = autotune.signature(FakeRenderer(seed=1), u1, 0, False)
    assert a == autotune.signature(FakeRenderer(seed=1), u1, 0, False)
    assert a != autotune.signature(FakeRenderer(seed=2), u1, 0, False)   # another scene
    assert a != autotune.signature(FakeRenderer(seed=1), u2, 0, False)   # another camera
    assert a != autotune.signature(FakeRenderer(seed=1), u1, 3, True)    # batched with probes
