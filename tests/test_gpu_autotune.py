"""The autotuner (lighthugger_gb300.autotune): every candidate launch shape
gives the same bits, the tuning it keeps is the fastest it timed, and it is
cached under the workload's signature (GPU, sizes, scene, camera) and applied
from the cache on the next call."""
import hashlib
import json

import pytest

pytestmark = pytest.mark.gpu


def test_tune_keeps_fastest_identical_outputs_and_caches(native, tmp_path):
    lh = native
    from lighthugger_gb300 import autotune
    scene = lh.Scene(2, detail=0.25, n_instances=1024, width=960, height=540).upload(0)
    d = scene.desc
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=1024,
                              max_draws=200000))
    r.set_scene(scene)
    u = scene.uniforms

    def digest():
        h = hashlib.sha1()
        for a in (r.visibility(), r.shadow_maps(), r.hdr()):
            h.update(a.tobytes())
        return h.hexdigest()

    path = str(tmp_path / "tuning.json")
    best, results = autotune.tune(r, u, frames=2, cache_path=path, digest=digest)
    digests = results.pop("digests")
    assert len(results) >= 15 and set(digests) == set(results)
    assert len(set(digests.values())) == 1, "a launch shape changed the output"
    assert best["ms"] == min(results.values())
    applied = r.tuning().as_dict()
    for k in autotune.KNOBS:
        assert applied[k] == best[k], k
    cache = json.load(open(path))
    key = autotune.signature(r, u, 0, False)
    assert key in cache and cache[key]["ms"] == best["ms"]
    # another camera is another workload
    u2 = lh.make_uniforms((10.0, 5.0, -140.0), 1.5, 0.05, 60.0, d.width, d.height, d.n_instances)
    assert autotune.signature(r, u2, 0, False) != key
    # the next call applies the cached tuning without timing anything
    r.set_tuning(occlusion_px=0, small_px=4, medium_px=4096)
    again, timed = autotune.tune(r, u, cache_path=path)
    assert timed == {} and r.tuning().as_dict()["occlusion_px"] == best["occlusion_px"]


def test_tune_backward_rows(native):
    """The adjoint's tile rows: every choice gives the same gradients (up to
    the order of float atomics) and the fastest is applied."""
    import ctypes as C
    import torch
    lh = native
    from lighthugger_gb300 import autotune
    scene = lh.Scene(4, width=256, height=256, n_instances=512).upload(0)
    d = scene.desc
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=1024, max_instances=1024,
                              max_draws=200000))
    r.set_scene(scene)
    r.frame(scene.uniforms)
    grad = torch.randn(d.height, d.width, 4, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1))
    light = torch.zeros(8, device="cuda")
    t = lh.GradTargets(instance_grads=0, texture_grads=0, light_dir=light.data_ptr(), light_color=light.data_ptr() + 16)
    outs = {}
    for rows in autotune.BACKWARD_ROWS:
        r.set_tuning(backward_rows=rows)
        light.zero_()
        assert lh.lib().lh_resolve_backward(r.ctx, grad.data_ptr(), C.byref(t), None) == 0
        torch.cuda.synchronize()
        outs[rows] = light.clone()
    ref = outs[8]
    for rows, g in outs.items():
        assert float((g - ref).abs().max()) <= 1e-4 * float(ref.abs().max()), rows
    best, timed = autotune.tune_backward(r, grad.data_ptr(), t, frames=2)
    assert best == min(timed, key=timed.get) and r.tuning().backward_rows == best
