"""Pipelined readback (lh_frame_readback): each frame's HDR image reaches its
host buffer intact while the next frame runs, and work that rewrites the
image (a later frame's resolve, a replayed graph) waits for the copy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(lh):
    scene = lh.Scene(1).upload(0)
    d = scene.desc
    cfg = lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=1024,
                    max_draws=200000, device=0)
    r = lh.Renderer(cfg)
    r.set_scene(scene)
    views = [scene.uniforms,
             lh.make_uniforms((10.0, 5.0, -140.0), 0.35, -0.1, 60.0, d.width, d.height, d.n_instances),
             lh.make_uniforms((-20.0, 0.0, -120.0), -0.3, 0.05, 50.0, d.width, d.height, d.n_instances)]
    return scene, r, views


def _expected(r, views):
    out = []
    for u in views:
        r.frame(u)
        out.append(r.hdr().copy())
    return out


def test_readback_frames_match_serial_frames(native):
    import torch
    lh = native
    scene, r, views = _setup(lh)
    ref = _expected(r, views)
    assert not np.array_equal(ref[0], ref[1])
    d = scene.desc
    bufs = [torch.empty(d.width * d.height * 4, dtype=torch.float32, pin_memory=True) for _ in range(2)]
    order = [0, 1, 2, 1, 0, 2, 2, 1]
    for i, v in enumerate(order):
        r.frame_readback(views[v], bufs[i & 1].data_ptr())
        if i:
            got = bufs[(i - 1) & 1].numpy().reshape(d.height, d.width, 4)
            assert np.array_equal(got, ref[order[i - 1]]), "frame %d (view %d)" % (i - 1, order[i - 1])
    r.readback_wait()
    got = bufs[(len(order) - 1) & 1].numpy().reshape(d.height, d.width, 4)
    assert np.array_equal(got, ref[order[-1]])
    assert r.status().flags == 0


def test_readback_then_graph_frame_waits_for_the_copy(native):
    import torch
    lh = native
    scene, r, views = _setup(lh)
    ref = _expected(r, views)
    d = scene.desc
    buf = torch.empty(d.width * d.height * 4, dtype=torch.float32, pin_memory=True)
    for _ in range(3):
        r.frame_readback(views[0], buf.data_ptr())
        r.frame_graph(views[1])  # its resolve rewrites the image being copied
        r.readback_wait()
        assert np.array_equal(buf.numpy().reshape(d.height, d.width, 4), ref[0])
        assert np.array_equal(r.hdr(), ref[1])


def test_readback_rejects_null_buffer(native):
    lh = native
    scene, r, views = _setup(lh)
    with pytest.raises(lh.LHError):
        r.frame_readback(views[0], None)
