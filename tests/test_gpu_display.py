"""Display transform on the GPU (lh_display_transform) against the oracle's
restatement of display_transform.comp on the same HDR image: 8-bit output
within one step (powf vs the host pow may differ in the last bit before
rounding), the stand-in LUT, a caller LUT and the cascade overlay."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _frame(lh, debug_shadowmaps=0):
    scene = lh.Scene(1).upload(0)
    d = scene.desc
    u = lh.Uniforms.from_buffer_copy(bytes(scene.uniforms))
    ctypes.memmove(ctypes.addressof(u) + 556, ctypes.byref(ctypes.c_uint32(debug_shadowmaps)), 4)
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=d.shadow_size, max_instances=1024,
                              max_draws=200000))
    r.set_scene(scene)
    r.frame(u)
    return scene, r


@pytest.mark.parametrize("debug_shadowmaps", [0, 1])
def test_display_transform_matches_oracle(native, oracle, debug_shadowmaps):
    import torch
    lh = native
    scene, r = _frame(lh, debug_shadowmaps)
    d = scene.desc
    out = torch.zeros(d.height * d.width * 4, dtype=torch.uint8, device="cuda")
    r.display_transform(out.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(d.height, d.width, 4)
    ref = oracle.display_transform(r.hdr(), shadow_maps=r.shadow_maps() if debug_shadowmaps else None,
                                   debug_shadowmaps=debug_shadowmaps)
    diff = np.abs(got.astype(np.int32) - ref.astype(np.int32))
    assert diff.max() <= 1, diff.max()
    assert (diff > 0).mean() < 1e-3
    assert len(np.unique(got[..., 0])) > 16


def test_display_transform_caller_lut(native, oracle):
    import torch
    lh = native
    scene, r = _frame(lh)
    d = scene.desc
    g = np.linspace(0, 1, 48, dtype=np.float32)
    lut = np.zeros((48, 48, 48, 4), np.float32)
    lut[..., 0] = g[None, None, :] ** 2  # a non-linear curve on r
    lut[..., 1] = g[None, :, None]
    lut[..., 2] = 1.0 - g[:, None, None]
    lut_dev = torch.from_numpy(lut).cuda()
    out = torch.zeros(d.height * d.width * 4, dtype=torch.uint8, device="cuda")
    r.display_transform(out.data_ptr(), lut_dev.data_ptr())
    torch.cuda.synchronize()
    got = out.cpu().numpy().reshape(d.height, d.width, 4)
    ref = oracle.display_transform(r.hdr(), lut=lut)
    assert np.abs(got.astype(np.int32) - ref.astype(np.int32)).max() <= 1
