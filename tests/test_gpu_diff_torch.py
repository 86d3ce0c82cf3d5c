"""The libtorch autograd Function around the resolve: its forward is the
frame's HDR image, its backward the GPU adjoint, and a gradient step on the
light colour moves the render towards a target rendered with another
colour."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(lh):
    scene = lh.Scene(4, width=256, height=256, n_instances=512).upload(0)
    d = scene.desc
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=1024, max_instances=1024,
                              max_draws=200000))
    r.set_scene(scene)
    return scene, r


def test_forward_equals_frame_and_backward_is_the_adjoint(native):
    import torch
    from lighthugger_gb300.diff import DiffResolve
    lh = native
    scene, r = _setup(lh)
    dr = DiffResolve(r, scene)
    hdr = dr()
    torch.cuda.synchronize()
    r.frame(scene.uniforms)
    ref = r.hdr()
    assert np.array_equal(hdr.detach().cpu().numpy(), ref)
    g = torch.randn(hdr.shape, device=hdr.device, generator=torch.Generator(device=hdr.device).manual_seed(5))
    (hdr * g).sum().backward()
    grads = {k: v.grad for k, v in dr.parameters().items()}
    assert all(t is not None for t in grads.values())
    assert float(grads["positions"].abs().sum()) > 0
    assert float(grads["light_color"].abs().sum()) > 0
    # light colour multiplies the sun term: dL/dc_k = sum over pixels of g_k * sun_k
    # (sun = hdr - ambient); checked against the image with c and 2c
    with torch.no_grad():
        base = dr().clone()
        dr.light_color.mul_(2.0)
        twice = dr().clone()
        dr.light_color.div_(2.0)
    sun = (twice - base)[..., :3]
    expect = (g[..., :3] * sun).sum(dim=(0, 1)) / dr.light_color.detach()
    mass = (g[..., :3] * sun).abs().sum(dim=(0, 1)) / dr.light_color.detach()
    got = grads["light_color"]
    # the backward recomputes the radiance in camera-relative coordinates
    # with approximate division (closer to FP64 than the forward's absolute
    # float32, a few ulp per pixel); the random signs of g cancel most of the
    # sum, so the bound is relative to the sum of magnitudes
    assert bool(((got - expect).abs() <= 1e-3 * mass + 1e-3).all()), (got, expect, mass)


def test_light_colour_fits_a_target(native):
    import torch
    from lighthugger_gb300.diff import DiffResolve
    lh = native
    scene, r = _setup(lh)
    dr = DiffResolve(r, scene)
    with torch.no_grad():
        dr.light_color.copy_(torch.tensor([1.5, 0.7, 0.4], device="cuda"))
        target = dr().clone()
        dr.light_color.copy_(torch.tensor([1.0, 1.0, 1.0], device="cuda"))
    opt = torch.optim.Adam([dr.light_color], lr=0.05)
    sched = torch.optim.lr_scheduler.StepLR(opt, step_size=60, gamma=0.2)
    losses = []
    for _ in range(150):
        opt.zero_grad()
        loss = ((dr() - target)[..., :3] ** 2).mean()
        loss.backward()
        opt.step()
        sched.step()
        losses.append(float(loss.detach()))
    assert losses[-1] < 0.01 * losses[0], losses[::15]
    assert torch.allclose(dr.light_color.detach(), torch.tensor([1.5, 0.7, 0.4], device="cuda"), atol=0.02)
