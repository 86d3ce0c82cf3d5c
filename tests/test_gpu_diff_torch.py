"""The libtorch autograd Function around the resolve: its forward is the
frame's HDR image, its backward the GPU adjoint (vertex, material, texel and
light gradients), both run on PyTorch's current stream, and gradient steps
on the light colour and on the materials' roughness (the green channel of
their metallic-roughness texels) move the render to a target rendered with
other values."""
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
    # texel gradients: base-colour texels and roughness / metalness
    assert float(grads["textures"].abs().sum()) > 0
    rough = [dr.texture_view(grads["textures"], i)[..., 1] for i in _roughness_textures(dr)]
    assert float(sum(t.abs().sum() for t in rough)) > 0
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


def _roughness_textures(dr):
    """Indices of the metallic-roughness textures: the scene's 1 x 1 textures
    whose red channel is 1 (green = roughness, blue = metalness)."""
    out = []
    for i, (h, w) in enumerate(dr.texture_shapes):
        if h * w == 1 and float(dr.texture_view(dr.textures.detach(), i)[0, 0, 0]) == 1.0:
            out.append(i)
    return out


def test_runs_on_the_current_stream(native):
    """Forward and backward enqueued on a side stream give the default
    stream's image and gradients (up to the order of the adjoint's float
    atomic sums, which no two runs share: the tolerance is relative to each
    parameter group's largest gradient)."""
    import torch
    from lighthugger_gb300.diff import DiffResolve
    lh = native
    scene, r = _setup(lh)
    dr = DiffResolve(r, scene)
    g = torch.randn((scene.desc.height, scene.desc.width, 4), device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(2))
    hdr0 = dr()
    (hdr0 * g).sum().backward()
    ref = {k: v.grad.clone() for k, v in dr.parameters().items()}
    ref_img = hdr0.detach().clone()
    for v in dr.parameters().values():
        v.grad = None
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        hdr1 = dr()
        (hdr1 * g).sum().backward()
        got_img = hdr1.detach().clone()
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    assert torch.equal(got_img, ref_img)
    for k, v in dr.parameters().items():
        scale = float(ref[k].abs().max())
        assert scale > 0, k
        err = float((v.grad - ref[k]).abs().max())
        assert err <= 1e-4 * scale, (k, err, scale)


def test_roughness_fits_a_target(native):
    """Roughness is a texel parameter: a target rendered with every
    material's roughness at 0.4 is recovered from 0.7 by descending the
    roughness texels' gradients."""
    import torch
    from lighthugger_gb300.diff import DiffResolve
    lh = native
    scene, r = _setup(lh)
    dr = DiffResolve(r, scene)
    mr = _roughness_textures(dr)
    assert mr
    idx = torch.tensor([dr.texture_offset(i) + 1 for i in mr], device="cuda")  # green channel of each 1 x 1 texel

    def set_roughness(v):
        with torch.no_grad():
            dr.textures[idx] = v

    set_roughness(0.4)
    with torch.no_grad():
        target = dr().clone()
    rough = torch.full((len(mr),), 0.7, device="cuda", requires_grad=True)
    opt = torch.optim.Adam([rough], lr=0.02)
    losses = []
    for _ in range(120):
        set_roughness(rough.detach())
        dr.textures.grad = None
        loss = ((dr() - target)[..., :3] ** 2).mean()
        loss.backward()
        rough.grad = dr.textures.grad[idx].clone()
        opt.step()
        with torch.no_grad():
            rough.clamp_(0.05, 1.0)
        losses.append(float(loss.detach()))
    assert losses[-1] < 0.01 * losses[0], losses[::12]
    # materials that cover enough pixels converge to the target roughness
    err = (rough.detach() - 0.4).abs()
    assert float(err.median()) < 0.02, rough.detach().cpu().numpy()
