"""The allocation-free instance cull (lh_cull_instances_noalloc) against lh_frame.

Callers that cannot allocate device memory (fixed-budget engines, frame
loops that must not stall on cudaMalloc, stream capture) use the no-alloc
entry point; it must give exactly the prefix sector that lh_frame's own
instance cull writes for the main view, on every call, since all calls share
one scratch array inside the library.  This file is collected last on
purpose.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_cull_matches_frame_twice(native):
    import torch
    lh = native
    L = lh.lib()
    L.lh_cull_instances_noalloc.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                            C.c_void_p]
    L.lh_cull_instances_noalloc.restype = C.c_int32
    # config 2 layout: 4,096 instances = 16 tiles, so the look-back runs
    scene = lh.Scene(2, detail=0.25, width=960, height=540).upload(0)
    d = scene.desc
    cap = 4096
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=512, max_instances=cap, max_draws=200000))
    r.set_scene(scene)
    u = scene.uniforms
    r.frame(u)
    ref = r.prefix_sector(0)
    ref_counter = int(ref[:8].view(np.uint64)[0])
    count = ref_counter >> 32
    assert count > 0
    torch.cuda.synchronize()
    sector = torch.empty(8 + 8 * cap, dtype=torch.uint8, device="cuda")
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    for call in range(2):
        sector.fill_(0xAB)  # stale bytes must be overwritten
        st = L.lh_cull_instances_noalloc(d.device_instances, d.n_instances, C.addressof(u), sector.data_ptr(), cap,
                                         flags.data_ptr(), None)
        assert st == 0, "call %d returned %d" % (call, st)
        torch.cuda.synchronize()
        got = sector.cpu().numpy()
        counter = int(got[:8].view(np.uint64)[0])
        assert counter == ref_counter, "call %d: counter %#x, lh_frame %#x" % (call, counter, ref_counter)
        assert np.array_equal(got[8:8 + 8 * count], ref[8:8 + 8 * count]), "call %d: entries differ" % call
        assert int(flags.item()) == 0


def test_noalloc_rejects_too_many_instances(native):
    lh = native
    L = lh.lib()
    L.lh_cull_instances_noalloc.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                            C.c_void_p]
    L.lh_cull_instances_noalloc.restype = C.c_int32
    u = lh.Uniforms()
    # 1,048,577 instances exceed the fixed scratch: rejected before any launch
    st = L.lh_cull_instances_noalloc(C.c_void_p(256), 1048577, C.addressof(u), C.c_void_p(256), 16, None, None)
    assert st == 4  # LH_ERR_CAPACITY
