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


def _bind(lh):
    L = lh.lib()
    L.lh_cull_instances_noalloc.argtypes = [C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                            C.c_void_p]
    L.lh_cull_instances_noalloc.restype = C.c_int32
    return L


def _frame_sector(lh):
    scene = lh.Scene(2, detail=0.25, width=960, height=540).upload(0)
    d = scene.desc
    r = lh.Renderer(lh.Config(width=d.width, height=d.height, shadow_size=512, max_instances=4096, max_draws=200000))
    r.set_scene(scene)
    u = scene.uniforms
    r.frame(u)
    return scene, u, r.prefix_sector(0)


def test_noalloc_overflow_null_flags_and_empty(native):
    """The paths beside the normal one: more visible instances than the
    caller's capacity (flag raised, true count kept, entries stop at the
    capacity), no flags buffer at all, and an empty instance list."""
    import torch
    lh = native
    L = _bind(lh)
    scene, u, ref = _frame_sector(lh)
    d = scene.desc
    ref_counter = int(ref[:8].view(np.uint64)[0])
    count = ref_counter >> 32
    assert count > 8
    cap = count // 2
    sector = torch.full((8 + 8 * count + 64,), 0xAB, dtype=torch.uint8, device="cuda")
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = L.lh_cull_instances_noalloc(d.device_instances, d.n_instances, C.addressof(u), sector.data_ptr(), cap,
                                     flags.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize()
    got = sector.cpu().numpy()
    assert int(got[:8].view(np.uint64)[0]) == ref_counter  # the true count and sum
    assert np.array_equal(got[8:8 + 8 * cap], ref[8:8 + 8 * cap])
    assert np.all(got[8 + 8 * cap:] == 0xAB), "entries written beyond the capacity"
    assert int(flags.item()) == lh.FLAG_INSTANCE_OVERFLOW
    # no flags buffer: same sector, LH_OK
    sector.fill_(0xAB)
    st = L.lh_cull_instances_noalloc(d.device_instances, d.n_instances, C.addressof(u), sector.data_ptr(), count,
                                     None, None)
    assert st == 0
    torch.cuda.synchronize()
    got = sector.cpu().numpy()
    assert int(got[:8].view(np.uint64)[0]) == ref_counter
    assert np.array_equal(got[8:8 + 8 * count], ref[8:8 + 8 * count])
    # no instances: the counter word is zeroed and nothing else is touched
    sector.fill_(0xAB)
    flags.zero_()
    st = L.lh_cull_instances_noalloc(d.device_instances, 0, C.addressof(u), sector.data_ptr(), count,
                                     flags.data_ptr(), None)
    assert st == 0
    torch.cuda.synchronize()
    got = sector.cpu().numpy()
    assert int(got[:8].view(np.uint64)[0]) == 0
    assert np.all(got[8:] == 0xAB)
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
