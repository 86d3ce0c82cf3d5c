"""C ABI of the native library: every declared symbol is exported, the C
layouts match the Python mirror, and host-side argument checks return status
codes (no GPU needed; no compute is launched)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from tests.conftest import HAS_GPU, ROOT

HEADERS = [os.path.join(ROOT, "include", "lh", h) for h in ("lh.h", "scene.h", "shared.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\*?\s+\*?(lh_[a-z0-9_]+)\s*\(", src, re.M):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported(native):
    names = declared_functions()
    assert len(names) >= 15, names
    L = native.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


@pytest.mark.parametrize("lang", ["c", "c++"])
def test_headers_compile_with_layout_asserts(lang):
    """The headers' static_asserts pin the reference's scalar-layout offsets."""
    r = subprocess.run(["gcc" if lang == "c" else "g++", "-fsyntax-only", "-x", lang, "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "include", "lh", "scene.h")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_python_mirror_sizes_match_c(native):
    lh = native
    prog = r"""
#include <stdio.h>
#include "lh/scene.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(lh_config), sizeof(lh_texture), sizeof(lh_frame_out),
         sizeof(lh_device_status), sizeof(lh_tuning), sizeof(lh_scene_params), sizeof(lh_scene_desc),
         sizeof(lh_camera));
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        src, exe = os.path.join(d, "s.c"), os.path.join(d, "s")
        open(src, "w").write(prog)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), src, "-o", exe], check=True)
        sizes = [int(x) for x in subprocess.run([exe], capture_output=True, text=True, check=True).stdout.split()]
    mine = [C.sizeof(t) for t in (lh.Config, lh.Texture, lh.FrameOut, lh.DeviceStatus, lh.Tuning, lh.SceneParams,
                                  lh.SceneDesc, lh.Camera)]
    assert sizes == mine


def test_null_and_bad_arguments_return_status(native):
    L = native.lib()
    P = C.c_void_p
    assert L.lh_create(None, None) == 1
    assert L.lh_set_scene(None, None, 0, None, 0) == 1
    assert L.lh_frame(None, None, None, None) == 1
    assert L.lh_read_status(None, None) == 1
    assert L.lh_last_error(None) == b"null context"
    L.lh_destroy(None)
    cfg = native.Config(width=0, height=0)
    h = P()
    assert L.lh_create(C.byref(cfg), C.byref(h)) == 1  # empty window
    cfg = native.Config(width=64, height=64, max_draws=1 << 24)  # 2*max_draws slots exceed the 24-bit ID
    assert L.lh_create(C.byref(cfg), C.byref(h)) == 1
    cfg = native.Config(width=64, height=64, shadow_size=64, max_instances=16, max_draws=16, flags=2)
    assert L.lh_create(C.byref(cfg), C.byref(h)) == 1  # unknown config flag
    assert L.lh_frame_readback(None, None, None, None, None) == 1
    assert L.lh_readback_wait(None) == 1
    assert L.lh_scene_create(9, 1, None, C.byref(h)) == 1
    cam = native.Camera()
    u = native.Uniforms()
    assert L.lh_make_uniforms(C.byref(cam), C.byref(u)) == 1  # zero-size window


@pytest.mark.skipif(HAS_GPU, reason="checks the no-device error path")
def test_create_without_device_reports_cuda_error(native):
    L = native.lib()
    cfg = native.Config(width=64, height=64, shadow_size=64)
    h = C.c_void_p()
    assert L.lh_create(C.byref(cfg), C.byref(h)) == 2  # LH_ERR_CUDA, no abort
    assert not h.value


def test_scene_upload_without_device_fails_cleanly(native):
    if HAS_GPU:
        pytest.skip("no-device path")
    s = native.Scene(1, detail=0.1, n_instances=2)
    with pytest.raises(native.LHError):
        s.upload(0)
