"""The oracle against its committed golden digests (tests/golden/
oracle_frames.json, written by tests/golden/make_golden.py): the same four
seeded scenes through the oracle must give byte-identical prefix sectors,
meshlet references, draw commands, visibility, shadow maps and MiscStorage,
and the same HDR sum and maximum to a relative 1e-6.  The GPU parity tests
compare the CUDA path with the oracle; these fixtures keep the oracle (and
the scene generator feeding both) from drifting unnoticed."""
import json
import os

import pytest

from tests.conftest import ROOT

GOLDEN = os.path.join(ROOT, "tests", "golden", "oracle_frames.json")
EXACT = ("instances_sha256", "views", "visibility_sha256", "shadow_maps_sha256", "misc_sha256", "covered_pixels",
         "flags", "size", "shadow_size")

with open(GOLDEN) as _f:
    _CASES = json.load(_f)


@pytest.mark.parametrize("name", sorted(_CASES))
def test_oracle_matches_golden_digests(native, name):
    from tests.golden.make_golden import CASES, frame_digest
    want = _CASES[name]
    config_id, params = CASES[name]
    got = frame_digest(config_id, params)
    assert got["seed"] == want["seed"]
    for k in EXACT:
        assert got[k] == want[k], "%s: %s differs" % (name, k)
    for k in ("hdr_sum", "hdr_max"):
        assert got[k] == pytest.approx(want[k], rel=1e-6), "%s: %s" % (name, k)
