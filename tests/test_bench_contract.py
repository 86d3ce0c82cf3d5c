"""bench.py's reference arm on the host cores (no GPU): one JSON line with
the GPU arm's metric and unit, `impl` "reference", a `cpu_baseline` of kind
"port" and an `e2e` block without host-device copies; ranks other than 0
print nothing and exit 0."""
import json
import os
import subprocess
import sys

from tests.conftest import ROOT


def _run(extra_env=None, *args):
    env = dict(os.environ)
    env.update(extra_env or {})
    return subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--config", "1",
                           "--steps", "2", "--warmup", "1", *args], capture_output=True, text=True, env=env,
                          cwd=ROOT, timeout=600)


def test_reference_arm_prints_one_line():
    sys.path.insert(0, ROOT)
    import bench
    r = _run()
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == "ms"
    assert d["higher_is_better"] is False and d["steps"] == 2 and d["warmup"] == 1
    assert d["value"] > 0 and d["ms_per_step"] == d["value"]
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("plain-small")


def test_reference_arm_other_ranks_exit_quietly():
    r = _run({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"})
    assert r.returncode == 0
    assert not [l for l in r.stdout.splitlines() if l.startswith("{")]


def test_roofline_traffic_comes_from_the_committed_capture():
    """The roofline's DRAM traffic is read from profiles/dram_bytes_c2_frame.txt
    (never measured in the bench): the sum of the stage's kernels' read and
    write bytes, the alpha-clip kernels only for a scene that has them, with
    the capture's provenance line."""
    sys.path.insert(0, ROOT)
    import bench
    per = {}
    with open(bench.TRAFFIC_FILE) as f:
        for line in f:
            if line.strip() and not line.startswith("#"):
                name, rd, wr = line.rsplit(None, 2)
                per[name.strip()] = per.get(name.strip(), 0.0) + float(rd) + float(wr)
    opaque, src = bench.committed_traffic("raster")
    with_alpha, _ = bench.committed_traffic("raster", True)
    want = sum(v for k, v in per.items() if k in bench.STAGE_KERNELS["raster"] and "alpha" not in k)
    assert opaque == want and with_alpha == want + per.get("k_raster_alpha<0>", 0.0)
    assert src.startswith("profiles/dram_bytes_c2_frame.txt: capture: commit")
    assert bench.committed_traffic("no_such_stage") == (None, None)
