"""The rasteriser's integer -> float conversions (lighthugger_gb300/csrc/
int_float.cuh), which keep the per-fragment edge-to-depth conversion off the
FP64 unit, compiled for the host and compared bit for bit with the
round-to-nearest-even conversion."""
import os
import subprocess
import tempfile

from tests.conftest import ROOT


def test_conversions_round_like_the_conversion_instructions():
    src = os.path.join(ROOT, "tests", "native", "int_float_check.cpp")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "int_float_check")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                        os.path.join(ROOT, "lighthugger_gb300", "csrc"), src, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout


def test_edge_runs_hold_exactly_the_covered_pixels():
    """lighthugger_gb300/csrc/edge_run.cuh (the big-triangle chunks' runs of
    covered pixels) against the per-pixel edge tests, host-compiled."""
    src = os.path.join(ROOT, "tests", "native", "edge_run_check.cpp")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "edge_run_check")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                        os.path.join(ROOT, "lighthugger_gb300", "csrc"), src, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout


def test_sphere_box_skips_only_meshlets_without_pixel_centres():
    """lighthugger_gb300/csrc/sphere_box.cuh (the raster's skip of meshlets
    whose world sphere reaches no pixel centre): sampled points of every
    skipped sphere, through the raster's transform and snap, reach none."""
    src = os.path.join(ROOT, "tests", "native", "sphere_box_check.cpp")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "sphere_box_check")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                        os.path.join(ROOT, "lighthugger_gb300", "csrc"), "-I", os.path.join(ROOT, "include"), src,
                        "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout


def test_column_quotient_from_the_reciprocal_is_the_ieee_quotient():
    """lighthugger_gb300/csrc/exact_div.cuh (the resolve's x / W from 1 / W
    and its PCF sum / 9, with Markstein's correction step) against the IEEE
    quotient for every 0 <= x <= W <= 16384 and every float in [0, 9] over
    9, host-compiled."""
    src = os.path.join(ROOT, "tests", "native", "exact_div_check.cpp")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "exact_div_check")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-pthread", "-I",
                        os.path.join(ROOT, "lighthugger_gb300", "csrc"), src, "-o", exe], check=True)
        r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout
