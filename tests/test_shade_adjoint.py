"""The resolve's hand-written adjoint (lighthugger_gb300/csrc/shade.cuh),
compiled for the host in double precision, against central differences of
the same forward: vertex positions, normals, uvs, base-colour factor, the
texels of both bilinear samples, light direction and colour."""
import os
import subprocess
import tempfile

from tests.conftest import ROOT


def test_adjoint_matches_central_differences():
    src = os.path.join(ROOT, "tests", "native", "shade_check.cpp")
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "shade_check")
        subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I",
                        os.path.join(ROOT, "lighthugger_gb300", "csrc"), src, "-o", exe], check=True)
        r = subprocess.run([exe, "400"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout
