"""The C++ drop-in (include/swc/DualParticleSphLiquid.hpp) runs the 2D dam break on the GPU."""
import os
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def test_cpp_dam_break_example(tmp_path):
    from swc import build

    exe = [e for e in build.build_examples() if e.endswith("dam_break_2d")][0]
    r = subprocess.run([exe, "5"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("step")]
    assert len(lines) == 5
    for l in lines:
        cg = int(l.split("cg")[1].split()[0])
        res = float(l.split("|r|/|b|")[1].split()[0])
        assert 0 < cg < 400 and res < 1e-6
    n = os.path.getsize(tmp_path / "dam_break_2d_out" / "last" / "particles.sav")
    assert n == 3200 * 2 * 8


def test_cpp_sand_rotating_box_example(tmp_path):
    """include/swc/DEMParticleSand.hpp: the builder's 2D scene, 5 frames of CFL-limited steps."""
    from swc import build

    exe = [e for e in build.build_examples() if e.endswith("sand_rotating_box_2d")][0]
    r = subprocess.run([exe, "5"], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("frame")]
    assert len(lines) == 5
    n = int(lines[0].split(" N ")[1].split()[0])
    assert n == 247  # the builder's box at scale 30 (tests/test_sand_oracle.py counts the same packing)
    vmax = [float(l.split("max|v|")[1]) for l in lines]
    assert all(0.2 < v < 0.5 for v in vmax)  # rigid rotation at 2 rad/s plus 1e-4 s of gravity per frame
    assert os.path.getsize(tmp_path / "sand_rotating_box_2d_out" / "last" / "particles.sav") == n * 2 * 8
    assert os.path.getsize(tmp_path / "sand_rotating_box_2d_out" / "last" / "particles.mesh") == 4 + n * 12
