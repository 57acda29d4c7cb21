"""The fused kernels' persistent work split (csrc/schedule.h, compiled here for the host with
g++): every (droplet, tile, plane) of a group is swept exactly once, in segments that stay in
one slab, for grids of 1 to 4096 CTAs, 1 to 64 droplets and N = 32 ... 512 (tests/schedule_check.cpp)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_persistent_split_covers_every_site_once(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "schedule_check")
    subprocess.check_call([gxx, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "bacterial-droplet_gb300", "csrc"),
                           os.path.join(ROOT, "tests", "schedule_check.cpp"), "-o", exe])
    out = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.startswith("ok"), out.stdout + out.stderr
