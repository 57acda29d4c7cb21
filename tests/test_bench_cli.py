"""bench.py's command line and workloads, without a GPU: the options the driver passes parse,
and the named workloads have the droplet sizes and counts the measurements are quoted on."""
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_help_lists_the_driver_options():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0, out.stderr
    for opt in ("--gpus", "--steps", "--warmup", "--impl", "--workload"):
        assert opt in out.stdout, opt


def test_workloads():
    sys.path.insert(0, ROOT)
    import bench
    sizes = {name: [d[0] for d in bench.workload(name)] for name in ("2x256", "1x256", "64x128", "24mixed", "1x512")}
    assert sizes["2x256"] == [256, 256] and sizes["1x256"] == [256] and sizes["1x512"] == [512]
    assert sizes["64x128"] == [128] * 64
    assert sorted(set(sizes["24mixed"])) == [96, 128, 160, 192] and len(sizes["24mixed"]) == 24
    # every droplet of a workload is a fused-form size (a multiple of 32) with a positive radius
    for name in sizes:
        for (N, R, xi, seed, zeta) in bench.workload(name):
            assert N % 32 == 0 and 0 < R < N / 2 and xi > 0 and zeta >= 0
