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


def test_snapshot_mode_is_offered():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                         timeout=300)
    assert out.returncode == 0 and "--snapshot" in out.stdout and "--snapshot-n" in out.stdout


def test_reference_input_with_T0_skips_nothing_else():
    """The reference program's input.dat writer (pure Python, used by the reference arm and the
    snapshot measurement): T0 lands on the 15th token and every other token keeps the reference
    defaults except N, Ts, dte."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_ref_golden as G
    base = open(os.path.join(ROOT, "tests", "golden", "input_default.dat")).read().split()
    tok = G.reference_input_text(64, 0.007, 0.005, expo=1, T0=1e-06).split()
    assert len(tok) == len(base)
    assert tok[14] == "1e-06" and tok[8:11] == ["64"] * 3 and tok[15] == "0.007" and tok[16] == "0.005"
    assert all(tok[i] == base[i] for i in range(len(base)) if i not in (8, 9, 10, 14, 15, 16))
