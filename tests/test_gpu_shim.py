"""The drop-in TTSH3D.cu shim, compiled with run_cuda.pl's own nvcc line and run the way
run_cuda.pl runs the reference (cwd holding data_<gpu_node>/input.dat), against the reference
program itself run the same way with the same seed: the same snapshot files, the same cadence,
the same values (1e-12 absolute on O(1) fields printed with 15 decimals)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import PKG

pytestmark = pytest.mark.gpu

# run_cuda.pl:4
NVCC_LINE = ["-std=c++14", "-I", "/usr/include/cuda/", "-L", "/usr/lib64/", "--cudart=shared", "-lcufft"]


def _nvcc():
    return shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"


def _run_dir(d, binary, env_extra, N, Ts, dte):
    import ttsh
    os.makedirs(os.path.join(d, "data_1"), exist_ok=True)
    ttsh.write_input(os.path.join(d, "data_1", "input.dat"), ttsh.default_input(Nx=N, Ny=N, Nz=N, Ts=Ts, dte=dte))
    env = dict(os.environ)
    env.update(env_extra)
    r = subprocess.run([binary], cwd=d, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return sorted(f for f in os.listdir(os.path.join(d, "data_1")) if f.startswith("conf_")), r.stdout


def test_shim_matches_reference_program(tmp_path):
    import sys
    import ttsh
    sys.path.insert(0, os.path.join(os.path.dirname(PKG), "oracle"))
    import make_ref
    ttsh.lib()
    ref_bin = make_ref.build()
    if ref_bin is None:
        pytest.skip("patched reference source not present")
    shim_dir = tmp_path / "shim"
    shim_dir.mkdir()
    shutil.copy(os.path.join(PKG, "shim", "TTSH3D.cu"), shim_dir / "TTSH3D.cu")
    subprocess.check_call([_nvcc()] + NVCC_LINE + ["TTSH3D.cu", "-o", "TTSH3D.out"], cwd=shim_dir)
    N, Ts, dte = 16, 0.019, 0.006
    env = {"TTSH_SEED": "4321", "TTSH_LIB": os.path.join(PKG, "lib", "libttsh.so")}
    shim_files, shim_out = _run_dir(str(shim_dir), str(shim_dir / "TTSH3D.out"), env, N, Ts, dte)
    ref_dir = tmp_path / "ref"
    ref_dir.mkdir()
    ref_files, _ = _run_dir(str(ref_dir), ref_bin, env, N, Ts, dte)
    assert shim_files == ref_files and len(ref_files) >= 3, (shim_files, ref_files)
    assert "Simulation finished." in shim_out
    for f in ref_files:
        a = np.loadtxt(shim_dir / "data_1" / f)
        b = np.loadtxt(ref_dir / "data_1" / f)
        assert a.shape == b.shape == (N ** 3, 7), f
        assert np.abs(a - b).max() <= 1e-12, (f, np.abs(a - b).max())


def test_shim_reports_bad_input(tmp_path):
    shim_dir = tmp_path / "shim"
    shim_dir.mkdir()
    shutil.copy(os.path.join(PKG, "shim", "TTSH3D.cu"), shim_dir / "TTSH3D.cu")
    subprocess.check_call([_nvcc()] + NVCC_LINE + ["TTSH3D.cu", "-o", "TTSH3D.out"], cwd=shim_dir)
    (shim_dir / "data_1").mkdir()
    (shim_dir / "data_1" / "input.dat").write_text("1\n2\n3\n")
    env = dict(os.environ, TTSH_LIB=os.path.join(PKG, "lib", "libttsh.so"))
    r = subprocess.run([str(shim_dir / "TTSH3D.out")], cwd=shim_dir, env=env, capture_output=True, text=True)
    assert r.returncode == 0
    assert "Error while reading the input file!" in r.stdout
