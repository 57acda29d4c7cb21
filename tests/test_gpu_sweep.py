"""The batched sweep driver (ttsh_run_dirs) against one-directory runs: droplets of different
sizes and constants advanced together write byte-identical conf_<te>.dat files, at the same times."""
import os

import pytest

pytestmark = pytest.mark.gpu


def _make(d, **kw):
    import ttsh
    os.makedirs(d, exist_ok=True)
    ttsh.write_input(os.path.join(d, "input.dat"), ttsh.default_input(**kw))


def test_run_dirs_batch_equals_single_runs(tmp_path):
    import ttsh
    specs = [dict(Nx=16, Ny=16, Nz=16, Ts=0.011, dte=0.004, eta=-0.187),
             dict(Nx=24, Ny=24, Nz=24, Ts=0.007, dte=0.002, eta=-0.25),
             dict(Nx=16, Ny=16, Nz=16, Ts=0.009, dte=0.006, kappa=-0.5, dt0=0.001)]
    batch = [str(tmp_path / ("b%d" % i)) for i in range(len(specs))]
    single = [str(tmp_path / ("s%d" % i)) for i in range(len(specs))]
    for i, sp in enumerate(specs):
        _make(batch[i], **sp)
        _make(single[i], **sp)
    ttsh.run_dirs(batch, seed=100)
    for i in range(len(specs)):
        ttsh.run_dirs([single[i]], seed=100 + i)
    for i in range(len(specs)):
        fb = sorted(f for f in os.listdir(batch[i]) if f.startswith("conf_"))
        fs = sorted(f for f in os.listdir(single[i]) if f.startswith("conf_"))
        assert fb == fs and len(fb) >= 2, (i, fb, fs)
        for f in fb:
            assert open(os.path.join(batch[i], f), "rb").read() == open(os.path.join(single[i], f), "rb").read(), f


def test_init_reference_is_deterministic():
    import numpy as np
    import ttsh
    inp = ttsh.default_input(Nx=8, Ny=8, Nz=8)
    a = ttsh.init_reference(inp, 7)
    b = ttsh.init_reference(inp, 7)
    c = ttsh.init_reference(inp, 8)
    assert all(np.array_equal(a[k], b[k]) for k in a)
    assert not np.array_equal(a["u"], c["u"])
    assert np.abs(a["u"]).max() <= 0.5e-4 + 1e-18


def test_run_dirs_with_autotuning(tmp_path, monkeypatch):
    """TTSH_TUNE=1 makes the sweep driver tune the batch on its initial fields and record the
    choices in TTSH_TUNE_CACHE; the snapshots agree with untuned runs (the FFT choice changes
    FP64 rounding only)."""
    import numpy as np
    import ttsh
    specs = [dict(Nx=16, Ny=16, Nz=16, Ts=0.009, dte=0.004), dict(Nx=24, Ny=24, Nz=24, Ts=0.007, dte=0.004)]
    tuned = [str(tmp_path / ("t%d" % i)) for i in range(len(specs))]
    plain = [str(tmp_path / ("p%d" % i)) for i in range(len(specs))]
    for i, sp in enumerate(specs):
        _make(tuned[i], **sp)
        _make(plain[i], **sp)
    cache = str(tmp_path / "tune.txt")
    monkeypatch.setenv("TTSH_TUNE", "1")
    monkeypatch.setenv("TTSH_TUNE_CACHE", cache)
    ttsh.run_dirs(tuned, seed=7)
    monkeypatch.delenv("TTSH_TUNE")
    monkeypatch.delenv("TTSH_TUNE_CACHE")
    ttsh.run_dirs(plain, seed=7)
    lines = open(cache).read().splitlines()
    assert len(lines) == 2 and all(" N16 " in l or " N24 " in l for l in lines), lines
    for i in range(len(specs)):
        files = sorted(f for f in os.listdir(plain[i]) if f.startswith("conf_"))
        assert files == sorted(f for f in os.listdir(tuned[i]) if f.startswith("conf_")) and len(files) >= 2
        for f in files:
            a = np.loadtxt(os.path.join(tuned[i], f))
            b = np.loadtxt(os.path.join(plain[i], f))
            np.testing.assert_allclose(a, b, rtol=0, atol=1e-12)


def test_run_dirs_matches_the_reference_program(tmp_path):
    """forEach.pl's sweep (one TTSH3D.out per directory, forEach.pl:33-44, :131) against the batched
    driver: three directories with different sizes, constants and cadences, each run by the
    reference program itself (seeded as the shim is, TTSH_SEED) and all three by one ttsh_run_dirs
    call with the same seeds: the same snapshot files with the same values (1e-12 absolute on
    fields printed with 15 decimals)."""
    import subprocess
    import sys

    import numpy as np
    import ttsh
    from conftest import ROOT
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import make_ref
    ttsh.lib()
    ref_bin = make_ref.build()
    if ref_bin is None:
        pytest.skip("patched reference source not present")
    specs = [dict(Nx=16, Ny=16, Nz=16, Ts=0.011, dte=0.004, eta=-0.187),
             dict(Nx=24, Ny=24, Nz=24, Ts=0.007, dte=0.002, eta=-0.25),
             dict(Nx=16, Ny=16, Nz=16, Ts=0.009, dte=0.006, kappa=-0.5, dt0=0.001)]
    seed = 500
    ours = []
    for i, sp in enumerate(specs):
        d = str(tmp_path / ("sweep%d" % i) / "data_1")
        _make(d, **sp)
        ours.append(d)
        ref_root = tmp_path / ("ref%d" % i)
        _make(str(ref_root / "data_1"), **sp)
        env = dict(os.environ, TTSH_SEED=str(seed + i))
        r = subprocess.run([ref_bin], cwd=str(ref_root), env=env, capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    ttsh.run_dirs(ours, seed=seed)
    for i in range(len(specs)):
        rd = str(tmp_path / ("ref%d" % i) / "data_1")
        fr = sorted(f for f in os.listdir(rd) if f.startswith("conf_"))
        fo = sorted(f for f in os.listdir(ours[i]) if f.startswith("conf_"))
        assert fo == fr and len(fr) >= 2, (i, fo, fr)
        N = specs[i]["Nx"]
        for f in fr:
            a = np.loadtxt(os.path.join(ours[i], f))
            b = np.loadtxt(os.path.join(rd, f))
            assert a.shape == b.shape == (N ** 3, 7), (i, f)
            assert np.abs(a - b).max() <= 1e-12, (i, f, np.abs(a - b).max())
