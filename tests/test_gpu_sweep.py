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
