"""The asynchronous snapshot writer (ttsh_write_conf_async): the file it writes while later steps
run is byte for byte the one ttsh_write_conf writes for the same state (itself byte-identical to
the reference's ExpoConf output, tests/test_boundary.py), in the fused FP32 and the FP64 forms;
and the call returns before the text is formatted."""
import os
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _sim(ttsh, N, precision):
    phi, P = ttsh.init_droplet(N, N / 4.0, 2.0, 3)
    s = ttsh.Sim(ttsh.default_input(Nx=N, Ny=N, Nz=N), ttsh.default_ext(precision=precision, zeta=0.02))
    s.set_state(0, phi, P, np.zeros_like(P))
    return s


@pytest.mark.parametrize("N,precision", [(32, 32), (16, 64)])
def test_async_snapshot_is_the_sync_one(tmp_path, N, precision):
    import ttsh
    a, b = str(tmp_path / "a.dat"), str(tmp_path / "b.dat")
    with _sim(ttsh, N, precision) as s:
        s.step(3)
        s.write_conf(0, a)
    with _sim(ttsh, N, precision) as s:
        s.step(3)
        s.write_conf_async(0, b)
        s.step(5)  # the snapshot holds the state of step 3 whatever runs after it
        s.conf_wait()
    assert open(a, "rb").read() == open(b, "rb").read()


def test_async_snapshot_overlaps_the_steps(tmp_path):
    import ttsh
    N = 128
    with _sim(ttsh, N, 32) as s:
        s.step(2)
        p = str(tmp_path / "warm.dat")
        s.write_conf(0, p)  # buffer allocated, formatter warm
        t0 = time.perf_counter()
        s.write_conf(0, str(tmp_path / "sync.dat"))
        t_sync = time.perf_counter() - t0
        t0 = time.perf_counter()
        s.write_conf_async(0, str(tmp_path / "async.dat"))
        t_call = time.perf_counter() - t0
        s.step(10)
        s.conf_wait()
    assert os.path.getsize(str(tmp_path / "async.dat")) == os.path.getsize(str(tmp_path / "sync.dat"))
    assert t_call < 0.5 * t_sync, (t_call, t_sync)
