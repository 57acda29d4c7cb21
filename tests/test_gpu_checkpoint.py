"""Checkpoint / resume: 6 steps in one go equal 3 steps, a checkpoint, a fresh handle, a load and
3 more steps, bit for bit, in both precisions (fused FP32 and plain FP64)."""
import numpy as np
import pytest

from conftest import random_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,N", [(64, 16), (32, 32)])
def test_checkpoint_resume_is_exact(tmp_path, precision, N):
    import ttsh
    st = random_state(N, seed=41)
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=precision, zeta=0.02)
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        s.step(6)
        want = s.get_state(0)
    ck = str(tmp_path / "ck.bin")
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        s.step(3)
        s.save_checkpoint(0, ck)
        t3 = s.time()
    with ttsh.Sim(inp, ext) as s:
        s.load_checkpoint(0, ck)
        assert s.time() == t3
        s.step(3)
        got = s.get_state(0)
    for k in ("phi", "P", "u", "pv", "pp"):
        assert np.array_equal(got[k], want[k]), k


def test_checkpoint_rejects_mismatch(tmp_path):
    import ttsh
    st = random_state(16, seed=1)
    ck = str(tmp_path / "ck.bin")
    with ttsh.Sim(ttsh.default_input(Nx=16, Ny=16, Nz=16), ttsh.default_ext(precision=64)) as s:
        s.set_state(0, st["phi"], st["P"], st["u"])
        s.save_checkpoint(0, ck)
    with ttsh.Sim(ttsh.default_input(Nx=32, Ny=32, Nz=32), ttsh.default_ext(precision=64)) as s:
        with pytest.raises(ttsh.TTSHError) as e:
            s.load_checkpoint(0, ck)
        assert e.value.code == ttsh.E_INVALID
    (tmp_path / "junk.bin").write_bytes(b"not a checkpoint at all")
    with ttsh.Sim(ttsh.default_input(Nx=16, Ny=16, Nz=16), ttsh.default_ext(precision=64)) as s:
        with pytest.raises(ttsh.TTSHError) as e:
            s.load_checkpoint(0, str(tmp_path / "junk.bin"))
        assert e.value.code == ttsh.E_PARSE
