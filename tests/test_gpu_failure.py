"""Failure detection without a GPU fault: a bounded device wait that runs out is reported.

The staged z pass of the FFT (TTSH_ZTMA=1, 256^3) waits for each TMA copy on an mbarrier for a
bounded number of SM clocks; when the limit runs out it sets the handle's device error word, waits
for its copies still in flight and returns, and ttsh_sync reports TTSH_E_CUDA. The test makes the
wait run out with the test hook TTSH_TEST_DROP_STAGED_COPY=1: every CTA skips its first copy (a
barrier that nothing completes) and waits with a short limit. Nothing faults or hangs; the
context stays usable, which the test checks by running steps on a fresh handle afterwards.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _droplet_sim(ttsh, N=256):
    phi, P = ttsh.init_droplet(N, N / 4.0, 2.0, 1)
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=32, zeta=0.02, form=ttsh.FORM_FUSED)
    s = ttsh.Sim(inp, ext)
    s.set_state(0, phi, P, np.zeros_like(P))
    return s


def test_expired_wait_is_reported_and_the_context_survives(monkeypatch):
    import ttsh
    monkeypatch.setenv("TTSH_ZTMA", "1")
    monkeypatch.setenv("TTSH_TEST_DROP_STAGED_COPY", "1")
    with _droplet_sim(ttsh) as s:
        s.step(1)
        rc = ttsh.lib().ttsh_sync(s.handle)
        assert rc == ttsh.E_CUDA, rc
        assert b"timed out" in ttsh.lib().ttsh_last_error()
    monkeypatch.delenv("TTSH_TEST_DROP_STAGED_COPY")
    with _droplet_sim(ttsh) as s:
        s.step(2)
        s.sync()
        st = s.reduce(0)
        assert st["nonfinite"] == 0


def test_staged_z_pass_without_the_hook_reports_nothing(monkeypatch):
    import ttsh
    monkeypatch.setenv("TTSH_ZTMA", "1")
    monkeypatch.delenv("TTSH_TEST_DROP_STAGED_COPY", raising=False)
    with _droplet_sim(ttsh) as s:
        s.step(2)
        assert ttsh.lib().ttsh_sync(s.handle) == ttsh.OK
