"""ttsh_step_noalloc: the step for callers that cannot allocate device memory.

Such callers (their GPU memory is owned by another allocator or capped per process, or they
cannot afford cudaFree's device-wide wait) hand in their own device arrays; the step's working
memory is a fixed array inside libttsh. These tests call the entry point through the C ABI twice
in a row on device buffers the test owns and check each result against the regular entry points
(ttsh_create / ttsh_set_state / ttsh_step / ttsh_get_state) run on the same inputs: the two paths
run the same kernels in the same order, so the results must be identical bit for bit (the FP64
tolerance of the other GPU tests, 1e-11 relative L2, would hide a changed kernel). Sizes from the
smallest (8) to the largest the working array holds (32, which fills it), with and without the
stale-halo quirk, on torch's current stream and on a non-blocking stream. Kept in its own file,
collected last.
"""
import ctypes

import numpy as np
import pytest

from conftest import random_state

pytestmark = pytest.mark.gpu


def _regular(inp, ext, st, counts):
    import ttsh
    out = []
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        for k in counts:
            s.step(k)
            w = s.get_state(0)
            w["us"], w["ps"] = s.get_provisional(0)
            out.append(w)
    return out


@pytest.mark.parametrize("N,quirks,nonblocking", [(8, 1, False), (24, 1, False), (32, 1, False), (32, 0, False),
                                                  (24, 0, True), (32, 1, True)])
def test_step_noalloc_matches_step_two_calls(N, quirks, nonblocking):
    import torch
    import ttsh

    st = random_state(N, seed=77 + N)
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=64, zeta=0.02, quirks=quirks)
    want = _regular(inp, ext, st, (3, 2))  # 3 steps, then 2 more

    dev = torch.device("cuda", 0)
    d = {k: torch.tensor(st[k], device=dev, dtype=torch.float64) for k in ("phi", "P", "u", "us", "ps")}
    d["pv"] = torch.zeros((N, N, N), device=dev, dtype=torch.float64)
    d["pp"] = torch.zeros((N, N, N), device=dev, dtype=torch.float64)
    torch.cuda.synchronize(dev)  # the buffers are ready before a stream that does not wait for others
    stream = torch.cuda.Stream(dev) if nonblocking else torch.cuda.current_stream(dev)
    lib = ttsh.lib()

    def call(nsteps):
        rc = lib.ttsh_step_noalloc(ctypes.byref(inp), ctypes.byref(ext), nsteps, d["phi"].data_ptr(),
                                   d["P"].data_ptr(), d["u"].data_ptr(), d["us"].data_ptr(), d["ps"].data_ptr(),
                                   d["pv"].data_ptr(), d["pp"].data_ptr(), stream.cuda_stream)
        assert rc == ttsh.OK, lib.ttsh_last_error().decode()
        stream.synchronize()

    for nsteps, w in zip((3, 2), want):
        call(nsteps)
        for k in ("phi", "P", "u", "pv", "pp", "us", "ps"):
            got = d[k].cpu().numpy()
            assert np.array_equal(got, w[k]), (nsteps, k, float(np.abs(got - w[k]).max()))


def test_step_noalloc_rejects_sizes_beyond_its_working_memory():
    import torch
    import ttsh
    N = 36  # > TTSH_NOALLOC_MAX_N (32)
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=64)
    buf = torch.zeros(3 * N ** 3, device="cuda", dtype=torch.float64)
    p = buf.data_ptr()
    rc = ttsh.lib().ttsh_step_noalloc(ctypes.byref(inp), ctypes.byref(ext), 1, p, p, p, p, p, p, p, None)
    assert rc == ttsh.E_UNSUPPORTED
    assert b"outside" in ttsh.lib().ttsh_last_error()


_FRESH = r"""
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[2])
import ttsh
from conftest import random_state
N = 24
st = random_state(N, seed=78)
inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
ext = ttsh.default_ext(precision=64, zeta=0.02)
dev = torch.device("cuda", 0)
d = {k: torch.tensor(st[k], device=dev, dtype=torch.float64) for k in ("phi", "P", "u", "us", "ps")}
d["pv"] = torch.zeros((N, N, N), device=dev, dtype=torch.float64)
d["pp"] = torch.zeros((N, N, N), device=dev, dtype=torch.float64)
lib = ttsh.lib()
# the no-allocation step first: nothing else in this process has prepared size N
rc = lib.ttsh_step_noalloc(ctypes.byref(inp), ctypes.byref(ext), 2, d["phi"].data_ptr(), d["P"].data_ptr(),
                           d["u"].data_ptr(), d["us"].data_ptr(), d["ps"].data_ptr(), d["pv"].data_ptr(),
                           d["pp"].data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
assert rc == ttsh.OK, lib.ttsh_last_error().decode()
torch.cuda.synchronize(dev)
got = {k: d[k].cpu().numpy() for k in ("phi", "P", "u", "pv", "pp")}
with ttsh.Sim(inp, ext) as s:
    s.set_state(0, st["phi"], st["P"], st["u"], st["us"], st["ps"])
    s.step(2)
    want = s.get_state(0)
for k in got:
    assert np.array_equal(got[k], want[k]), (k, float(np.abs(got[k] - want[k]).max()))
print("ok")
"""


def test_step_noalloc_first_in_a_fresh_process():
    """The no-allocation step prepares everything its kernels read (the FFT's constant twiddle
    table included) by itself: run first in a fresh process, before any ttsh_create of the size,
    it still matches the regular entry points."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "-c", _FRESH, os.path.join(root, "bacterial-droplet_gb300"),
                          os.path.join(root, "tests")], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0 and out.stdout.strip().endswith("ok"), out.stdout[-2000:] + out.stderr[-2000:]
