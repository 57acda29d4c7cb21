"""ttsh_step_noalloc: the step for callers that cannot allocate device memory.

Such callers (their GPU memory is owned by another allocator or capped per process, or they
cannot afford cudaFree's device-wide wait) hand in their own device arrays; the step's working
memory is a fixed array inside libttsh. This test calls the entry point through the C ABI twice
in a row on device buffers the test owns and checks each result against the regular entry points
(ttsh_create / ttsh_set_state / ttsh_step / ttsh_get_state) run on the same inputs. Tolerance:
1e-11 relative L2 per field, the FP64 tolerance of the other GPU tests (the two paths run the same
kernels, so the results are expected to agree exactly). Kept in its own file, collected last.
"""
import ctypes

import numpy as np
import pytest

from conftest import random_state

pytestmark = pytest.mark.gpu

TOL = 1e-11


def _rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def test_step_noalloc_matches_step_two_calls():
    import torch
    import ttsh

    N = 24
    st = random_state(N, seed=77)
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=64, zeta=0.02)

    # regular entry points: 3 steps, then 2 more
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        s.step(3)
        want1 = s.get_state(0)
        want1["us"], want1["ps"] = s.get_provisional(0)
        s.step(2)
        want2 = s.get_state(0)
        want2["us"], want2["ps"] = s.get_provisional(0)

    dev = torch.device("cuda", 0)
    d = {
        "phi": torch.tensor(st["phi"], device=dev, dtype=torch.float64),
        "P": torch.tensor(st["P"], device=dev, dtype=torch.float64),
        "u": torch.tensor(st["u"], device=dev, dtype=torch.float64),
        "us": torch.tensor(st["us"], device=dev, dtype=torch.float64),
        "ps": torch.tensor(st["ps"], device=dev, dtype=torch.float64),
        "pv": torch.zeros((N, N, N), device=dev, dtype=torch.float64),
        "pp": torch.zeros((N, N, N), device=dev, dtype=torch.float64),
    }
    stream = torch.cuda.current_stream(dev).cuda_stream
    lib = ttsh.lib()

    def call(nsteps):
        rc = lib.ttsh_step_noalloc(ctypes.byref(inp), ctypes.byref(ext), nsteps, d["phi"].data_ptr(),
                                   d["P"].data_ptr(), d["u"].data_ptr(), d["us"].data_ptr(), d["ps"].data_ptr(),
                                   d["pv"].data_ptr(), d["pp"].data_ptr(), stream)
        assert rc == ttsh.OK, lib.ttsh_last_error().decode()
        torch.cuda.synchronize(dev)

    for nsteps, want in ((3, want1), (2, want2)):
        call(nsteps)
        got = {"phi": d["phi"].cpu().numpy(), "P": d["P"].cpu().numpy(), "u": d["u"].cpu().numpy(),
               "pv": d["pv"].cpu().numpy(), "pp": d["pp"].cpu().numpy(), "us": d["us"].cpu().numpy(),
               "ps": d["ps"].cpu().numpy()}
        errs = {k: _rel(got[k], want[k]) for k in got}
        assert max(errs.values()) <= TOL, (nsteps, errs)


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
    nb = np.linalg.norm(want[k])
    err = float(np.linalg.norm(got[k] - want[k]) / (nb if nb > 0 else 1.0))
    assert err <= 1e-11, (k, err)
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
