"""The host interface's two routes for FP64 host arrays: page-locked arrays are read and written in
place by the conversion kernels (and, for the strided FP64 pressures, a gather kernel); pageable
ones are staged by the copy engines. Both must give the same bits, in every form, for the
state, the pressures and the provisional fields; and the page-locked route must move the state
at >= 100 GB/s."""
import time

import numpy as np
import pytest

from conftest import random_state

pytestmark = pytest.mark.gpu

NAMES = ("phi", "P", "u", "pv", "pp")


def _pinned(shape):
    import torch
    t = torch.zeros(shape, dtype=torch.float64, pin_memory=True)
    return t, t.numpy()


def _roundtrip(ttsh, st, precision, form, pinned, steps=2):
    N = st["phi"].shape[0]
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=precision, zeta=0.02, form=form)
    keep = []

    def host(a):
        if not pinned:
            return np.ascontiguousarray(a, np.float64)
        t, v = _pinned(a.shape)
        v[...] = a
        keep.append(t)
        return v

    with ttsh.Sim(inp, ext) as s:
        args = [host(st[k]) for k in ("phi", "P", "u", "us", "ps")]
        ttsh._check(ttsh.lib().ttsh_set_state(s.handle, 0, *[ttsh._p(a) for a in args]))
        s.step(steps)
        outs = {}
        for k, shp in (("phi", (N, N, N)), ("P", (3, N, N, N)), ("u", (3, N, N, N)), ("pv", (N, N, N)),
                       ("pp", (N, N, N)), ("us", (3, N, N, N)), ("ps", (3, N, N, N))):
            if pinned:
                t, v = _pinned(shp)
                keep.append(t)
            else:
                v = np.empty(shp)
            outs[k] = v
        ttsh._check(ttsh.lib().ttsh_get_state(s.handle, 0, *[ttsh._p(outs[k]) for k in NAMES]))
        ttsh._check(ttsh.lib().ttsh_get_provisional(s.handle, 0, ttsh._p(outs["us"]), ttsh._p(outs["ps"])))
        return {k: v.copy() for k, v in outs.items()}


@pytest.mark.parametrize("precision,form", [(64, 1), (32, 1), (32, 2)])
def test_pinned_and_pageable_routes_agree(precision, form):
    import ttsh
    st = random_state(32, seed=77)
    a = _roundtrip(ttsh, st, precision, form, pinned=True)
    b = _roundtrip(ttsh, st, precision, form, pinned=False)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_pinned_state_transfer_rate():
    """set_state + get_state of two 256^3 droplets in the fused FP32 form from and into
    page-locked FP64 arrays: 2 x 7 fields x 128 MiB each way, >= 100 GB/s each way."""
    import torch
    import ttsh
    N = 256
    phi, P = ttsh.init_droplet(N, 64.0, 2.0, 1)
    inps = [ttsh.default_input(Nx=N, Ny=N, Nz=N)] * 2
    exts = [ttsh.default_ext(precision=32, zeta=z, form=ttsh.FORM_FUSED) for z in (0.005, 0.02)]
    _, hphi = _pinned((N, N, N))
    _, hP = _pinned((3, N, N, N))
    _, hu = _pinned((3, N, N, N))
    hphi[...] = phi
    hP[...] = P
    with ttsh.Sim(inps, exts) as s:
        for i in range(2):  # warm-up: first-use allocations
            s.set_state(i, hphi, hP, hu)
        s.step(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in range(2):
            s.set_state(i, hphi, hP, hu)
        t1 = time.perf_counter()
        for i in range(2):
            ttsh._check(ttsh.lib().ttsh_get_state(s.handle, i, ttsh._p(hphi), ttsh._p(hP), ttsh._p(hu), None, None))
        s.sync()
        t2 = time.perf_counter()
    nbytes = 2 * 7 * N ** 3 * 8
    up, down = nbytes / (t1 - t0) / 1e9, nbytes / (t2 - t1) / 1e9
    print("set_state %.0f GB/s, get_state %.0f GB/s" % (up, down))
    assert up >= 100 and down >= 100, (up, down)
