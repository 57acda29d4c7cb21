"""Cross-check of libttsh's FFT projection against cuFFT (through torch.fft on the GPU).

The reference solves the Poisson problem with cuFFT (getP / getStream, TTSH3D.cu:635-691;
plan at :1123). libttsh uses its own FFT kernels; cuFFT is kept only as this check. After one
step, the provisional fields u*, P* and the pressures p_v, p_p are read back; the projection is
recomputed in FP64 on the GPU with cuFFT from those u*, P*:

    src = D.u*/dt + i D.P*/dt        (27-point D, periodic; stale-halo quirk off)
    p   = ifft( -fft(src) / k^2 )    (continuous k^2 of initPoissonSolver, k2[0] = 1)

Tolerances (relative L2, written in the asserts): the FP64 form 1e-12; the FP32 fused form 2e-5
(its divergence, FFT and divide run in FP32 on the same FP32 u*, P*).
"""
import numpy as np
import pytest

from conftest import random_state

pytestmark = pytest.mark.gpu


def relerr(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def cufft_projection(us, ps, h, dt):
    import torch
    dev = torch.device("cuda", 0)
    N = us.shape[1]

    def D(f, axis):
        # (1/(2h)) (1/36) delta_a s_b s_c f, s = [1, 4, 1]; arrays are [z][y][x]
        def s(g, ax):
            return torch.roll(g, 1, ax) + 4 * g + torch.roll(g, -1, ax)
        d = torch.roll(f, -1, axis) - torch.roll(f, 1, axis)
        for ax in (0, 1, 2):
            if ax != axis:
                d = s(d, ax)
        return d / (2 * h) / 36

    def div(v):
        t = torch.as_tensor(v, dtype=torch.float64, device=dev)
        return D(t[0], 2) + D(t[1], 1) + D(t[2], 0)

    src = torch.complex(div(us) / dt, div(ps) / dt)
    m = torch.arange(N, device=dev, dtype=torch.float64)
    k = 2 * np.pi * torch.where(m < N // 2, m, m - N) / (N * h)
    k2 = k[:, None, None] ** 2 + k[None, :, None] ** 2 + k[None, None, :] ** 2
    k2[0, 0, 0] = 1.0
    p = torch.fft.ifftn(-torch.fft.fftn(src) / k2)
    return p.real.cpu().numpy(), p.imag.cpu().numpy()


@pytest.mark.parametrize("precision,N,tol", [(64, 32, 1e-12), (64, 48, 1e-12), (32, 64, 2e-5), (32, 128, 2e-5)])
def test_projection_matches_cufft(precision, N, tol):
    import ttsh
    st = random_state(N, seed=N + 3)
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=precision, quirks=0, zeta=0.02)
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        s.step(3)
        g = s.get_state(0)
        us, ps = s.get_provisional(0)
    pv, pp = cufft_projection(us, ps, inp.h, inp.dt0)
    assert relerr(g["pv"], pv) <= tol, relerr(g["pv"], pv)
    assert relerr(g["pp"], pp) <= tol, relerr(g["pp"], pp)
