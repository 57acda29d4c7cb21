"""CPU tests of the FP64 oracle: known answers, an independent numpy restatement, and the
golden vectors produced by the reference program itself (tests/golden/ref_N12.npz)."""
import os

import numpy as np
import pytest

import np_restatement as R
from conftest import GOLDEN

KERNEL_FIELDS = ["phi", "px", "py", "pz", "vx", "vy", "vz", "vxs", "vys", "vzs", "pxs", "pys", "pzs", "pv", "pp"]


@pytest.mark.parametrize("N", [8, 12, 20, 30, 32, 48])
def test_fft_matches_numpy(oracle_mod, N):
    rng = np.random.default_rng(N)
    c = rng.standard_normal((N, N, N)) + 1j * rng.standard_normal((N, N, N))
    f = oracle_mod.fft3(c, -1)
    ref = np.fft.fftn(c)
    assert np.abs(f - ref).max() <= 1e-13 * np.abs(ref).max()
    back = oracle_mod.fft3(f, +1) / N ** 3
    assert np.abs(back - c).max() <= 1e-13
    # Parseval
    assert abs(np.vdot(f, f).real / N ** 3 - np.vdot(c, c).real) <= 1e-11 * np.vdot(c, c).real


def plane_wave(N, h, m):
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    k = [2 * np.pi * mm / (N * h) for mm in m]
    return np.exp(1j * (k[0] * x * h + k[1] * y * h + k[2] * z * h)), k


@pytest.mark.parametrize("m", [(2, 3, 5), (0, 1, 7), (8, 8, 8)])
def test_stencil_symbols(oracle_mod, m):
    """D_a = i sin(k_a h)/h prod_{b!=a}(2+cos k_b h)/3 and L = [(2/3) prod cos + (4/3) sum cos - 14/3]/h^2."""
    N, h = 16, 0.7
    f, k = plane_wave(N, h, m)
    c = [(2 + np.cos(kk * h)) / 3 for kk in k]
    s = [np.sin(kk * h) / h for kk in k]
    for op in range(3):
        sym = 1j * s[op] * np.prod([c[b] for b in range(3) if b != op])
        got = oracle_mod.stencil(f.real, h, op) + 1j * oracle_mod.stencil(f.imag, h, op)
        assert np.abs(got - sym * f).max() <= 1e-13
    symL = ((2 / 3) * np.prod([np.cos(kk * h) for kk in k]) + (4 / 3) * sum(np.cos(kk * h) for kk in k) - 14 / 3) / h ** 2
    got = oracle_mod.stencil(f.real, h, 3) + 1j * oracle_mod.stencil(f.imag, h, 3)
    assert np.abs(got - symL * f).max() <= 1e-12


@pytest.mark.parametrize("k2_mode", [0, 1])
def test_poisson_single_mode(oracle_mod, k2_mode):
    """u* = (A sin(k.x), 0, 0): p = -(D_x u*_x)/dt / k^2 with k^2 continuous or the D symbol squared."""
    N, h, dt, A = 16, 1.0, 0.002, 0.3
    m = (3, 1, 2)
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    k = [2 * np.pi * mm / (N * h) for mm in m]
    th = k[0] * x * h + k[1] * y * h + k[2] * z * h
    us = A * np.sin(th)
    zero = np.zeros_like(us)
    p = oracle_mod.project(us, zero, zero, h, dt, k2_mode)
    c = [(2 + np.cos(kk * h)) / 3 for kk in k]
    s = [np.sin(kk * h) / h for kk in k]
    Kx = s[0] * c[1] * c[2]
    if k2_mode == 0:
        k2 = sum(kk * kk for kk in k)
    else:
        k2 = Kx ** 2 + (c[0] * s[1] * c[2]) ** 2 + (c[0] * c[1] * s[2]) ** 2
    expect = -(A * Kx * np.cos(th)) / dt / k2
    assert np.abs(p - expect).max() <= 1e-12 * np.abs(expect).max()


def test_projection_residual(oracle_mod):
    """discrete_k2 leaves div_D u ~ 0; reference_k2 (quirk Q3) leaves most of it (white noise, 32^3)."""
    N, h, dt = 32, 1.0, 0.002
    rng = np.random.default_rng(0)
    us = [rng.standard_normal((N, N, N)) for _ in range(3)]

    def div(v):
        return sum(oracle_mod.stencil(v[a], h, a) for a in range(3))

    d0 = np.abs(div(us)).max()
    for mode, lo, hi in ((1, 0.0, 1e-12), (0, 0.5, 0.95)):
        p = oracle_mod.project(us[0], us[1], us[2], h, dt, mode)
        u = [us[a] - dt * oracle_mod.stencil(p, h, a) for a in range(3)]
        ratio = np.abs(div(u)).max() / d0
        assert lo <= ratio <= hi, (mode, ratio)


@pytest.mark.parametrize("k2_mode,stale,zeta,A", [(0, 1, 0.0, 0.0), (0, 0, 0.05, 0.3), (1, 1, 0.02, 0.0),
                                                  (1, 0, 0.0, 0.3)])
def test_oracle_matches_numpy_restatement(oracle_mod, k2_mode, stale, zeta, A):
    N = 10
    rng = np.random.default_rng(3)
    s = oracle_mod.new_state(N)
    for k in s:
        s[k][:] = 0.3 * rng.standard_normal((N, N, N))
    s["phi"][:] = rng.uniform(0, 1, (N, N, N))
    p = dict(oracle_mod.DEFAULTS)
    p.update(zeta=zeta, A=A)
    a = {k: v.copy() for k, v in s.items()}
    b = {k: v.copy() for k, v in s.items()}
    b = R.step(b, p, k2_mode=k2_mode, stale=bool(stale))
    oracle_mod.step(a, 1, N, k2_mode=k2_mode, stale_halo=stale, **p)
    for k in a:
        nb = np.abs(b[k]).max()
        assert np.abs(a[k] - b[k]).max() <= 1e-13 * max(nb, 1.0), k


def test_zeta_term_analytic(oracle_mod):
    """u* difference between zeta and zeta=0 equals -dt*zeta*D_x(phi P_x P_x) for P = (c0 + c1 sin kx, 0, 0), phi = 1."""
    N, h, dt, zeta = 16, 1.0, 0.002, 0.05
    x = np.arange(N)
    k = 2 * np.pi * 2 / N
    px1 = 0.4 + 0.3 * np.sin(k * x)
    base = oracle_mod.new_state(N)
    base["phi"][:] = 1.0
    base["px"][:] = px1[None, None, :]
    a = {kk: v.copy() for kk, v in base.items()}
    b = {kk: v.copy() for kk, v in base.items()}
    oracle_mod.step(a, 1, N, zeta=zeta, stale_halo=0)
    oracle_mod.step(b, 1, N, zeta=0.0, stale_halo=0)
    # q = px^2 = c0^2 + c1^2/2 + 2 c0 c1 sin(kx) - c1^2/2 cos(2kx); D_x symbol on x-only modes: i sin(kh)/h
    c0, c1 = 0.4, 0.3
    dq = 2 * c0 * c1 * np.sin(k) * np.cos(k * x) + (c1 ** 2 / 2) * np.sin(2 * k) * np.sin(2 * k * x)
    expect = -dt * zeta * dq
    got = a["vxs"] - b["vxs"]
    assert np.abs(got - expect[None, None, :]).max() <= 1e-14


def test_oracle_is_deterministic_across_thread_counts(oracle_mod):
    N = 12
    rng = np.random.default_rng(9)
    s = oracle_mod.new_state(N)
    for k in s:
        s[k][:] = 0.1 * rng.standard_normal((N, N, N))
    a = {k: v.copy() for k, v in s.items()}
    b = {k: v.copy() for k, v in s.items()}
    n0 = oracle_mod.set_threads(0)
    oracle_mod.set_threads(1)
    oracle_mod.step(a, 2, N, zeta=0.01)
    oracle_mod.set_threads(max(2, n0))
    oracle_mod.step(b, 2, N, zeta=0.01)
    oracle_mod.set_threads(n0)
    for k in a:
        assert np.array_equal(a[k], b[k]), k


REF_GOLDEN = os.path.join(GOLDEN, "ref_N12.npz")


@pytest.mark.skipif(not os.path.exists(REF_GOLDEN), reason="reference golden fixture not generated")
def test_oracle_matches_reference_program_golden(oracle_mod):
    """Pins the oracle: 5 steps at 12^3 of the reference's own CUDA program (stale halo, continuous k^2)."""
    g = np.load(REF_GOLDEN)
    N = g["init_phi"].shape[0]
    s = {k: np.ascontiguousarray(g["init_" + k]) for k in KERNEL_FIELDS}
    oracle_mod.step(s, 5, N, k2_mode=0, stale_halo=1, zeta=0.0)
    for k in KERNEL_FIELDS:
        ref = g["final_" + k]
        nr = np.linalg.norm(ref) or 1.0
        assert np.linalg.norm(s[k] - ref) / nr <= 1e-12, k


@pytest.mark.skipif(not os.path.exists(REF_GOLDEN), reason="reference golden fixture not generated")
def test_stale_halo_quirk_is_needed_for_reference_parity(oracle_mod):
    """Without quirk Q2 the oracle departs from the reference program (so the quirk is real)."""
    g = np.load(REF_GOLDEN)
    N = g["init_phi"].shape[0]
    s = {k: np.ascontiguousarray(g["init_" + k]) for k in KERNEL_FIELDS}
    oracle_mod.step(s, 5, N, k2_mode=0, stale_halo=0, zeta=0.0)
    ref = g["final_vx"]
    assert np.linalg.norm(s["vx"] - ref) / np.linalg.norm(ref) > 1e-8
