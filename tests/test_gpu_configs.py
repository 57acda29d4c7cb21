"""GPU tests of the configurations the benchmark names, FP32 fused form against the FP64 form
(itself pinned to the oracle and the reference program at 1e-10 .. 1e-11, tests/test_gpu_parity.py,
tests/test_gpu_reference.py), and of non-default model constants in both forms.

Tolerances (relative L2 per field, written in each test):
  * 256^3, 1000 steps, zeta 0.005 and 0.02, the reference's k^2: phi, P, u, p_p <= 1e-5, p_v
    <= 3e-5 (measured 2.2e-5). The p_v difference is not the error of one step (one FP32 step from
    the FP64 state at step 999: 3.8e-7) but grows with the steps taken in FP32 (50: 4e-6, 500:
    1.9e-5), all of it at high wavenumbers: the FP32 rounding of the velocity update's stress
    terms has a divergent part, and at high wavenumbers the projection with the reference's
    continuous k^2 (which the 27-point divergence does not invert) leaves that part in u from
    step to step, where D.u / dt carries it into the next p_v;
  * the same with the discrete k^2 (which the projection inverts exactly): phi, P, u <= 1e-5,
    and ||D.u||_inf <= 1e-6;
  * the batched 64 x 128^3 sweep after 2000 steps, 4 sampled droplets against single FP64 runs:
    TOL_Q3; the radix-3/5 sizes 96, 160, 192 after 100 steps: 1e-5;
  * non-default constants: FP64 form vs the oracle 1e-11, FP32 fused vs FP64 form 1e-5;
  * the 512^3 droplet, 500 steps: finite, mass drift < 1e-6; its 256^3 equivalent vs FP64: TOL_Q3.
"""
import sys

import numpy as np
import pytest

from conftest import ROOT
from test_gpu_parity import FP64_TOL, run_oracle

pytestmark = pytest.mark.gpu

TARGET = 1e-5
FIELDS5 = ("phi", "P", "u", "pv", "pp")
# the reference's k^2: p_v's FP32 rounding accumulates in modes the projection leaves in place
TOL_Q3 = dict(phi=1e-5, P=1e-5, u=1e-5, pv=3e-5, pp=1e-5)


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def run(ttsh, N, phi, P, steps, precision, form, zeta, k2_mode=0, quirks=1, **inp_kw):
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N, **inp_kw)
    ext = ttsh.default_ext(precision=precision, zeta=zeta, k2_mode=k2_mode, quirks=quirks, form=form)
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, phi, P, np.zeros_like(P))
        s.step(steps)
        out = s.get_state(0)
        out["stats"] = s.reduce(0)
    return out


@pytest.mark.parametrize("zeta", [0.005, 0.02])
def test_fp32_fused_vs_fp64_256_1000_steps(zeta):
    """The headline case: 256^3, R = 64, xi = 2, seed 1, 1000 steps at the reference dt, the
    reference's k^2; the FP32 fused form against the FP64 form (TOL_Q3)."""
    import ttsh
    N = 256
    phi, P = ttsh.init_droplet(N, 64.0, 2.0, 1)
    a = run(ttsh, N, phi, P, 1000, 64, ttsh.FORM_PLAIN, zeta)
    b = run(ttsh, N, phi, P, 1000, 32, ttsh.FORM_FUSED, zeta)
    errs = {k: rel(b[k], a[k]) for k in FIELDS5}
    assert all(errs[k] <= TOL_Q3[k] for k in FIELDS5), errs
    # the FP32 mass drift is the scheme's own (within 2x of the FP64 form's), and the divergence
    # left by the reference's k^2 is the same in both precisions (quirk Q3)
    m0 = phi.sum()
    d32, d64 = (b["stats"]["mass"] - m0) / m0, (a["stats"]["mass"] - m0) / m0
    assert abs(d32 - d64) <= max(abs(d64), 1e-9), (d32, d64)
    assert abs(b["stats"]["max_div_u"] - a["stats"]["max_div_u"]) <= 0.1 * a["stats"]["max_div_u"], (b["stats"], a["stats"])


def test_fp32_fused_discrete_k2_256_1000_steps():
    """The same case with the discrete k^2 and no stale halo, so that the projection removes the
    divergence D measures: phi, P, u within 1e-5 of the FP64 form (measured 7e-9, 3e-7, 7e-7)
    and ||D.u||_inf <= 1e-6 after 1000 steps (the reference's continuous k^2 is not discretely
    solenoidal in either precision, quirk Q3). The pressures are not compared here: with the
    discrete k^2 the near-null modes of the 27-point gradient divide round-off by |K|^2 (p_v,
    p_p differ by 1e-4 between the precisions) and the correction multiplies them back by K."""
    import ttsh
    N = 256
    phi, P = ttsh.init_droplet(N, 64.0, 2.0, 1)
    a = run(ttsh, N, phi, P, 1000, 64, ttsh.FORM_PLAIN, 0.02, k2_mode=1, quirks=0)
    b = run(ttsh, N, phi, P, 1000, 32, ttsh.FORM_FUSED, 0.02, k2_mode=1, quirks=0)
    assert b["stats"]["max_div_u"] <= 1e-6, b["stats"]
    errs = {k: rel(b[k], a[k]) for k in ("phi", "P", "u")}
    assert max(errs.values()) <= TARGET, errs


@pytest.mark.parametrize("N,zeta", [(96, 0.01), (160, 0.03), (192, 0.01)])
def test_fp32_fused_radix_3_5_sizes_vs_fp64(N, zeta):
    """The sizes of the uneven batch whose FFTs use radix-3 and radix-5 register kernels
    (96 = 24 x 4, 160 = 40 x 4, 192 = 24 x 8): R = 0.3 N, 100 steps, FP32 fused vs FP64 form."""
    import ttsh
    phi, P = ttsh.init_droplet(N, 0.3 * N, 2.0, 200 + N)
    a = run(ttsh, N, phi, P, 100, 64, ttsh.FORM_PLAIN, zeta)
    b = run(ttsh, N, phi, P, 100, 32, ttsh.FORM_FUSED, zeta)
    errs = {k: rel(b[k], a[k]) for k in FIELDS5}
    assert max(errs.values()) <= TARGET, errs


def test_batched_sweep_sampled_instances_vs_fp64():
    """The batched sweep of 64 droplets on 128^3 grids (R ~ U[20, 40], zeta log-uniform in
    [1e-3, 5e-2], seeds 100-163), 2000 steps in one batch; 4 sampled droplets against single
    FP64-form runs of the same droplet."""
    import ttsh
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from bench import workload
    drops = workload("64x128")
    inps = [ttsh.default_input(Nx=d[0], Ny=d[0], Nz=d[0]) for d in drops]
    exts = [ttsh.default_ext(precision=32, zeta=d[4], form=ttsh.FORM_FUSED) for d in drops]
    init = {}
    with ttsh.Sim(inps, exts) as s:
        for i, (N, R, xi, seed, zeta) in enumerate(drops):
            phi, P = ttsh.init_droplet(N, R, xi, seed)
            if i in (0, 21, 42, 63):
                init[i] = (phi, P)
            s.set_state(i, phi, P, np.zeros_like(P))
        s.step(2000)
        got = {i: s.get_state(i) for i in init}
    for i, (phi, P) in init.items():
        N, R, xi, seed, zeta = drops[i]
        a = run(ttsh, N, phi, P, 2000, 64, ttsh.FORM_PLAIN, zeta)
        errs = {k: rel(got[i][k], a[k]) for k in FIELDS5}
        assert all(errs[k] <= TOL_Q3[k] for k in FIELDS5), (i, errs)


CONSTS = dict(h=0.7, A=0.3, La=1.3, kPhi=0.8, aPhi=1.1)


@pytest.mark.parametrize("k2_mode,quirks", [(0, 1), (1, 0)])
def test_nondefault_constants_fp64_vs_oracle(oracle_mod, k2_mode, quirks):
    """A, h, La, kPhi != aPhi away from the reference defaults (forEach.pl:12-23 sweeps them): the
    FP64 form against the oracle, 10 steps of a 32^3 droplet with zeta = 0.02, 1e-11."""
    import ttsh
    N = 32
    phi, P = ttsh.init_droplet(N, 8.0, 2.0, 3)
    z = np.zeros((3, N, N, N))
    st = dict(phi=phi, P=P, u=z, us=z, ps=z)
    g = run(ttsh, N, phi, P, 10, 64, ttsh.FORM_PLAIN, 0.02, k2_mode, quirks, **CONSTS)
    o = run_oracle(oracle_mod, st, 10, k2_mode, quirks, 0.02, **CONSTS)
    errs = {k: rel(g[k], o[k]) for k in FIELDS5}
    assert max(errs.values()) <= FP64_TOL, errs


@pytest.mark.parametrize("N", [32, 64])
def test_nondefault_constants_fp32_fused_vs_fp64(N):
    """The same constants, FP32 fused form vs FP64 form, 200 steps, every field within 1e-5 (the
    A-term of the P update, TTSH3D.cu:623-629, runs here)."""
    import ttsh
    phi, P = ttsh.init_droplet(N, N / 4.0, 2.0, 4)
    a = run(ttsh, N, phi, P, 200, 64, ttsh.FORM_PLAIN, 0.02, **CONSTS)
    b = run(ttsh, N, phi, P, 200, 32, ttsh.FORM_FUSED, 0.02, **CONSTS)
    errs = {k: rel(b[k], a[k]) for k in FIELDS5}
    assert max(errs.values()) <= TARGET, errs


def test_large_droplet_512_500_steps_and_its_256_equivalent():
    """The large single droplet: 512^3, R = 160, xi = 3, zeta = 0.02, seed 7, 1 % Gaussian angular
    noise, 500 steps in the FP32 fused form: finite, and the FP64-reduced mass drifts by less than
    1e-6. Its error is stated on the 1/8-subvolume equivalent at 256^3 (every length halved:
    R = 80, xi = 1.5, the same seed and noise), FP32 fused against the FP64 form after 500 steps
    (TOL_Q3)."""
    import ttsh
    N = 512
    phi, P = ttsh.init_droplet(N, 160.0, 3.0, 7, angular_noise=0.01)
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=32, zeta=0.02, form=ttsh.FORM_FUSED)
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, phi, P, np.zeros_like(P))
        m0 = s.reduce(0)["mass"]
        s.step(500)
        st = s.reduce(0)
    del phi, P
    assert st["nonfinite"] == 0, st
    assert abs(st["mass"] - m0) <= 1e-6 * m0, (st["mass"], m0)
    N = 256
    phi, P = ttsh.init_droplet(N, 80.0, 1.5, 7, angular_noise=0.01)
    a = run(ttsh, N, phi, P, 500, 64, ttsh.FORM_PLAIN, 0.02)
    b = run(ttsh, N, phi, P, 500, 32, ttsh.FORM_FUSED, 0.02)
    errs = {k: rel(b[k], a[k]) for k in FIELDS5}
    assert all(errs[k] <= TOL_Q3[k] for k in FIELDS5), errs
