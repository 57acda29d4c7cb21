"""GPU tests of the FP32 forms (fused kernels and plain kernels) against each other and against
the FP64 oracle. Tolerances (relative L2 per field) are stated next to each test."""
import numpy as np
import pytest

from conftest import random_state
from test_gpu_parity import field_errors, run_oracle

pytestmark = pytest.mark.gpu


def run(st, nsteps, form, precision=32, k2_mode=0, quirks=1, zeta=0.0):
    import ttsh
    N = st["phi"].shape[0]
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=precision, k2_mode=k2_mode, quirks=quirks, zeta=zeta, form=form)
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        s.step(nsteps)
        out = s.get_state(0)
        out["us"], out["ps"] = s.get_provisional(0)
        out["stats"] = s.reduce(0)
    return out


def droplet_state(N, seed=0, zeta_u=0.0):
    import ttsh
    phi, P = ttsh.init_droplet(N, N / 4.0, 2.0, seed)
    z = np.zeros((3, N, N, N))
    return dict(phi=phi, P=P, u=z, us=z, ps=z)


@pytest.mark.parametrize("N", [32, 64])
@pytest.mark.parametrize("k2_mode,quirks,zeta", [(0, 1, 0.0), (0, 1, 0.02), (1, 0, 0.02)])
def test_fused_matches_plain_fp32(N, k2_mode, quirks, zeta):
    """Same FP32 arithmetic up to the order of the stress sum: 2e-5 relative L2 after 5 steps.

    With the discrete k^2 the pressure of white-noise data is ill-conditioned (near-null modes of
    the 27-point gradient divide round-off by |K|^2 ~ 1e-4), so there only the fields, whose
    gradient correction multiplies those modes back by K, are compared."""
    import ttsh
    st = random_state(N, seed=N + 1)
    f = run(st, 5, ttsh.FORM_FUSED, k2_mode=k2_mode, quirks=quirks, zeta=zeta)
    p = run(st, 5, ttsh.FORM_PLAIN, k2_mode=k2_mode, quirks=quirks, zeta=zeta)
    errs = field_errors(f, p)
    if k2_mode == 1:
        errs.pop("pv")
        errs.pop("pp")
    assert max(errs.values()) <= 2e-5, errs


def test_fused_fp32_vs_oracle_droplet(oracle_mod):
    """64^3 droplet, zeta = 0.01, 200 steps: FP32 fused vs the FP64 oracle, every field within 1e-5."""
    import ttsh
    st = droplet_state(64)
    f = run(st, 200, ttsh.FORM_FUSED, zeta=0.01)
    o = run_oracle(oracle_mod, st, 200, 0, 1, 0.01)
    errs = field_errors(f, o)
    assert max(errs.values()) <= 1e-5, errs


def test_fused_batch_mixed_sizes_match_single():
    import ttsh
    sizes = [64, 32, 96, 32]
    states = [random_state(N, seed=300 + i) for i, N in enumerate(sizes)]
    inps = [ttsh.default_input(Nx=N, Ny=N, Nz=N) for N in sizes]
    exts = [ttsh.default_ext(precision=32, zeta=0.01 * i, form=ttsh.FORM_FUSED) for i in range(len(sizes))]
    with ttsh.Sim(inps, exts) as s:
        for i, st in enumerate(states):
            s.set_state(i, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        s.step(3)
        got = [s.get_state(i) for i in range(len(sizes))]
    for i, st in enumerate(states):
        single = run(st, 3, ttsh.FORM_FUSED, zeta=0.01 * i)
        for k in ("phi", "P", "u", "pv", "pp"):
            assert np.array_equal(got[i][k], single[k]), (i, k)


def test_fused_rejects_unsupported_size():
    import ttsh
    inp = ttsh.default_input(Nx=24, Ny=24, Nz=24)
    with pytest.raises(ttsh.TTSHError) as e:
        ttsh.Sim(inp, ttsh.default_ext(precision=32, form=ttsh.FORM_FUSED))
    assert e.value.code == ttsh.E_UNSUPPORTED


def test_fused_discrete_k2_divergence_small():
    """Discrete k^2 in FP32: the projected velocity is solenoidal to FP32 round-off."""
    import ttsh
    st = droplet_state(64)
    f = run(st, 50, ttsh.FORM_FUSED, k2_mode=1, quirks=0, zeta=0.02)
    umax = np.abs(f["u"]).max()
    assert f["stats"]["max_div_u"] <= 1e-5 * max(umax, 1e-3), (f["stats"], umax)


def test_fused_fp32_vs_fp64_at_256():
    """The headline size: one 256^3 droplet (R = 64, xi = 2, seed 1, zeta = 0.02), 200 steps, FP32
    fused form against the FP64 form. phi, P, u within the 1e-5 relative L2 target (measured after
    1000 steps: 2e-8, 4e-7, 5e-7); the FP32 mass drift within 2x of the FP64 form's (the phi
    update is compensated)."""
    import ttsh
    st = droplet_state(256, seed=1)
    outs = {}
    for prec, form in ((64, ttsh.FORM_PLAIN), (32, ttsh.FORM_FUSED)):
        outs[prec] = run(st, 200, form, precision=prec, zeta=0.02)
    errs = field_errors(outs[32], outs[64])
    for k in ("phi", "P", "u"):
        assert errs[k] <= 1e-5, errs
    m0 = st["phi"].sum()
    d32 = (outs[32]["stats"]["mass"] - m0) / m0
    d64 = (outs[64]["stats"]["mass"] - m0) / m0
    assert abs(d32 - d64) <= max(abs(d64), 1e-9), (d32, d64)


def test_fused_fp32_at_512():
    """The largest configuration (512^3, R = 160, xi = 3, seed 7, zeta = 0.02, discrete k^2):
    20 steps stay finite, the mass changes by the scheme's drift only, and the projected velocity
    is solenoidal to FP32 round-off."""
    import ttsh
    N = 512
    phi, P = ttsh.init_droplet(N, 160.0, 3.0, 7, angular_noise=0.01)
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    ext = ttsh.default_ext(precision=32, zeta=0.02, k2_mode=1, quirks=0, form=ttsh.FORM_FUSED)
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, phi, P, np.zeros_like(P))
        m0 = s.reduce(0)["mass"]
        s.step(20)
        st = s.reduce(0)
    assert st["nonfinite"] == 0
    assert abs(st["mass"] - m0) <= 1e-6 * m0, (st["mass"], m0)
    assert st["max_div_u"] <= 1e-5 * max(st["max_abs_u"], 1e-3), st
