"""GPU parity: libttsh's CUDA step, called through the C ABI, against the FP64 CPU oracle.

Tolerances (relative L2 per field, written here and in the asserts):
  FP64 plain form vs oracle: 1e-11 (differences are FMA contraction and summation order only)
  FP32 forms: tests/test_gpu_fp32.py.
"""
import numpy as np
import pytest

from conftest import oracle_state, random_state

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-11


def relerr(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def run_gpu(st, nsteps, precision=64, k2_mode=0, quirks=1, zeta=0.0, **inp_kw):
    import ttsh
    N = st["phi"].shape[0]
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N, **inp_kw)
    ext = ttsh.default_ext(precision=precision, k2_mode=k2_mode, quirks=quirks, zeta=zeta)
    with ttsh.Sim(inp, ext) as s:
        s.set_state(0, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        s.step(nsteps)
        out = s.get_state(0)
        out["us"], out["ps"] = s.get_provisional(0)
        out["stats"] = s.reduce(0)
    return out


def run_oracle(O, st, nsteps, k2_mode=0, stale=1, zeta=0.0, **consts):
    N = st["phi"].shape[0]
    s = oracle_state(st)
    O.step(s, nsteps, N, k2_mode=k2_mode, stale_halo=stale, zeta=zeta, **consts)
    return dict(phi=s["phi"], P=np.stack([s["px"], s["py"], s["pz"]]), u=np.stack([s["vx"], s["vy"], s["vz"]]),
                pv=s["pv"], pp=s["pp"], us=np.stack([s["vxs"], s["vys"], s["vzs"]]),
                ps=np.stack([s["pxs"], s["pys"], s["pzs"]]))


FIELDS = ("phi", "P", "u", "pv", "pp", "us", "ps")


def field_errors(g, o):
    return {k: relerr(g[k], o[k]) for k in FIELDS}


@pytest.mark.parametrize("N", [16, 20, 24, 32])
@pytest.mark.parametrize("k2_mode,stale,zeta", [(0, 1, 0.0), (0, 1, 0.02), (1, 0, 0.02), (1, 1, 0.0)])
def test_fp64_matches_oracle(oracle_mod, N, k2_mode, stale, zeta):
    st = random_state(N, seed=N + 7)
    g = run_gpu(st, 5, 64, k2_mode, stale, zeta)
    o = run_oracle(oracle_mod, st, 5, k2_mode, stale, zeta)
    errs = field_errors(g, o)
    assert max(errs.values()) <= FP64_TOL, errs


def test_fp64_config1_200_steps(oracle_mod):
    """64^3 droplet (R=16, xi=2, seed 0), zeta=0.01, 200 steps at dt=0.002: all fields and mass."""
    import ttsh
    N = 64
    phi, P = ttsh.init_droplet(N, 16.0, 2.0, 0)
    z = np.zeros((3, N, N, N))
    st = dict(phi=phi, P=P, u=z, us=z, ps=z)
    g = run_gpu(st, 200, 64, 0, 1, 0.01)
    o = run_oracle(oracle_mod, st, 200, 0, 1, 0.01)
    errs = field_errors(g, o)
    assert max(errs.values()) <= FP64_TOL, errs
    assert abs(g["stats"]["mass"] - oracle_mod.mass(o["phi"])) <= 1e-12 * abs(oracle_mod.mass(o["phi"]))


def test_batch_uneven_sizes_match_single_runs():
    """Droplets of different sizes in one batch give exactly the single-droplet results."""
    import ttsh
    sizes = [16, 24, 16, 32]
    states = [random_state(N, seed=100 + i) for i, N in enumerate(sizes)]
    exts = [ttsh.default_ext(precision=64, zeta=0.01 * i) for i in range(len(sizes))]
    inps = [ttsh.default_input(Nx=N, Ny=N, Nz=N) for N in sizes]
    with ttsh.Sim(inps, exts) as s:
        for i, st in enumerate(states):
            s.set_state(i, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        s.step(4)
        batch = [s.get_state(i) for i in range(len(sizes))]
    for i, st in enumerate(states):
        single = run_gpu(st, 4, 64, zeta=0.01 * i)
        for k in ("phi", "P", "u", "pv", "pp"):
            assert np.array_equal(batch[i][k], single[k]), (i, k)


def test_batch_of_stockham_sizes_match_single_runs():
    """Sizes served only by the Stockham FFT kernel (one kernel for all sizes, with a shared-memory
    limit per kernel): the larger size must still launch after the smaller one is set up."""
    import ttsh
    sizes = [40, 20, 40]
    states = [random_state(N, seed=200 + i) for i, N in enumerate(sizes)]
    exts = [ttsh.default_ext(precision=64, zeta=0.01) for _ in sizes]
    inps = [ttsh.default_input(Nx=N, Ny=N, Nz=N) for N in sizes]
    with ttsh.Sim(inps, exts) as s:
        for i, st in enumerate(states):
            s.set_state(i, st["phi"], st["P"], st["u"], st["us"], st["ps"])
        s.step(3)
        batch = [s.get_state(i) for i in range(len(sizes))]
    for i, st in enumerate(states):
        single = run_gpu(st, 3, 64, zeta=0.01)
        for k in ("phi", "P", "u", "pv", "pp"):
            assert np.array_equal(batch[i][k], single[k]), (i, k)


def test_stats_and_watchdog():
    import ttsh
    N = 16
    st = random_state(N, seed=3)
    g = run_gpu(st, 2)
    assert g["stats"]["nonfinite"] == 0
    assert abs(g["stats"]["mass"] - g["phi"].sum()) <= 1e-12 * abs(g["phi"].sum())
    assert g["stats"]["steps"] == 2
    bad = dict(st)
    bad["phi"] = st["phi"].copy()
    bad["phi"][3, 4, 5] = np.nan
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    with ttsh.Sim(inp, ttsh.default_ext()) as s:
        s.set_state(0, bad["phi"], bad["P"], bad["u"])
        s.step(1)
        r = s.reduce(0, check=False)
        assert r["nonfinite"] == 1
        with pytest.raises(ttsh.TTSHError) as e:
            s.reduce(0)
        assert e.value.code == ttsh.E_UNSTABLE


def test_discrete_k2_is_solenoidal_fp64():
    st = random_state(32, seed=5)
    g = run_gpu(st, 3, 64, k2_mode=1, quirks=0)
    assert g["stats"]["max_div_u"] <= 1e-12 * max(1.0, np.abs(g["u"]).max())


def test_reference_k2_is_not_solenoidal_fp64():
    """Quirk Q3: the continuous k^2 with the 27-point divergence leaves a residual divergence."""
    st = random_state(32, seed=5)
    g = run_gpu(st, 3, 64, k2_mode=0, quirks=1)
    assert g["stats"]["max_div_u"] > 1e-8


@pytest.mark.parametrize("N", [16, 32, 48])
def test_fft_kernels_agree(oracle_mod, N, monkeypatch):
    """The register-resident FFT kernels (one launch per axis pass, or x and y of a plane in one
    launch) and the shared-memory Stockham passes all match the oracle; the two register forms
    run the same arithmetic, so they agree bit for bit."""
    st = random_state(N, seed=N + 11)
    o = run_oracle(oracle_mod, st, 3, 0, 1, 0.01)
    runs = {}
    for kind in ("stockham", "separate", None):
        if kind is None:
            monkeypatch.delenv("TTSH_FFT", raising=False)
        else:
            monkeypatch.setenv("TTSH_FFT", kind)
        runs[kind] = run_gpu(st, 3, 64, 0, 1, 0.01)
    monkeypatch.delenv("TTSH_FFT", raising=False)
    for g in runs.values():
        errs = field_errors(g, o)
        assert max(errs.values()) <= FP64_TOL, errs
    for k in FIELDS:
        assert np.array_equal(runs["separate"][k], runs[None][k]), k


@pytest.mark.parametrize("N", [64, 256])
def test_plane_fft_matches_separate_passes_fp32(N, monkeypatch):
    """FP32 fused form: x and y of each plane in one launch equals one launch per axis pass."""
    import ttsh
    st = random_state(N, seed=N + 5)
    runs = {}
    for kind in ("separate", None):
        if kind is None:
            monkeypatch.delenv("TTSH_FFT", raising=False)
        else:
            monkeypatch.setenv("TTSH_FFT", kind)
        runs[kind] = run_gpu(st, 2, 32, 0, 1, 0.02)
    monkeypatch.delenv("TTSH_FFT", raising=False)
    for k in FIELDS:
        assert np.array_equal(runs["separate"][k], runs[None][k]), k


@pytest.mark.parametrize("fft", [None, "separate"])
def test_staged_z_pass_matches_direct_loads(fft, monkeypatch):
    """FP32, 256^3: the z pass whose input the tensor memory accelerator stages in shared memory
    (TTSH_ZTMA=1) gives the same bits as the z pass that loads its input directly (the default)."""
    N = 256
    st = random_state(N, seed=N + 9)
    if fft:
        monkeypatch.setenv("TTSH_FFT", fft)
    runs = {}
    for zt in ("1", None):
        if zt is None:
            monkeypatch.delenv("TTSH_ZTMA", raising=False)
        else:
            monkeypatch.setenv("TTSH_ZTMA", zt)
        runs[zt] = run_gpu(st, 2, 32, 0, 1, 0.02)
    monkeypatch.delenv("TTSH_ZTMA", raising=False)
    monkeypatch.delenv("TTSH_FFT", raising=False)
    for k in FIELDS:
        assert np.array_equal(runs["1"][k], runs[None][k]), k


def test_reduce_all_matches_single_reduce():
    """ttsh_reduce_all (one pass per size group) equals ttsh_reduce per droplet; mass-only mode too."""
    import ttsh
    sizes = [16, 24, 16]
    states = [random_state(N, seed=50 + i) for i, N in enumerate(sizes)]
    inps = [ttsh.default_input(Nx=N, Ny=N, Nz=N) for N in sizes]
    with ttsh.Sim(inps, [ttsh.default_ext(precision=64) for _ in sizes]) as s:
        for i, st in enumerate(states):
            s.set_state(i, st["phi"], st["P"], st["u"])
        s.step(2)
        one = [s.reduce(i) for i in range(len(sizes))]
        allf = s.reduce_all()
        mass = s.reduce_all(mass_only=True)
    for a, b, m in zip(one, allf, mass):
        assert a == b
        assert m["mass"] == a["mass"] and m["nonfinite"] == 0 and m["max_div_u"] == -1.0


@pytest.mark.parametrize("precision", [64, 32])
def test_reduce_all_async_matches_reduce_all(precision):
    """ttsh_reduce_all_async + ttsh_stats_from_partials give ttsh_reduce_all's values, bit for
    bit, for buffers filled at different steps and read only after one final sync."""
    import torch
    import ttsh
    sizes = [32, 48, 32] if precision == 32 else [16, 24, 16]
    states = [random_state(N, seed=70 + i) for i, N in enumerate(sizes)]
    inps = [ttsh.default_input(Nx=N, Ny=N, Nz=N) for N in sizes]

    def run(async_mode):
        with ttsh.Sim(inps, [ttsh.default_ext(precision=precision) for _ in sizes]) as s:
            for i, st in enumerate(states):
                s.set_state(i, st["phi"], st["P"], st["u"])
            if not async_mode:
                out = []
                for k in range(4):
                    s.step(1)
                    out.append(s.reduce_all(mass_only=(k % 2 == 1)))
                return out
            m = s.partials_size()
            assert m > 2 + len(sizes)
            bufs = torch.empty((4, m), dtype=torch.float64, pin_memory=True).numpy()
            for k in range(4):
                s.step(1)
                s.reduce_all_async(bufs[k], mass_only=(k % 2 == 1))
            s.sync()
            return [s.stats_from_partials(bufs[k]) for k in range(4)]

    got, want = run(True), run(False)
    assert got == want
    assert [g[0]["steps"] for g in got] == [1, 2, 3, 4]
