"""The autotuner (ttsh_autotune / ttsh_set_tuning / ttsh_get_tuning) on the GPU.

It must leave the state as it was, keep the results (the z-extent of the fused kernels' tiles
changes nothing; the FFT choice changes rounding only: FP32 relative L2 <= 1e-5 against an
untuned run, FP64 <= 1e-12), reject configurations the kernels do not support, and reuse a
cache file without timing again.
"""
import numpy as np
import pytest

from conftest import random_state

pytestmark = pytest.mark.gpu


def relerr(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (nb if nb > 0 else 1.0))


def make(ttsh, sizes, precision):
    inps = [ttsh.default_input(Nx=N, Ny=N, Nz=N) for N in sizes]
    ext = ttsh.default_ext(precision=precision, zeta=0.02)
    s = ttsh.Sim(inps, [ext] * len(sizes))
    states = [random_state(N, seed=11 + k) for k, N in enumerate(sizes)]
    for k, st in enumerate(states):
        s.set_state(k, st["phi"], st["P"], st["u"], st["us"], st["ps"])
    return s


@pytest.mark.parametrize("precision,sizes,tol", [(32, (64, 32, 64), 1e-5), (64, (16, 24), 1e-12)])
def test_autotune_keeps_state_and_results(precision, sizes, tol):
    import ttsh
    with make(ttsh, sizes, precision) as a, make(ttsh, sizes, precision) as b:
        a.step(2)
        b.step(2)
        before = [a.get_state(k) for k in range(len(sizes))]
        cfg = a.autotune()
        assert len(cfg) == len(set(sizes))
        for c in cfg:
            assert c["ms"]["fft"] > 0
            if precision == 32:
                assert min(c["ms"][k] for k in ("fused_rhs", "fused_div", "fused_correct")) > 0
                assert all(z >= 0 for z in c["zc"])
            assert int(np.prod(c["radix"])) == c["N"]
        after = [a.get_state(k) for k in range(len(sizes))]
        for x, y in zip(before, after):
            for f in ("phi", "P", "u", "pv", "pp"):
                assert np.array_equal(x[f], y[f]), f
        a.step(5)
        b.step(5)
        for k in range(len(sizes)):
            ga, gb = a.get_state(k), b.get_state(k)
            for f in ("phi", "P", "u", "pv", "pp"):
                assert relerr(ga[f], gb[f]) <= tol, (k, f, relerr(ga[f], gb[f]))


@pytest.mark.parametrize("sizes,zc", [((64,), [8, 32, 128]), ((64,), [0, 64, 16]), ((96, 96, 96), [0, 0, 0]),
                                      ((32, 32), [0, 0, 8]), ((64, 64), [16, 0, 0])])
def test_zc_choice_is_bit_exact(sizes, zc):
    """The z extents of the fused kernels, and their persistent grids (zc 0: equal shares of the
    group's sites per CTA, segments crossing tile columns and droplets), give the same bits."""
    import ttsh
    with make(ttsh, sizes, 32) as a, make(ttsh, sizes, 32) as b:
        cfg = a.tuning()[0]
        cfg["zc"] = zc
        a.set_tuning(0, cfg)
        assert a.tuning()[0]["zc"] == zc
        a.step(4)
        b.step(4)
        for k in range(len(sizes)):
            ga, gb = a.get_state(k), b.get_state(k)
            for f in ("phi", "P", "u", "pv", "pp"):
                assert np.array_equal(ga[f], gb[f]), (k, f)


def test_set_tuning_rejects_unsupported():
    import ttsh
    with make(ttsh, (64,), 32) as a:
        good = a.tuning()[0]
        for bad in ({"radix": [4, 4, 2]}, {"radix": [8, 8]}, {"fft_lb": 3}, {"fft_kind": 3}, {"zc": [-1, 64, 64]},
                    {"zc": [64, -2, 64]}, {"zc": [64, 64, -8]},
                    {"N": 32}):
            cfg = dict(good, **bad)
            with pytest.raises(ttsh.TTSHError) as e:
                a.set_tuning(0, cfg)
            assert e.value.code == ttsh.E_INVALID
        assert a.tuning()[0] == good


def test_tuning_cache_round_trip(tmp_path):
    import ttsh
    cache = str(tmp_path / "tune.txt")
    with make(ttsh, (64, 32), 32) as a:
        first = a.autotune(cache)
    text = open(cache).read()
    assert text.count("\n") == 2
    with make(ttsh, (64, 32), 32) as b:
        second = b.autotune(cache)
    assert open(cache).read() == text
    strip = lambda cs: [{k: v for k, v in c.items() if k != "ms"} for c in cs]
    assert strip(second) == strip(first)
    assert all(v == 0 for c in second for v in c["ms"].values())
