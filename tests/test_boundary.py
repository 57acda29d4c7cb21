"""CPU tests of the drop-in boundary: input.dat (GetInput), the snapshot text layout
(ExpoConf, readDraw.py), the build-defined initial condition, and the C ABI exports."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, ROOT
from make_ref import REF_DIR  # oracle/ is on the path (conftest)


def test_library_exports_every_declared_symbol():
    import ttsh
    L = ttsh.lib()
    syms = ttsh.declared_symbols()
    assert len(syms) >= 20
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing


def test_read_input_golden_from_run_cuda_pl():
    """input.dat printed by run_cuda.pl:53-87 (tests/golden/input_default.dat) parses to its defaults."""
    import ttsh
    got = ttsh.read_input(os.path.join(GOLDEN, "input_default.dat")).as_dict()
    want = ttsh.default_input().as_dict()
    assert got == want


def test_write_input_is_byte_identical_to_perl(tmp_path):
    import ttsh
    p = tmp_path / "input.dat"
    ttsh.write_input(str(p), ttsh.default_input())
    assert p.read_bytes() == open(os.path.join(GOLDEN, "input_default.dat"), "rb").read()


def test_read_input_sentinel_and_errors(tmp_path):
    import ttsh
    toks = open(os.path.join(GOLDEN, "input_default.dat")).read().split()
    bad = tmp_path / "bad.dat"
    bad.write_text("\n".join(toks[:-1] + ["-1"]) + "\n")
    with pytest.raises(ttsh.TTSHError) as e:
        ttsh.read_input(str(bad))
    assert e.value.code == ttsh.E_PARSE
    short = tmp_path / "short.dat"
    short.write_text("\n".join(toks[:20]) + "\n")
    with pytest.raises(ttsh.TTSHError) as e:
        ttsh.read_input(str(short))
    assert e.value.code == ttsh.E_PARSE
    with pytest.raises(ttsh.TTSHError) as e:
        ttsh.read_input(str(tmp_path / "missing.dat"))
    assert e.value.code == ttsh.E_IO
    # a float token where the reference reads an int stops the stream, as `>>` does
    floaty = tmp_path / "floaty.dat"
    floaty.write_text("\n".join(["1.5"] + toks[1:]) + "\n")
    with pytest.raises(ttsh.TTSHError):
        ttsh.read_input(str(floaty))


def _fields(N, seed):
    rng = np.random.default_rng(seed)
    phi = rng.uniform(-1, 2, (N, N, N))
    P = rng.standard_normal((3, N, N, N)) * 10.0 ** rng.integers(-20, 3, (3, N, N, N))
    u = rng.standard_normal((3, N, N, N)) * 1e-3
    u[0, 0, 0, 0] = -0.0
    u[1, 0, 0, 0] = 5e-16
    u[2, 0, 0, 0] = -5e-16
    return phi, P, u


def test_conf_layout_matches_expoconf(tmp_path):
    """One line per site, y outer, x, z inner; 'vx vy vz px py pz phi' as fixed/setprecision(15)."""
    import ttsh
    N = 6
    phi, P, u = _fields(N, 1)
    f = tmp_path / "conf_0.dat"
    ttsh.format_conf(str(f), phi, P, u, expo_data=1)
    lines = []
    for y in range(N):
        for x in range(N):
            for z in range(N):
                vals = [u[0, z, y, x], u[1, z, y, x], u[2, z, y, x], P[0, z, y, x], P[1, z, y, x], P[2, z, y, x],
                        phi[z, y, x]]
                lines.append(" ".join("%.15f" % v for v in vals) + "\n")
    assert f.read_text() == "".join(lines)
    g = tmp_path / "conf_m1.dat"
    ttsh.format_conf(str(g), phi, P, u, expo_data=-1)
    want = "".join("%.15f %.15f " % (u[0, z, y, x], u[1, z, y, x])
                   for y in range(N) for x in range(N) for z in range(N))
    assert g.read_text() == want
    e = tmp_path / "conf_e.dat"
    ttsh.format_conf(str(e), phi, P, u, expo_data=0)
    assert e.read_text() == ""


def test_conf_readdraw_mirror(tmp_path):
    """numpy restatement of readDraw.py:205-215 (pd.read_csv(sep=' ', names=...), reshape (Ly,Lx,Lz))."""
    import ttsh
    N = 8
    phi, P, u = _fields(N, 2)
    f = tmp_path / "conf_3.dat"
    ttsh.format_conf(str(f), phi, P, u)
    data = np.loadtxt(str(f))
    names = ["vx", "vy", "vz", "px", "py", "pz", "phi"]
    cols = {n: data[:, i].reshape((N, N, N)) for i, n in enumerate(names)}
    # readDraw's array is indexed [y][x][z]; ours is [z][y][x]
    np.testing.assert_allclose(cols["phi"], np.transpose(phi, (1, 2, 0)), rtol=0, atol=1e-15)
    np.testing.assert_allclose(cols["vy"], np.transpose(u[1], (1, 2, 0)), rtol=0, atol=1e-15)
    np.testing.assert_allclose(cols["pz"], np.transpose(P[2], (1, 2, 0)), rtol=0, atol=1e-15 * 1e3)


def test_conf_parallel_writer_large(tmp_path):
    """Multi-chunk path (N large enough for several formatting rounds) stays in loop order."""
    import ttsh
    N = 40
    phi, P, u = _fields(N, 3)
    f = tmp_path / "big.dat"
    ttsh.format_conf(str(f), phi, P, u)
    with open(f) as fh:
        lines = fh.readlines()
    assert len(lines) == N ** 3
    for li in (0, 1, N, N * N, N ** 3 - 1, 12345):
        y, rem = divmod(li, N * N)
        x, z = divmod(rem, N)
        assert float(lines[li].split()[6]) == pytest.approx(phi[z, y, x], abs=1e-15)


def test_init_droplet_properties():
    import ttsh
    N, R, xi = 32, 8.0, 2.0
    phi, P = ttsh.init_droplet(N, R, xi, seed=0)
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    r = np.sqrt((x - N / 2) ** 2 + (y - N / 2) ** 2 + (z - N / 2) ** 2)
    np.testing.assert_allclose(phi, 0.5 * (1 - np.tanh((r - R) / xi)), rtol=0, atol=1e-15)
    mag = np.sqrt((P ** 2).sum(0))
    assert np.all(mag[phi <= 0.5] == 0)
    assert np.all(mag <= 1 + 1e-12)
    assert (mag[phi > 0.5] > 0).mean() > 0.99
    phi2, P2 = ttsh.init_droplet(N, R, xi, seed=0)
    assert np.array_equal(P, P2)
    _, P3 = ttsh.init_droplet(N, R, xi, seed=1)
    assert not np.array_equal(P, P3)
    _, Pn = ttsh.init_droplet(N, R, xi, seed=0, angular_noise=0.01)
    d = np.abs(Pn - P)[:, phi > 0.5]
    assert 0 < d.max() < 0.1


REF_CONFS = sorted(glob.glob(os.path.join(GOLDEN, "ref_N12_conf_*.dat")))


@pytest.mark.skipif(not REF_CONFS, reason="reference golden fixture not generated")
def test_conf_writer_byte_identical_to_reference_expoconf(tmp_path):
    """The reference program's own conf_0.dat (written from its initial state) is reproduced byte for byte."""
    import ttsh
    g = np.load(os.path.join(GOLDEN, "ref_N12.npz"))
    conf0 = [c for c in REF_CONFS if c.endswith("conf_0.dat")]
    assert conf0
    P = np.stack([g["init_px"], g["init_py"], g["init_pz"]])
    u = np.stack([g["init_vx"], g["init_vy"], g["init_vz"]])
    f = tmp_path / "conf_0.dat"
    ttsh.format_conf(str(f), np.ascontiguousarray(g["init_phi"]), P, u)
    assert f.read_bytes() == open(conf0[0], "rb").read()


def test_golden_fixture_script_is_committed():
    assert os.path.exists(os.path.join(ROOT, "tests", "golden", "make_ref_golden.py"))
    assert os.path.exists(os.path.join(ROOT, "tests", "golden", "make_input_dat.py"))


OP_PY = os.path.join(REF_DIR, "op.py")


@pytest.mark.skipif(not os.path.exists(OP_PY), reason="reference sources not present")
def test_readdraw_restatement_matches_op_py():
    """The numpy restatement of op.py's d1xO4/d1yO4 equals op.py itself (imported from the reference)."""
    import importlib.util
    import readdraw_restatement as RD
    spec = importlib.util.spec_from_file_location("ref_op", OP_PY)
    op = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(op)
    rng = np.random.default_rng(0)
    u = rng.standard_normal((12, 16))
    np.testing.assert_allclose(RD.d1xO4(u, 0.7), op.d1xO4(u, 0.7), rtol=0, atol=1e-13)
    np.testing.assert_allclose(RD.d1yO4(u, 0.7), op.d1yO4(u, 0.7), rtol=0, atol=1e-13)


def test_struct_layouts_match_the_library():
    """ctypes mirrors of ttsh_input, ttsh_ext, ttsh_stats, ttsh_tuning have the library's sizes."""
    import ctypes
    import ttsh
    L = ttsh.lib()
    for k, cls in enumerate((ttsh.Input, ttsh.Ext, ttsh.Stats, ttsh.Tuning)):
        assert L.ttsh_struct_size(k) == ctypes.sizeof(cls), cls.__name__
    assert L.ttsh_struct_size(4) == -1


def test_binding_signatures_match_header():
    """Every entry point the ctypes binding declares exists in include/ttsh.h with the same number
    of parameters and a result of the same kind (int, double, size_t, string, void)."""
    import ctypes
    import re
    import ttsh
    text = open(os.path.join(ROOT, "include", "ttsh.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    text = "\n".join(l for l in text.split("\n") if not l.lstrip().startswith("#"))  # preprocessor lines
    decls = {}
    for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(ttsh_\w+)\s*\(([^;{)]*)\)\s*;", text):
        ret, name, params = " ".join(m.group(1).split()), m.group(2), m.group(3).strip()
        n = 0 if params in ("", "void") else params.count(",") + 1
        decls[name] = (ret, n)
    kind = {ctypes.c_int: "int", ctypes.c_double: "double", ctypes.c_size_t: "size_t", ctypes.c_char_p: "const char*",
            None: "void"}
    for name, (args, res) in ttsh._signatures().items():
        assert name in decls, name
        ret, n = decls[name]
        assert n == len(args), (name, n, len(args))
        assert kind[res] == ret.replace("const char *", "const char*"), (name, ret, kind[res])


def test_oracle_init_droplet_is_the_library_one():
    """The oracle's restatement of the benchmark droplet (used by the timed reference arm, which must
    not load libttsh) gives exactly libttsh's ttsh_init_droplet, with and without angular noise."""
    import oracle
    import ttsh
    for (N, R, xi, seed, noise) in ((20, 5.0, 2.0, 3, 0.0), (24, 7.2, 3.0, 7, 0.01), (16, 4.0, 2.0, 1, 0.0)):
        a = ttsh.init_droplet(N, R, xi, seed, angular_noise=noise)
        b = oracle.init_droplet(N, R, xi, seed, angular_noise=noise)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), (N, seed, noise)


def test_reference_input_text_is_the_writer_output(tmp_path):
    """The pure-Python input.dat of the reference arm is byte for byte what ttsh.write_input prints."""
    import make_ref_golden as G
    import ttsh
    for (N, Ts, dte, expo) in ((256, 0.0495, 1e9, 0), (12, 0.009, 0.004, 1), (64, 1000.0, 10.0, 1)):
        p = tmp_path / ("in_%d.dat" % N)
        ttsh.write_input(str(p), ttsh.default_input(Nx=N, Ny=N, Nz=N, Ts=Ts, dte=dte, ExpoData=expo))
        assert G.reference_input_text(N, Ts, dte, expo) == p.read_text(), N


def test_snapshot_number_format_on_hard_values(tmp_path):
    """The snapshot writer prints every value exactly as printf "%.15f" does (the reference's
    `fixed << setprecision(15)`): its exact binary value rounded to 15 decimals with ties to even,
    the sign of -0.0 and of negatives that round to zero kept. Checked against Python's correctly
    rounded formatting on exact ties (odd multiples of 2^-16, whose 16th decimal is a final 5),
    values next to the 2^13 bound of the integer path and beyond it, subnormals and random values
    over many magnitudes."""
    import numpy as np
    import ttsh
    rng = np.random.default_rng(5)
    special = [0.0, -0.0, 1.0, -1.0, 0.5, 1 / 65536, 3 / 65536, -5 / 65536, 2 ** -17, 7 * 2 ** -18,
               1e-15, 5e-16, -5e-16, 4.9999999999999996e-16, -1e-17, 1e-300, -1e-300, 5e-324, -5e-324,
               2.2250738585072014e-308, 8191.999999999999, 8191.9999999999995, 8192.0, -8192.0, 8192.5,
               12345.678901234567, -1e10, 1.7976931348623157e308, 0.1, 0.2, 0.3, 2 / 3, -2 / 3,
               1 - 2 ** -53, 1 + 2 ** -52, 999.9999999999995, 0.0000000000000015, 0.0000000000000025]
    ties = list((2 * rng.integers(0, 2 ** 20, 200) + 1) / 65536.0 * rng.choice([-1, 1], 200))
    mags = list(rng.standard_normal(2000) * 10.0 ** rng.integers(-18, 4, 2000))
    vals = np.array(special + ties + mags, dtype=np.float64)
    N = 8
    n = N ** 3
    buf = np.resize(vals, 7 * n)
    u = buf[:3 * n].reshape(3, N, N, N).copy()
    P = buf[3 * n:6 * n].reshape(3, N, N, N).copy()
    phi = buf[6 * n:].reshape(N, N, N).copy()
    path = str(tmp_path / "conf_1.dat")
    ttsh.format_conf(path, phi, P, u)
    lines = open(path).read().split("\n")
    assert len(lines) == n + 1 and lines[-1] == ""
    k = 0
    for y in range(N):
        for x in range(N):
            for z in range(N):
                vs = [u[0, z, y, x], u[1, z, y, x], u[2, z, y, x], P[0, z, y, x], P[1, z, y, x],
                      P[2, z, y, x], phi[z, y, x]]
                assert lines[k] == " ".join("%.15f" % v for v in vs), (k, lines[k])
                k += 1
    # the 2-column layout (ExpoData == -1): "vx vy " per site, no newline
    path2 = str(tmp_path / "conf_2.dat")
    ttsh.format_conf(path2, phi, P, u, expo_data=-1)
    exp = "".join("%.15f %.15f " % (u[0, z, y, x], u[1, z, y, x])
                  for y in range(N) for x in range(N) for z in range(N))
    assert open(path2).read() == exp


def _minstd_canonical_stream(seed, count):
    """The reference's draws (TTSH3D.cu:40, :801-824): std::default_random_engine (libstdc++:
    minstd_rand0, x <- 16807 x mod 2^31 - 1) through uniform_real_distribution<double>(0, 1), i.e.
    generate_canonical<double, 53>: two engine outputs per draw, (x1 - 1) + (x2 - 1) r over r^2 with
    r = 2^31 - 2, in double arithmetic."""
    m, a = 2147483647, 16807
    x = seed % m or 1
    r = 2147483646.0
    out = []
    for _ in range(count):
        x = x * a % m
        s = float(x - 1) * 1.0
        x = x * a % m
        s = s + float(x - 1) * r
        v = s / (r * r)
        out.append(v if v < 1.0 else 0.9999999999999999)
    return out


def test_init_reference_draws_follow_the_reference_generator():
    """ttsh_init_reference with InitCond 1 (the shim's and the sweep driver's initial state) against
    a pure-Python restatement of the reference's generator: 14 draws per site in the reference's
    loop order (x outer, z inner): u, u*, P, P* as init0 (draw - 1/2), then p_v and p_p."""
    import numpy as np
    import ttsh
    N = 8
    inp = ttsh.default_input(Nx=N, Ny=N, Nz=N)
    for seed in (12345, 0, 2147483647, 4294967295):  # 0 and multiples of 2^31 - 1 seed the state 1
        _check_reference_draws(np, ttsh, inp, N, seed)


def _check_reference_draws(np, ttsh, inp, N, seed):
    st = ttsh.init_reference(inp, seed)
    d = _minstd_canonical_stream(seed, 14 * N ** 3)
    init0 = inp.init0
    k = 0
    for i in range(N):
        for j in range(N):
            for z in range(N):
                vals = [init0 * (d[k + c] - 0.5) for c in range(12)]
                k += 14
                got = [st["u"][0, z, j, i], st["u"][1, z, j, i], st["u"][2, z, j, i],
                       st["us"][0, z, j, i], st["us"][1, z, j, i], st["us"][2, z, j, i],
                       st["P"][0, z, j, i], st["P"][1, z, j, i], st["P"][2, z, j, i],
                       st["ps"][0, z, j, i], st["ps"][1, z, j, i], st["ps"][2, z, j, i]]
                assert got == vals, (i, j, z)
                r = np.sqrt((i - N / 2) ** 2 + (j - N / 2) ** 2 + (z - N / 2) ** 2)
                # (numpy's tanh and the C library's may differ in the last bit)
                assert abs(st["phi"][z, j, i] - (1 - np.tanh((r - N / 4) * 2)) / 2) <= 1e-15
