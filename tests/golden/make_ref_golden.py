"""Generate golden fixtures by running the reference's own TTSH3D program (patched only in
init/dump/timing by oracle/make_ref.py) on a GPU.

Usage (on a machine with a CUDA GPU; the patched source must exist in oracle/_ref/):
    python tests/golden/make_ref_golden.py OUTDIR

Writes to OUTDIR:
  ref_N12.npz          init and final fields (15 each, FP64, [z,y,x]) of a 5-step run at 12^3
  ref_N12_input.dat    the input.dat used (reference defaults except N, Ts, dte, ExpoData)
  ref_N12_conf_<te>.dat  the reference's own snapshot files (ExpoConf text layout)
The fixtures are committed under tests/golden/ and checked by the CPU tests (oracle vs
reference, snapshot writer byte-for-byte vs the reference's ExpoConf).
"""
import os
import shutil
import subprocess
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "bacterial-droplet_gb300"))

FIELDS = ["phi", "px", "py", "pz", "vx", "vy", "vz", "vxs", "vys", "vzs", "pxs", "pys", "pzs", "pv", "pp"]


def smooth_random_state(N, seed):
    """Droplet phi plus smooth random P, u, u*, P* (low Fourier modes), pressures zero."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(N), np.arange(N), np.arange(N), indexing="ij")
    r = np.sqrt((x - N / 2) ** 2 + (y - N / 2) ** 2 + (z - N / 2) ** 2)
    st = {"phi": 0.5 * (1 - np.tanh((r - N / 4) / 2.0))}

    def smooth(amp):
        f = np.zeros((N, N, N))
        for _ in range(4):
            k = rng.integers(-2, 3, size=3)
            ph = rng.uniform(0, 2 * np.pi)
            f += amp * rng.uniform(0.5, 1) * np.cos(2 * np.pi * (k[0] * x + k[1] * y + k[2] * z) / N + ph)
        return f

    for n in FIELDS[1:13]:
        st[n] = smooth(0.3 if n in ("px", "py", "pz") else 0.05)
    st["pv"] = np.zeros((N, N, N))
    st["pp"] = np.zeros((N, N, N))
    return st


def write_bin(path, st, N, nfields=15):
    with open(path, "wb") as fh:
        np.array([N, nfields], np.int32).tofile(fh)
        for n in FIELDS[:nfields]:
            np.ascontiguousarray(st[n], np.float64).tofile(fh)


def read_bin(path):
    with open(path, "rb") as fh:
        N, nf = np.fromfile(fh, np.int32, 2)
        out = {}
        for n in FIELDS[:nf]:
            out[n] = np.fromfile(fh, np.float64, N ** 3).reshape(N, N, N)
    return out


# Token positions in input.dat (run_cuda.pl:53-86, TTSH3D.cu:702-739) of the values the runs change.
_POS = {"ExpoData": 4, "Nx": 8, "Ny": 9, "Nz": 10, "dt0": 13, "T0": 14, "Ts": 15, "dte": 16}


def _perl_number(v):
    """A number as run_cuda.pl prints it (integers without a decimal point)."""
    if isinstance(v, int):
        return "%d" % v
    s = repr(float(v))
    return s[:-2] if s.endswith(".0") else s


def reference_input_text(N, Ts, dte, expo=1, dt0=0.002, T0=0):
    """input.dat for the reference program: the reference defaults (tests/golden/input_default.dat,
    written by run_cuda.pl's own lines) with N, Ts, dte, ExpoData, dt0 and T0 replaced (T0 != 0:
    no conf_0.dat before the loop, evolve :301-304). Pure Python, so that the timed reference arm
    loads nothing of libttsh."""
    tok = open(os.path.join(ROOT, "tests", "golden", "input_default.dat")).read().split()
    for k, v in (("ExpoData", int(expo)), ("Nx", int(N)), ("Ny", int(N)), ("Nz", int(N)), ("dt0", float(dt0)),
                 ("T0", T0), ("Ts", float(Ts)), ("dte", float(dte))):
        tok[_POS[k]] = _perl_number(v)
    return "\n".join(tok) + "\n"


def run_reference(binary, workdir, N, st, Ts, dte, expo=1, warmup=0, nfields=15, timeout=3600, T0=0):
    os.makedirs(os.path.join(workdir, "data_1"), exist_ok=True)
    with open(os.path.join(workdir, "data_1", "input.dat"), "w") as fh:
        fh.write(reference_input_text(N, Ts, dte, expo, T0=T0))
    write_bin(os.path.join(workdir, "data_1", "init.bin"), st, N, nfields)
    env = dict(os.environ)
    env["TTSH_REF_WARMUP"] = str(warmup)
    r = subprocess.run([binary], cwd=workdir, env=env, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError("reference run failed (%d): %s" % (r.returncode, r.stdout[-2000:] + r.stderr[-2000:]))
    return r.stdout


def main(outdir):
    import make_ref
    binary = make_ref.build()
    if binary is None:
        raise SystemExit("patched reference source missing (oracle/_ref/TTSH3D_ref.cu)")
    os.makedirs(outdir, exist_ok=True)
    N = 12
    st = smooth_random_state(N, seed=12)
    work = os.path.join(outdir, "work_N12")
    shutil.rmtree(work, ignore_errors=True)
    # 5 steps (T = 0.010 > Ts = 0.009), snapshots every dte = 0.004
    log = run_reference(binary, work, N, st, Ts=0.009, dte=0.004)
    fin = read_bin(os.path.join(work, "data_1", "final.bin"))
    np.savez(os.path.join(outdir, "ref_N12.npz"), **{"init_" + k: v for k, v in st.items()},
             **{"final_" + k: v for k, v in fin.items()})
    shutil.copy(os.path.join(work, "data_1", "input.dat"), os.path.join(outdir, "ref_N12_input.dat"))
    for f in sorted(os.listdir(os.path.join(work, "data_1"))):
        if f.startswith("conf_"):
            shutil.copy(os.path.join(work, "data_1", f), os.path.join(outdir, "ref_N12_" + f))
    print(log.strip().splitlines()[-1] if log.strip() else "")
    shutil.rmtree(work, ignore_errors=True)
    print("golden written to", outdir)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_ref_golden.py OUTDIR")
    main(sys.argv[1])
