"""ctypes front end of the FP64 CPU oracle (oracle/ttsh_oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker that the CUDA path is compared against.
Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference
legs may import this module. The product (libttsh) never calls it.

The oracle restates the reference step of TTSH3D.cu (EEuler, :347-359) in FP64
C++ with OpenMP; see the header of ttsh_oracle.cpp for the line-by-line map.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libttsh_oracle.so")
SRC = os.path.join(HERE, "ttsh_oracle.cpp")


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (-ffp-contract=off: same bits on x86 and aarch64)."""
    os.makedirs(BUILD, exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp%d" % os.getpid()
        subprocess.check_call(["g++", "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                               "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


class Params(ctypes.Structure):
    _fields_ = [("N", ctypes.c_int), ("h", ctypes.c_double), ("dt", ctypes.c_double)] + [
        (n, ctypes.c_double) for n in
        ("mu", "cA", "alpha", "beta", "eta", "La", "kappa", "lambda0", "aPhi", "kPhi", "gamma", "A", "zeta")
    ] + [("k2_mode", ctypes.c_int), ("stale_halo", ctypes.c_int)]


STATE_FIELDS = ("phi", "px", "py", "pz", "vx", "vy", "vz",
                "vxs", "vys", "vzs", "pxs", "pys", "pzs", "pv", "pp")


class State(ctypes.Structure):
    _fields_ = [(n, ctypes.POINTER(ctypes.c_double)) for n in STATE_FIELDS]


# Reference defaults (run_cuda.pl:19,30-44).
DEFAULTS = dict(h=1.0, dt=0.002, mu=1.0, cA=-1.0, alpha=-0.02, beta=4.366, eta=-0.187, La=1.0,
                kappa=-0.364, lambda0=9.0, aPhi=1.0, kPhi=1.0, gamma=1.0, A=0.0, zeta=0.0)

_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        d = ctypes.POINTER(ctypes.c_double)
        _lib.orc_step.argtypes = [ctypes.POINTER(Params), ctypes.POINTER(State), ctypes.c_int]
        _lib.orc_stencil.argtypes = [d, ctypes.c_int, ctypes.c_double, ctypes.c_int, d]
        _lib.orc_fft3.argtypes = [d, ctypes.c_int, ctypes.c_int]
        _lib.orc_project.argtypes = [d, d, d, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, d]
        _lib.orc_mass.argtypes = [d, ctypes.c_int, ctypes.c_double]
        _lib.orc_mass.restype = ctypes.c_double
        _lib.orc_max_div.argtypes = [d, d, d, ctypes.c_int, ctypes.c_double]
        _lib.orc_max_div.restype = ctypes.c_double
        _lib.orc_init_droplet.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_uint64, ctypes.c_double, d, d]
        _lib.orc_set_threads.argtypes = [ctypes.c_int]
        _lib.orc_set_threads.restype = ctypes.c_int
    return _lib


def _ptr(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def set_threads(n: int) -> int:
    return lib().orc_set_threads(n)


def make_params(N: int, k2_mode: int = 0, stale_halo: int = 1, **kw) -> Params:
    v = dict(DEFAULTS)
    v.update(kw)
    p = Params()
    p.N = N
    for k, x in v.items():
        setattr(p, k, float(x))
    p.k2_mode = k2_mode
    p.stale_halo = stale_halo
    return p


def new_state(N: int) -> dict:
    return {k: np.zeros((N, N, N), np.float64) for k in STATE_FIELDS}


def step(state: dict, nsteps: int, N: int, **kw) -> dict:
    """Advance `state` (dict of C-contiguous (N,N,N) float64 arrays, z-major) in place."""
    p = make_params(N, **kw)
    s = State(*[_ptr(state[k]) for k in STATE_FIELDS])
    rc = lib().orc_step(ctypes.byref(p), ctypes.byref(s), nsteps)
    if rc != 0:
        raise RuntimeError("orc_step failed (%d)" % rc)
    return state


def stencil(f: np.ndarray, h: float, op: int) -> np.ndarray:
    """op 0/1/2 = D_x/D_y/D_z (27-point), 3 = L (15-point); f is (N,N,N) indexed [z,y,x]."""
    f = np.ascontiguousarray(f, np.float64)
    out = np.empty_like(f)
    lib().orc_stencil(_ptr(f), f.shape[0], h, op, _ptr(out))
    return out


def fft3(c: np.ndarray, sign: int) -> np.ndarray:
    c = np.ascontiguousarray(c, np.complex128).copy()
    lib().orc_fft3(c.view(np.float64).ctypes.data_as(ctypes.POINTER(ctypes.c_double)), c.shape[0], sign)
    return c


def project(xs, ys, zs, h: float, dt: float, k2_mode: int = 0) -> np.ndarray:
    xs, ys, zs = (np.ascontiguousarray(a, np.float64) for a in (xs, ys, zs))
    out = np.empty_like(xs)
    lib().orc_project(_ptr(xs), _ptr(ys), _ptr(zs), xs.shape[0], h, dt, k2_mode, _ptr(out))
    return out


def init_droplet(N: int, R: float, xi: float, seed: int, h: float = 1.0, angular_noise: float = 0.0):
    """The benchmark droplet's initial (phi, P), restated from libttsh's ttsh_init_droplet (same bits)."""
    phi = np.zeros((N, N, N))
    P = np.zeros((3, N, N, N))
    if lib().orc_init_droplet(N, h, R, xi, seed, angular_noise, _ptr(phi), _ptr(P)) != 0:
        raise ValueError("orc_init_droplet: bad arguments")
    return phi, P


def mass(phi: np.ndarray, h: float = 1.0) -> float:
    phi = np.ascontiguousarray(phi, np.float64)
    return lib().orc_mass(_ptr(phi), phi.shape[0], h)


def max_div(vx, vy, vz, h: float = 1.0) -> float:
    vx, vy, vz = (np.ascontiguousarray(a, np.float64) for a in (vx, vy, vz))
    return lib().orc_max_div(_ptr(vx), _ptr(vy), _ptr(vz), vx.shape[0], h)
