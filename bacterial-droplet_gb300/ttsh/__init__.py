"""Python front end of libttsh (the C ABI in include/ttsh.h), through ctypes.

This mirrors the reference program's host interface for the TTSH3D step
(bacterial_droplet_12-16/TTSH3D.cu): `read_input` is GetInput (:696-752),
`Sim.set_state` is InitConf's host-to-device copy (:755-896), `Sim.step` is
EEuler/run (:336-359), `Sim.get_state` and `Sim.write_conf` are ExpoConf
(:899-1014). All compute runs in libttsh's CUDA kernels; there is no CPU
fallback: if libttsh.so is missing or no GPU is visible, calls raise.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG, "lib", "libttsh.so")
HEADER = os.path.join(os.path.dirname(PKG), "include", "ttsh.h")

OK, E_INVALID, E_IO, E_PARSE, E_CUDA, E_NODEVICE, E_NOMEM, E_UNSTABLE, E_UNSUPPORTED = range(9)
K2_REFERENCE, K2_DISCRETE = 0, 1
FORM_AUTO, FORM_PLAIN, FORM_FUSED = 0, 1, 2
QUIRK_STALE_HALO = 1
READ_SUCCESS = -8848

_INT_FIELDS_A = ("TimeScheme", "RKStage", "ExplImpi", "AdapTime", "ExpoData", "InitCond", "isSimplified",
                 "checkUnStable", "Nx", "Ny", "Nz", "Nb")
_DBL_FIELDS = ("h", "dt0", "T0", "Ts", "dte", "dtVarC", "dtMax", "mu", "cA", "alpha", "beta", "eta", "La",
               "kappa", "lambda0", "aPhi", "kPhi", "gamma", "A", "init0")
# input.dat token order (run_cuda.pl:53-86, TTSH3D.cu:702-739)
INPUT_ORDER = _INT_FIELDS_A + _DBL_FIELDS + ("ReadSuccess",)


class Input(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int) for n in _INT_FIELDS_A] + [(n, ctypes.c_double) for n in _DBL_FIELDS]
                + [("ReadSuccess", ctypes.c_int)])

    def as_dict(self):
        return {n: getattr(self, n) for n in INPUT_ORDER}


class Ext(ctypes.Structure):
    _fields_ = [("zeta", ctypes.c_double), ("R", ctypes.c_double), ("xi", ctypes.c_double),
                ("seed", ctypes.c_uint64), ("precision", ctypes.c_int), ("k2_mode", ctypes.c_int),
                ("quirks", ctypes.c_int), ("form", ctypes.c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("mass", ctypes.c_double), ("max_div_u", ctypes.c_double), ("max_abs_u", ctypes.c_double),
                ("T", ctypes.c_double), ("steps", ctypes.c_int64), ("nonfinite", ctypes.c_int),
                ("reserved", ctypes.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_ if n != "reserved"}


class Tuning(ctypes.Structure):
    """ttsh_tuning: the kernel configuration of one group of equal-N droplets."""
    _fields_ = [("N", ctypes.c_int), ("n", ctypes.c_int), ("fft_kind", ctypes.c_int), ("fft_lb", ctypes.c_int),
                ("nstages", ctypes.c_int), ("radix", ctypes.c_int * 16), ("zc", ctypes.c_int * 3),
                ("ms", ctypes.c_double * 4)]

    def as_dict(self):
        return {"N": self.N, "n": self.n, "fft_kind": self.fft_kind, "fft_lb": self.fft_lb,
                "radix": list(self.radix[:self.nstages]), "zc": list(self.zc),
                "ms": {"fft": self.ms[0], "fused_rhs": self.ms[1], "fused_div": self.ms[2],
                       "fused_correct": self.ms[3]}}

    @classmethod
    def from_dict(cls, d):
        t = cls()
        t.N, t.n, t.fft_kind, t.fft_lb = d["N"], d["n"], d["fft_kind"], d["fft_lb"]
        t.nstages = len(d["radix"])
        for k, r in enumerate(d["radix"]):
            t.radix[k] = r
        for k, z in enumerate(d["zc"]):
            t.zc[k] = z
        return t


class TTSHError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s (%d): %s" % (_strerror(code), code, msg))
        self.code = code


_lib = None
_D = ctypes.POINTER(ctypes.c_double)
_VP = ctypes.c_void_p


def _signatures():
    """ctypes argument and result types of every C-ABI entry point the binding uses."""
    return {
        "ttsh_read_input": ([ctypes.c_char_p, ctypes.POINTER(Input)], ctypes.c_int),
        "ttsh_default_input": ([ctypes.POINTER(Input)], None),
        "ttsh_default_ext": ([ctypes.POINTER(Ext)], None),
        "ttsh_create": ([ctypes.POINTER(Input), ctypes.POINTER(Ext), ctypes.c_int, ctypes.POINTER(_VP)],
                        ctypes.c_int),
        "ttsh_batch_create": ([ctypes.POINTER(Input), ctypes.POINTER(Ext), ctypes.c_int, ctypes.c_int,
                               ctypes.POINTER(_VP)], ctypes.c_int),
        "ttsh_set_stream": ([_VP, _VP], ctypes.c_int),
        "ttsh_set_state": ([_VP, ctypes.c_int, _D, _D, _D, _D, _D], ctypes.c_int),
        "ttsh_init_droplet": ([ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                               ctypes.c_double, _D, _D], ctypes.c_int),
        "ttsh_step": ([_VP, ctypes.c_int], ctypes.c_int),
        "ttsh_sync": ([_VP], ctypes.c_int),
        "ttsh_get_state": ([_VP, ctypes.c_int, _D, _D, _D, _D, _D], ctypes.c_int),
        "ttsh_get_provisional": ([_VP, ctypes.c_int, _D, _D], ctypes.c_int),
        "ttsh_reduce": ([_VP, ctypes.c_int, ctypes.POINTER(Stats)], ctypes.c_int),
        "ttsh_write_conf": ([_VP, ctypes.c_int, ctypes.c_char_p], ctypes.c_int),
        "ttsh_write_conf_async": ([_VP, ctypes.c_int, ctypes.c_char_p], ctypes.c_int),
        "ttsh_conf_wait": ([_VP], ctypes.c_int),
        "ttsh_reduce_all": ([_VP, ctypes.c_int, ctypes.POINTER(Stats)], ctypes.c_int),
        "ttsh_format_conf": ([ctypes.c_int, ctypes.c_int, _D, _D, _D, ctypes.c_char_p], ctypes.c_int),
        "ttsh_destroy": ([_VP], None),
        "ttsh_strerror": ([ctypes.c_int], ctypes.c_char_p),
        "ttsh_last_error": ([], ctypes.c_char_p),
        "ttsh_num_instances": ([_VP], ctypes.c_int),
        "ttsh_instance_n": ([_VP, ctypes.c_int], ctypes.c_int),
        "ttsh_time": ([_VP], ctypes.c_double),
        "ttsh_profile_kernels": ([_VP, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_char_p), _D,
                                  ctypes.POINTER(ctypes.c_int64)], ctypes.c_int),
        "ttsh_launches_per_step": ([_VP], ctypes.c_int),
        "ttsh_struct_size": ([ctypes.c_int], ctypes.c_int),
        "ttsh_save_checkpoint": ([_VP, ctypes.c_int, ctypes.c_char_p], ctypes.c_int),
        "ttsh_init_reference": ([ctypes.POINTER(Input), ctypes.c_uint, ctypes.c_char_p, _D, _D, _D, _D, _D],
                                ctypes.c_int),
        "ttsh_run_dirs": ([ctypes.POINTER(ctypes.c_char_p), ctypes.c_int, ctypes.POINTER(Ext), ctypes.c_uint64,
                           ctypes.c_int], ctypes.c_int),
        "ttsh_snapshot_slice": ([_VP, ctypes.c_int, _D, ctypes.POINTER(ctypes.c_int), _D], ctypes.c_int),
        "ttsh_load_checkpoint": ([_VP, ctypes.c_int, ctypes.c_char_p], ctypes.c_int),
        "ttsh_partials_size": ([_VP], ctypes.c_size_t),
        "ttsh_reduce_all_async": ([_VP, ctypes.c_int, _D], ctypes.c_int),
        "ttsh_stats_from_partials": ([_VP, _D, ctypes.POINTER(Stats)], ctypes.c_int),
        "ttsh_num_groups": ([_VP], ctypes.c_int),
        "ttsh_get_tuning": ([_VP, ctypes.c_int, ctypes.POINTER(Tuning)], ctypes.c_int),
        "ttsh_set_tuning": ([_VP, ctypes.c_int, ctypes.POINTER(Tuning)], ctypes.c_int),
        "ttsh_autotune": ([_VP, ctypes.c_char_p], ctypes.c_int),
        "ttsh_step_noalloc": ([ctypes.POINTER(Input), ctypes.POINTER(Ext), ctypes.c_int] + [_VP] * 7 + [_VP],
                              ctypes.c_int),
    }


def lib():
    """Load libttsh.so (building it first if it is absent)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            from . import build as _b
            _b.build()
        L = ctypes.CDLL(LIB_PATH)
        sig = _signatures()
        for name, (args, res) in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = res
        _lib = L
    return _lib


def _strerror(code):
    try:
        return lib().ttsh_strerror(code).decode()
    except Exception:  # pragma: no cover - only when the library itself is broken
        return "error"


def _check(rc):
    if rc != OK:
        raise TTSHError(rc, lib().ttsh_last_error().decode())


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous, "arrays must be C-contiguous float64"
    return a.ctypes.data_as(_D)


def declared_symbols(header: str = HEADER):
    """Function names declared in include/ttsh.h."""
    import re
    txt = open(header).read()
    return sorted(set(re.findall(r"\b(ttsh_[a-z0-9_]+)\s*\(", txt)))


def default_input(**kw) -> Input:
    x = Input()
    lib().ttsh_default_input(ctypes.byref(x))
    for k, v in kw.items():
        setattr(x, k, v)
    return x


def default_ext(**kw) -> Ext:
    e = Ext()
    lib().ttsh_default_ext(ctypes.byref(e))
    for k, v in kw.items():
        setattr(e, k, v)
    return e


def read_input(path: str) -> Input:
    x = Input()
    _check(lib().ttsh_read_input(path.encode(), ctypes.byref(x)))
    return x


def write_input(path: str, inp: Input):
    """input.dat as run_cuda.pl:53-86 prints it (one token per line, Perl number formatting)."""
    with open(path, "w") as fh:
        for n in INPUT_ORDER:
            v = getattr(inp, n)
            if isinstance(v, float):
                s = repr(v)
                if s.endswith(".0"):
                    s = s[:-2]
                fh.write(s + "\n")
            else:
                fh.write("%d\n" % v)


def init_droplet(N: int, R: float, xi: float, seed: int, h: float = 1.0, angular_noise: float = 0.0):
    """Build-defined initial condition (host only): returns (phi, P) with P shaped (3, N, N, N)."""
    phi = np.zeros((N, N, N))
    P = np.zeros((3, N, N, N))
    _check(lib().ttsh_init_droplet(N, h, R, xi, seed, angular_noise, _p(phi), _p(P)))
    return phi, P


def init_reference(inp: Input, seed: int, conf0_path: str | None = None):
    """The reference program's own initial state (InitConf, InitCond 1 noise or InitCond 0 file)."""
    N = inp.Nx
    phi = np.zeros((N, N, N))
    P, u, us, ps = (np.zeros((3, N, N, N)) for _ in range(4))
    _check(lib().ttsh_init_reference(ctypes.byref(inp), seed, conf0_path.encode() if conf0_path else None,
                                     _p(phi), _p(P), _p(u), _p(us), _p(ps)))
    return dict(phi=phi, P=P, u=u, us=us, ps=ps)


def run_dirs(dirs, ext: Ext | None = None, seed: int = 0, device: int = -1):
    """forEach.pl's sweep as one batched run over directories that each hold an input.dat."""
    arr = (ctypes.c_char_p * len(dirs))(*[d.encode() for d in dirs])
    _check(lib().ttsh_run_dirs(arr, len(dirs), ctypes.byref(ext) if ext is not None else None, seed, device))


def format_conf(path: str, phi, P, u, expo_data: int = 1):
    N = phi.shape[0]
    _check(lib().ttsh_format_conf(N, expo_data, _p(np.ascontiguousarray(phi)), _p(np.ascontiguousarray(P)),
                                  _p(np.ascontiguousarray(u)), path.encode()))


class Sim:
    """A batch of droplets on one GPU (ttsh_batch_create)."""

    def __init__(self, inputs, exts=None, device: int = -1):
        if isinstance(inputs, Input):
            inputs = [inputs]
        if exts is not None and isinstance(exts, Ext):
            exts = [exts]
        n = len(inputs)
        ia = (Input * n)(*inputs)
        ea = (Ext * n)(*exts) if exts is not None else None
        h = _VP()
        _check(lib().ttsh_batch_create(ia, ea, n, device, ctypes.byref(h)))
        self._h = h
        self.n = n
        self.sizes = [lib().ttsh_instance_n(h, i) for i in range(n)]

    def close(self):
        if getattr(self, "_h", None):
            lib().ttsh_destroy(self._h)
            self._h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_stream(self, stream_ptr: int | None):
        _check(lib().ttsh_set_stream(self._h, stream_ptr))

    def set_state(self, inst, phi, P, u, ustar=None, Pstar=None):
        c = np.ascontiguousarray
        args = [c(phi, np.float64), c(P, np.float64), c(u, np.float64)]
        us = None if ustar is None else c(ustar, np.float64)
        ps = None if Pstar is None else c(Pstar, np.float64)
        _check(lib().ttsh_set_state(self._h, inst, _p(args[0]), _p(args[1]), _p(args[2]), _p(us), _p(ps)))

    def step(self, nsteps: int = 1):
        _check(lib().ttsh_step(self._h, nsteps))

    def sync(self):
        _check(lib().ttsh_sync(self._h))

    def get_state(self, inst: int = 0):
        N = self.sizes[inst]
        phi = np.empty((N, N, N))
        P = np.empty((3, N, N, N))
        u = np.empty((3, N, N, N))
        pv = np.empty((N, N, N))
        pp = np.empty((N, N, N))
        _check(lib().ttsh_get_state(self._h, inst, _p(phi), _p(P), _p(u), _p(pv), _p(pp)))
        return dict(phi=phi, P=P, u=u, pv=pv, pp=pp)

    def get_provisional(self, inst: int = 0):
        N = self.sizes[inst]
        us = np.empty((3, N, N, N))
        ps = np.empty((3, N, N, N))
        _check(lib().ttsh_get_provisional(self._h, inst, _p(us), _p(ps)))
        return us, ps

    def reduce(self, inst: int = 0, check: bool = True) -> dict:
        st = Stats()
        rc = lib().ttsh_reduce(self._h, inst, ctypes.byref(st))
        if check or rc != E_UNSTABLE:
            _check(rc)
        return st.as_dict()

    def partials_size(self) -> int:
        return int(lib().ttsh_partials_size(self._h))

    def reduce_all_async(self, buf, mass_only: bool = False):
        """Enqueue the diagnostics of every droplet into `buf` (float64, contiguous, at least
        partials_size() values; page-locked for an asynchronous copy) without waiting."""
        assert buf.dtype == np.float64 and buf.flags.c_contiguous and buf.size >= self.partials_size()
        _check(lib().ttsh_reduce_all_async(self._h, 1 if mass_only else 0, buf.ctypes.data_as(_D)))

    def stats_from_partials(self, buf, check: bool = True):
        """Per-droplet diagnostics of a buffer filled by reduce_all_async (after sync())."""
        arr = (Stats * self.n)()
        rc = lib().ttsh_stats_from_partials(self._h, buf.ctypes.data_as(_D), arr)
        if check or rc != E_UNSTABLE:
            _check(rc)
        return [a.as_dict() for a in arr]

    def reduce_all(self, mass_only: bool = False, check: bool = True):
        """FP64 diagnostics of every droplet (one pass per size group, one copy back)."""
        arr = (Stats * self.n)()
        rc = lib().ttsh_reduce_all(self._h, 1 if mass_only else 0, arr)
        if check or rc != E_UNSTABLE:
            _check(rc)
        return [a.as_dict() for a in arr]

    def write_conf(self, inst: int, path: str):
        _check(lib().ttsh_write_conf(self._h, inst, path.encode()))

    def write_conf_async(self, inst: int, path: str):
        """Enqueue the snapshot file; it is formatted while later steps run (conf_wait to finish)."""
        _check(lib().ttsh_write_conf_async(self._h, inst, path.encode()))

    def conf_wait(self):
        _check(lib().ttsh_conf_wait(self._h))

    SLICE_NAMES = ("vx", "vy", "vz", "px", "py", "pz", "phi", "vortex", "Pvortex")

    def snapshot_slice(self, inst: int = 0):
        """readDraw.py's centroid, centroid z-slice and vorticities, computed on the GPU."""
        N = self.sizes[inst]
        c = (ctypes.c_double * 3)()
        idx = (ctypes.c_int * 3)()
        out = np.empty((9, N, N))
        _check(lib().ttsh_snapshot_slice(self._h, inst, c, idx, _p(out)))
        res = {n: out[i] for i, n in enumerate(self.SLICE_NAMES)}
        res["centroid"] = tuple(c)
        res["index"] = tuple(idx)
        return res

    def save_checkpoint(self, inst: int, path: str):
        _check(lib().ttsh_save_checkpoint(self._h, inst, path.encode()))

    def load_checkpoint(self, inst: int, path: str):
        _check(lib().ttsh_load_checkpoint(self._h, inst, path.encode()))

    def time(self) -> float:
        return lib().ttsh_time(self._h)

    def launches_per_step(self) -> int:
        return lib().ttsh_launches_per_step(self._h)

    def tuning(self):
        """The kernel configuration of every group of equal-N droplets (list of dicts)."""
        out = []
        for g in range(lib().ttsh_num_groups(self._h)):
            t = Tuning()
            _check(lib().ttsh_get_tuning(self._h, g, ctypes.byref(t)))
            out.append(t.as_dict())
        return out

    def set_tuning(self, group: int, cfg: dict):
        _check(lib().ttsh_set_tuning(self._h, group, ctypes.byref(Tuning.from_dict(cfg))))

    def autotune(self, cache: str = None):
        """Times the kernel candidates of every group on the current fields and keeps the fastest
        (the state is left as it was); returns the chosen configurations with their timings."""
        _check(lib().ttsh_autotune(self._h, None if cache is None else cache.encode()))
        return self.tuning()

    def profile_kernels(self, nsteps: int):
        cap = 16
        names = (ctypes.c_char_p * cap)()
        ms = (ctypes.c_double * cap)()
        cnt = (ctypes.c_int64 * cap)()
        k = lib().ttsh_profile_kernels(self._h, nsteps, cap, names, ms, cnt)
        if k < 0:
            _check(-k)
        return {names[i].decode(): (ms[i], int(cnt[i])) for i in range(k)}
