"""numpy front end for the CPU oracle.  TEST INFRASTRUCTURE ONLY.

`Oracle("orc")` drives liboracle.so, the C restatement of KFR's DFT path (kfr_oracle.c); `Oracle("ref")`
drives oracle/_ref/libkfr_ref.so, KFR 7.0.1 itself built from the reference sources (ref_driver.cpp),
which exists only where the reference is present.  Both expose the same entry points, so every check can
be run against either.  Only tests, the smoke check and the benchmark's CPU-baseline leg import this.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATHS = {
    "orc": os.path.join(HERE, "liboracle.so"),
    "ref": os.path.join(HERE, "_ref", "libkfr_ref.so"),
}

_c_size = ctypes.c_size_t
_c_int = ctypes.c_int
_ptr = ctypes.c_void_p


REF_SRC_DEFAULT = os.path.join(os.path.dirname(HERE), "baseline", "_ref", "kfr")


def ref_sources() -> str | None:
    """Where the reference's sources for oracle/_ref are: $KFR_SRC, else the git-ignored copy that
    oracle/stage_ref.sh makes under baseline/_ref/kfr; None if neither exists."""
    for d in (os.environ.get("KFR_SRC"), REF_SRC_DEFAULT):
        if d and os.path.exists(os.path.join(d, "src", "dft", "dft.cpp")):
            return d
    return None


def build_command(ref: bool = False) -> list[str] | None:
    """make command for liboracle.so (ref=False) or for the reference library (ref=True; None when the
    reference sources are absent)."""
    if not ref:
        return ["make", "-s", "-C", HERE, "oracle"]
    src = ref_sources()
    return ["make", "-s", "-C", HERE, f"-j{os.cpu_count() or 4}", "ref", f"KFR_SRC={src}"] if src else None


def build(ref: bool = False) -> None:
    """Compile liboracle.so and, if asked and the reference sources exist, try the reference library (a
    failure there leaves only the restatement available)."""
    subprocess.check_call(build_command(False))
    cmd = build_command(True) if ref else None
    if cmd and subprocess.call(cmd) != 0:
        print("oracle/_ref: the reference library did not build; the oracle's restatement stays available")


def available(kind: str) -> bool:
    return os.path.exists(LIB_PATHS[kind])


def _p(a: np.ndarray):
    return a.ctypes.data_as(_ptr)


class Oracle:
    """CPU DFT oracle with KFR's conventions: unscaled inverses, CCs/Perm real packing, DCT-II/III."""

    def __init__(self, kind: str = "orc"):
        path = LIB_PATHS[kind]
        if not os.path.exists(path):
            if kind == "orc":
                build()
            else:
                raise FileNotFoundError(path)
        self.kind = kind
        self.lib = ctypes.CDLL(path)
        pre = "orc_" if kind == "orc" else "ref_"
        self.pre = pre
        for sfx in ("_f64", "_f32"):
            for name, res, args in [
                ("dft", _c_int, [_ptr, _ptr, _c_size, _c_size, _c_int, _c_int]),
                ("dft_real", _c_int, [_ptr, _ptr, _c_size, _c_int, _c_size, _c_int]),
                ("dft_real_inverse", _c_int, [_ptr, _ptr, _c_size, _c_int, _c_size, _c_int]),
                ("dct", _c_int, [_ptr, _ptr, _c_size, _c_int, _c_size, _c_int]),
                ("convolve", _c_size, [_ptr, _ptr, _c_size, _ptr, _c_size, _c_int, _c_int]),
                ("filter_create", _ptr, [_ptr, _c_size, _c_size, _c_int]),
                ("filter_process", None, [_ptr, _ptr, _ptr, _c_size]),
                ("filter_reset", None, [_ptr]),
                ("filter_delete", None, [_ptr]),
            ]:
                f = getattr(self.lib, pre + name + sfx)
                f.restype = res
                f.argtypes = args
        if kind == "orc":
            self.lib.orc_filter_batch_f32.restype = None
            self.lib.orc_filter_batch_f32.argtypes = [_ptr, _ptr, _c_size, _c_size, _ptr, _c_size, _c_size, _c_int]

    def _fn(self, name, dtype):
        return getattr(self.lib, self.pre + name + ("_f64" if dtype == np.float64 else "_f32"))

    @staticmethod
    def _rdt(precision):
        return np.float64 if precision == "f64" else np.float32

    # ---- complex DFT -------------------------------------------------------------------------------
    def dft(self, x, inverse=False, precision="f64", threads=1):
        """Unscaled complex DFT along the last axis (forward: e^{-2 pi i nk/N})."""
        rdt = self._rdt(precision)
        cdt = np.complex128 if rdt == np.float64 else np.complex64
        x = np.ascontiguousarray(x, dtype=cdt)
        n = x.shape[-1]
        batch = x.size // n if n else 0
        out = np.empty_like(x)
        if n:
            self._fn("dft", rdt)(_p(out), _p(x), n, batch, int(inverse), threads)
        return out

    def dft_time(self, x, inverse=False, threads=1, reps=3):
        """Best wall time (seconds) of one c32 DFT pass over the batch x (signals along the last axis) with
        the plan built once beforehand and shared by `threads` threads (KFR's dft_plan<float>; ref only)."""
        if self.kind != "ref":
            raise RuntimeError("dft_time times the reference library")
        f = self.lib.ref_dft_time_f32
        f.restype = ctypes.c_double
        f.argtypes = [_ptr, _ptr, _c_size, _c_size, _c_int, _c_int, _c_int]
        x = np.ascontiguousarray(x, dtype=np.complex64)
        n = x.shape[-1]
        out = np.empty_like(x)
        return float(f(_p(out), _p(x), n, x.size // n, int(inverse), threads, reps))

    def fft_multiply(self, a, b, acc=None, perm=False):
        """fft_multiply(a, b) or, with acc, fft_multiply_accumulate(acc, a, b) along the last axis (element 0
        part by part in the Perm format); precision follows a's dtype (complex64 or complex128)."""
        a = np.ascontiguousarray(a)
        f = getattr(self.lib, self.pre + "fft_multiply" + ("_f64" if a.dtype == np.complex128 else "_f32"))
        f.restype = None
        f.argtypes = [_ptr, _ptr, _ptr, _ptr, _c_size, _c_int]
        b = np.ascontiguousarray(np.broadcast_to(b, a.shape), dtype=a.dtype)
        acc = None if acc is None else np.ascontiguousarray(np.broadcast_to(acc, a.shape), dtype=a.dtype)
        out = np.empty_like(a)
        n = a.shape[-1]
        for i in range(a.size // n if n else 0):
            sl = np.s_[i * n:(i + 1) * n]
            o, x, y = out.reshape(-1)[sl], a.reshape(-1)[sl], b.reshape(-1)[sl]
            z = None if acc is None else acc.reshape(-1)[sl]
            f(_p(o), None if z is None else _p(z), _p(x), _p(y), n, int(perm))
        return out

    # ---- real DFT ----------------------------------------------------------------------------------
    def dft_real(self, x, ccs=True, precision="f64", threads=1):
        rdt = self._rdt(precision)
        cdt = np.complex128 if rdt == np.float64 else np.complex64
        x = np.ascontiguousarray(x, dtype=rdt)
        n = x.shape[-1]
        batch = x.size // n
        cs = n // 2 + 1 if ccs else n // 2
        out = np.zeros(x.shape[:-1] + (cs,), dtype=cdt)
        rc = self._fn("dft_real", rdt)(_p(out), _p(x), n, int(ccs), batch, threads)
        if rc != 0:
            raise ValueError("dft_plan_real requires size to be even")
        return out

    def dft_real_inverse(self, X, n, ccs=True, precision="f64", threads=1):
        rdt = self._rdt(precision)
        cdt = np.complex128 if rdt == np.float64 else np.complex64
        X = np.ascontiguousarray(X, dtype=cdt)
        cs = n // 2 + 1 if ccs else n // 2
        assert X.shape[-1] == cs
        batch = X.size // cs
        out = np.zeros(X.shape[:-1] + (n,), dtype=rdt)
        rc = self._fn("dft_real_inverse", rdt)(_p(out), _p(X), n, int(ccs), batch, threads)
        if rc != 0:
            raise ValueError("dft_plan_real requires size to be even")
        return out

    # ---- DCT ---------------------------------------------------------------------------------------
    def dct(self, x, inverse=False, precision="f64", threads=1):
        rdt = self._rdt(precision)
        x = np.ascontiguousarray(x, dtype=rdt)
        n = x.shape[-1]
        batch = x.size // n
        out = np.empty_like(x)
        self._fn("dct", rdt)(_p(out), _p(x), n, int(inverse), batch, threads)
        return out

    # ---- convolution -------------------------------------------------------------------------------
    def convolve(self, a, b, correlate=False, precision="f64"):
        rdt = self._rdt(precision)
        is_complex = np.iscomplexobj(a) or np.iscomplexobj(b)
        if is_complex:
            cdt = np.complex128 if rdt == np.float64 else np.complex64
            a = np.ascontiguousarray(a, dtype=cdt)
            b = np.ascontiguousarray(b, dtype=cdt)
            out = np.zeros(len(a) + len(b) - 1, dtype=cdt)
        else:
            a = np.ascontiguousarray(a, dtype=rdt)
            b = np.ascontiguousarray(b, dtype=rdt)
            out = np.zeros(len(a) + len(b) - 1, dtype=rdt)
        n = self._fn("convolve", rdt)(_p(out), _p(a), len(a), _p(b), len(b), int(correlate), int(is_complex))
        return out[:n]

    # ---- multi-dimensional (reference library only) ---------------------------------------------------
    def dft_md(self, x, inverse=False):
        """dft_plan_md<double> over the whole array (reference build only)."""
        x = np.ascontiguousarray(x, dtype=np.complex128)
        shp = (ctypes.c_uint * x.ndim)(*x.shape)
        out = np.empty_like(x)
        f = self.lib.ref_dft_md_f64
        f.restype = _c_int
        f.argtypes = [_ptr, _ptr, _c_size, _ptr, _c_int]
        f(_p(out), _p(x), x.ndim, ctypes.cast(shp, _ptr), int(inverse))
        return out

    def dft_md_real(self, x, inverse=False, shape=None, real_out_is_enough=False):
        """dft_plan_md_real<double>: forward real -> CCs complex (last axis N/2+1), inverse back (reference only)."""
        f = self.lib.ref_dft_md_real_f64
        f.restype = _c_int
        f.argtypes = [_ptr, _ptr, _c_size, _ptr, _c_int, _c_int]
        if not inverse:
            x = np.ascontiguousarray(x, dtype=np.float64)
            shape = x.shape
            out = np.zeros(shape[:-1] + (shape[-1] // 2 + 1,), dtype=np.complex128)
        else:
            x = np.ascontiguousarray(x, dtype=np.complex128)
            out = np.zeros(shape, dtype=np.float64)
        shp = (ctypes.c_uint * len(shape))(*shape)
        f(_p(out), _p(x), len(shape), ctypes.cast(shp, _ptr), int(inverse), int(real_out_is_enough))
        return out

    def filter(self, taps, block=1024, precision="f64"):
        return _Filter(self, taps, block, precision)

    def fir(self, taps, precision="f64"):
        """Streaming direct-form FIR (fir_filter<T>): y[n] = sum_k taps[k] x[n - k], state across calls."""
        return _Fir(self, taps, precision)


class _Filter:
    """Streaming convolve_filter state (reset, process)."""

    def __init__(self, orc: Oracle, taps, block, precision):
        self.orc = orc
        self.rdt = Oracle._rdt(precision)
        self.is_complex = np.iscomplexobj(taps)
        self.dt = (np.complex128 if self.rdt == np.float64 else np.complex64) if self.is_complex else self.rdt
        t = np.ascontiguousarray(taps, dtype=self.dt)
        self.h = orc._fn("filter_create", self.rdt)(_p(t), len(t), block, int(self.is_complex))

    def process(self, x):
        x = np.ascontiguousarray(x, dtype=self.dt)
        out = np.empty_like(x)
        self.orc._fn("filter_process", self.rdt)(self.h, _p(out), _p(x), len(x))
        return out

    def reset(self):
        self.orc._fn("filter_reset", self.rdt)(self.h)

    def __del__(self):
        try:
            self.orc._fn("filter_delete", self.rdt)(self.h)
        except Exception:
            pass


def rel_rms(got, ref) -> float:
    """Relative RMS error ||got - ref||_2 / ||ref||_2, computed in float64."""
    got = np.asarray(got, dtype=np.complex128 if np.iscomplexobj(got) or np.iscomplexobj(ref) else np.float64)
    ref = np.asarray(ref, dtype=got.dtype)
    den = np.sqrt(np.sum(np.abs(ref) ** 2))
    num = np.sqrt(np.sum(np.abs(got - ref) ** 2))
    return float(num / den) if den > 0 else float(num)


def c32_tolerance(n: int) -> float:
    """Relative-RMS bound for single-precision complex results: 2 * log2(N) * 2^-24 (at least N=2)."""
    return 2.0 * max(np.log2(max(n, 2)), 1.0) * 2.0 ** -24


def c64_tolerance(n: int) -> float:
    """Relative-RMS bound for double-precision complex results: 4 * log2(N) * 2^-53."""
    return 4.0 * max(np.log2(max(n, 2)), 1.0) * 2.0 ** -53


class _Fir:
    """Streaming fir_filter state (reset, process); real samples."""

    def __init__(self, orc: Oracle, taps, precision):
        self.orc = orc
        self.rdt = Oracle._rdt(precision)
        sfx = "_f64" if self.rdt == np.float64 else "_f32"
        self.fns = {}
        for name, res, args in (("create", _ptr, [_ptr, _c_size]), ("process", None, [_ptr, _ptr, _ptr, _c_size]),
                                ("reset", None, [_ptr]), ("delete", None, [_ptr])):
            f = getattr(orc.lib, orc.pre + "fir_" + name + sfx)
            f.restype = res
            f.argtypes = args
            self.fns[name] = f
        t = np.ascontiguousarray(taps, dtype=self.rdt)
        self.h = self.fns["create"](_p(t), len(t))

    def process(self, x):
        x = np.ascontiguousarray(x, dtype=self.rdt)
        out = np.empty_like(x)
        self.fns["process"](self.h, _p(out), _p(x), len(x))
        return out

    def reset(self):
        self.fns["reset"](self.h)

    def __del__(self):
        try:
            self.fns["delete"](self.h)
        except Exception:
            pass
