"""kfr_gb300: KFR's DFT hot path on one GB300 GPU, behind KFR's own C API.

The product is the shared library kfr_gb300/lib/libkfr_capi.so (CUDA kernels for sm_103a plus the C ABI
declared in include/kfr_capi.h).  This module is a thin ctypes mirror of the reference's plan objects, used
by the tests and the benchmark and usable from Python directly:

    dft_plan(n, "f32").execute(out, x)              # include/kfr/dft/fft.hpp:183-456
    dft_plan_real(n, "CCs").execute(out, x)         # include/kfr/dft/fft.hpp:458-566
    dct_plan(n).execute(out, x, inverse=False)      # include/kfr/dft/fft.hpp:926-978
    convolve_filter(taps, block_size).apply(y, x)   # include/kfr/dft/convolution.hpp:98-148

Buffers may be numpy arrays (host memory) or torch tensors / objects exposing data_ptr() (device or host).
Errors reported by the library through kfr_last_error() are raised as KfrError.  There is no CPU fallback:
if the library or a GPU is missing, calls fail.
"""
from __future__ import annotations

import ctypes
import os
import re

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libkfr_capi.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "kfr_capi.h")

__all__ = ["KfrError", "lib", "dft_plan", "dft_plan_md", "dft_plan_real", "dft_plan_md_real", "dct_plan",
           "convolve_filter", "fir_filter", "declared_symbols", "fft_multiply", "CCs", "Perm"]

CCs = 1
Perm = 0


class KfrError(RuntimeError):
    pass


_lib = None

_P = ctypes.c_void_p
_S = ctypes.c_size_t
_B = ctypes.c_bool

# name -> (restype, argtypes); every pointer is passed as an integer address
_SIGS = {}
for sfx in ("f32", "f64"):
    _SIGS.update({
        f"kfr_dft_create_plan_{sfx}": (_P, [_S]),
        f"kfr_dft_create_2d_plan_{sfx}": (_P, [_S, _S]),
        f"kfr_dft_create_3d_plan_{sfx}": (_P, [_S, _S, _S]),
        f"kfr_dft_create_md_plan_{sfx}": (_P, [_S, _P]),
        f"kfr_dft_dump_{sfx}": (None, [_P]),
        f"kfr_dft_get_size_{sfx}": (_S, [_P]),
        f"kfr_dft_get_temp_size_{sfx}": (_S, [_P]),
        f"kfr_dft_get_temp_size_batch_{sfx}": (_S, [_P, _S]),
        f"kfr_dft_execute_{sfx}": (None, [_P, _P, _P, _P]),
        f"kfr_dft_execute_inverse_{sfx}": (None, [_P, _P, _P, _P]),
        f"kfr_dft_execute_batch_{sfx}": (None, [_P, _S, _P, _P, _P, _B, _P]),
        f"kfr_dft_delete_plan_{sfx}": (None, [_P]),
        f"kfr_dft_real_create_plan_{sfx}": (_P, [_S, ctypes.c_int]),
        f"kfr_dft_real_create_2d_plan_{sfx}": (_P, [_S, _S, _B]),
        f"kfr_dft_real_create_3d_plan_{sfx}": (_P, [_S, _S, _S, _B]),
        f"kfr_dft_real_create_md_plan_{sfx}": (_P, [_S, _P, _B]),
        f"kfr_dft_real_dump_{sfx}": (None, [_P]),
        f"kfr_dft_real_get_size_{sfx}": (_S, [_P]),
        f"kfr_dft_real_get_temp_size_{sfx}": (_S, [_P]),
        f"kfr_dft_real_get_temp_size_batch_{sfx}": (_S, [_P, _S]),
        f"kfr_dft_real_execute_{sfx}": (None, [_P, _P, _P, _P]),
        f"kfr_dft_real_execute_inverse_{sfx}": (None, [_P, _P, _P, _P]),
        f"kfr_dft_real_execute_batch_{sfx}": (None, [_P, _S, _P, _P, _P, _P]),
        f"kfr_dft_real_execute_inverse_batch_{sfx}": (None, [_P, _S, _P, _P, _P, _P]),
        f"kfr_dft_real_delete_plan_{sfx}": (None, [_P]),
        f"kfr_dct_create_plan_{sfx}": (_P, [_S]),
        f"kfr_dct_dump_{sfx}": (None, [_P]),
        f"kfr_dct_get_size_{sfx}": (_S, [_P]),
        f"kfr_dct_get_temp_size_{sfx}": (_S, [_P]),
        f"kfr_dct_get_temp_size_batch_{sfx}": (_S, [_P, _S]),
        f"kfr_dct_execute_{sfx}": (None, [_P, _P, _P, _P]),
        f"kfr_dct_execute_inverse_{sfx}": (None, [_P, _P, _P, _P]),
        f"kfr_dct_execute_batch_{sfx}": (None, [_P, _S, _P, _P, _P, _B, _P]),
        f"kfr_dct_delete_plan_{sfx}": (None, [_P]),
        f"kfr_filter_create_fir_plan_{sfx}": (_P, [_P, _S]),
        f"kfr_filter_create_iir_plan_{sfx}": (_P, [_P, _S]),
        f"kfr_filter_create_convolution_plan_{sfx}": (_P, [_P, _S, _S]),
        f"kfr_filter_process_{sfx}": (None, [_P, _P, _P, _S]),
        f"kfr_filter_reset_{sfx}": (None, [_P]),
        f"kfr_filter_delete_plan_{sfx}": (None, [_P]),
        f"kfr_dft_adjoint_batch_{sfx}": (None, [_P, _S, _P, _P, _P, _B, _P]),
        f"kfr_dft_real_adjoint_batch_{sfx}": (None, [_P, _S, _P, _P, _P, _P]),
        f"kfr_dft_real_adjoint_inverse_batch_{sfx}": (None, [_P, _S, _P, _P, _P, _P]),
        f"kfr_dct_adjoint_batch_{sfx}": (None, [_P, _S, _P, _P, _P, _B, _P]),
        f"kfr_fir_backward_{sfx}": (None, [_P, _S, _S, _S, _P, _P, _P, _P, _P]),
        f"kfr_filter_create_convolution_plan_channels_{sfx}": (_P, [_P, _S, _S, _S]),
    })
for fn in ("convolve", "correlate"):
    for sfx in ("f32", "f64", "c32", "c64"):
        _SIGS[f"kfr_{fn}_{sfx}"] = (_S, [_P, _P, _S, _P, _S])
_SIGS.update({
    "kfr_version_string": (ctypes.c_char_p, []),
    "kfr_version": (ctypes.c_uint32, []),
    "kfr_enabled_archs": (ctypes.c_char_p, []),
    "kfr_current_arch": (ctypes.c_int, []),
    "kfr_last_error": (ctypes.c_char_p, []),
    "kfr_allocate": (_P, [_S]),
    "kfr_allocate_aligned": (_P, [_S, _S]),
    "kfr_deallocate": (None, [_P]),
    "kfr_reallocate": (_P, [_P, _S]),
    "kfr_reallocate_aligned": (_P, [_P, _S, _S]),
    "kfr_add_ref": (_P, [_P]),
    "kfr_release": (None, [_P]),
    "kfr_allocated_size": (_S, [_P]),
    "kfr_dft_describe_f64": (_S, [_P, ctypes.c_char_p, _S]),
    "kfr_set_wait_limit": (ctypes.c_uint32, [ctypes.c_uint32]),
    "kfr_dft_progressive_total_steps_f32": (_S, [_P]),
    "kfr_dft_progressive_total_steps_f64": (_S, [_P]),
    "kfr_dft_progressive_start_f32": (_S, [_P, _P, _P, _P, _B]),
    "kfr_dft_progressive_start_f64": (_S, [_P, _P, _P, _P, _B]),
    "kfr_dft_progressive_step_f32": (_B, [_P, _S]),
    "kfr_dft_progressive_step_f64": (_B, [_P, _S]),
    "kfr_dft_uneven_set_unreachable_stage_f32": (None, [_P, _B]),
    "kfr_fft_multiply_f32": (None, [_P, _P, _P, _S, _S, _B, ctypes.c_int, _P]),
    "kfr_fft_multiply_f64": (None, [_P, _P, _P, _S, _S, _B, ctypes.c_int, _P]),
    "kfr_fft_multiply_accumulate_f32": (None, [_P, _P, _P, _P, _S, _S, _B, ctypes.c_int, _P]),
    "kfr_fft_multiply_accumulate_f64": (None, [_P, _P, _P, _P, _S, _S, _B, ctypes.c_int, _P]),
    "kfr_dft_get_launch_count_f64": (_S, [_P, _S]),
    "kfr_dft_get_launch_count_f32": (_S, [_P, _S]),
    "kfr_dft_describe_f32": (_S, [_P, ctypes.c_char_p, _S]),
    "kfr_dft_execute_static_scratch_f32": (None, [_P, _S, _P, _P, _B, _P]),
    "kfr_dft_cache_size": (_S, []),
    "kfr_dft_cache_clear": (None, []),
    "kfr_autocorrelate_f32": (_S, [_P, _P, _S]),
    "kfr_autocorrelate_f64": (_S, [_P, _P, _S]),
    "kfr_dft_create_uneven_plan_f32": (_P, [_P, _S, _B]),
    "kfr_dft_create_plan_tensor_f32": (_P, [_S, ctypes.c_int]),
    "kfr_dft_uneven_get_size_f32": (_S, [_P]),
    "kfr_dft_uneven_execute_f32": (None, [_P, _P, _P, _B, _P]),
    "kfr_dft_uneven_execute_per_signal_f32": (None, [_P, _P, _P, _B, _P]),
    "kfr_dft_uneven_describe_f32": (_S, [_P, ctypes.c_char_p, _S]),
    "kfr_dft_uneven_delete_plan_f32": (None, [_P]),
})


def declared_symbols(header: str = HEADER) -> list[str]:
    """Every function name declared in include/kfr_capi.h."""
    text = open(header).read()
    return sorted(set(re.findall(r"KFR_API_SPEC\s+[\w\s\*]+?\b(kfr_\w+)\s*\(", text)))


def lib():
    """The loaded C-ABI library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise KfrError(f"{LIB_PATH} is missing: build it with `python -m kfr_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def _check():
    msg = lib().kfr_last_error()
    if msg:
        raise KfrError(msg.decode())


def _call(name, *args):
    r = getattr(lib(), name)(*args)
    _check()
    return r


def _addr(x):
    """Address of a buffer: numpy array (host), torch tensor (host or device), int, or None."""
    if x is None:
        return None
    if isinstance(x, int):
        return x
    if isinstance(x, np.ndarray):
        if not x.flags["C_CONTIGUOUS"]:
            raise ValueError("buffers must be contiguous")
        return x.ctypes.data
    if hasattr(x, "data_ptr"):
        if hasattr(x, "is_contiguous") and not x.is_contiguous():
            raise ValueError("buffers must be contiguous")
        return x.data_ptr()
    raise TypeError(f"unsupported buffer type {type(x)}")


def _sfx(dtype) -> str:
    d = str(dtype)
    if d in ("f32", "float32", "complex64", "<class 'numpy.float32'>", "<class 'numpy.complex64'>", "torch.float32",
             "torch.complex64"):
        return "f32"
    if d in ("f64", "float64", "complex128", "<class 'numpy.float64'>", "<class 'numpy.complex128'>",
             "torch.float64", "torch.complex128"):
        return "f64"
    raise ValueError(f"unsupported precision {dtype}")


def _stream_addr(stream):
    if stream is None:
        return None
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream) if hasattr(stream, "cuda_stream") else int(stream)


class _plan:
    _prefix = ""

    def __init__(self, handle, sfx):
        if not handle:
            _check()
            raise KfrError("plan creation failed")
        self.handle = handle
        self.sfx = sfx

    def _fn(self, op):
        return f"{self._prefix}_{op}_{self.sfx}"

    def close(self):
        if getattr(self, "handle", None):
            getattr(lib(), self._fn("delete_plan"))(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def dump(self):
        _call(self._fn("dump"), self.handle)


class dft_plan(_plan):
    """Complex DFT of length `size` (dft_plan<T>, include/kfr/dft/fft.hpp:183-456); unscaled inverse."""

    _prefix = "kfr_dft"

    def __init__(self, size: int, dtype="f32"):
        sfx = _sfx(dtype)
        super().__init__(_call(f"kfr_dft_create_plan_{sfx}", size), sfx)

    @property
    def size(self):
        return _call(self._fn("get_size"), self.handle)

    @property
    def temp_size(self):
        return _call(self._fn("get_temp_size"), self.handle)

    def temp_size_batch(self, batch):
        return _call(self._fn("get_temp_size_batch"), self.handle, batch)

    def execute(self, out, inp, temp=None, inverse=False):
        op = "execute_inverse" if inverse else "execute"
        _call(self._fn(op), self.handle, _addr(out), _addr(inp), _addr(temp))

    def execute_batch(self, out, inp, batch, temp=None, inverse=False, stream=None):
        _call(self._fn("execute_batch"), self.handle, batch, _addr(out), _addr(inp), _addr(temp), bool(inverse),
              _stream_addr(stream))

    def adjoint_batch(self, grad_in, grad_out, batch, inverse=False, stream=None):
        """Gradient of the input of execute_batch(inverse) from the gradient of its output."""
        _call(self._fn("adjoint_batch"), self.handle, batch, _addr(grad_in), _addr(grad_out), None, bool(inverse),
              _stream_addr(stream))

    def describe(self) -> str:
        buf = ctypes.create_string_buffer(512)
        _call(f"kfr_dft_describe_{self.sfx}", self.handle, buf, 512)
        return buf.value.decode()

    def progressive_total_steps(self) -> int:
        """Steps of a progressive execution: one kernel launch each (include/kfr/dft/fft.hpp:403-405)."""
        return _call(self._fn("progressive_total_steps"), self.handle)

    def progressive_start(self, out, inp, temp=None, inverse=False) -> int:
        """Records one execution for these buffers; returns its number of steps."""
        self._prog = (out, inp, temp)  # keep the buffers alive until the last step
        return _call(self._fn("progressive_start"), self.handle, _addr(out), _addr(inp), _addr(temp), inverse)

    def progressive_step(self, step: int) -> bool:
        """Runs one step; True while steps remain."""
        return bool(_call(self._fn("progressive_step"), self.handle, step))

    def launch_count(self, batch=1):
        return _call(f"kfr_dft_get_launch_count_{self.sfx}", self.handle, batch)


class dft_plan_tensor(dft_plan):
    """Complex c32 plan whose radix-16 passes run on the tensor cores with split 16-bit operands (split:
    "bf16" = hi + mid + lo, "fp16" = scaled hi + lo); lengths 256, 4096, 2^16, 2^20 and 2^24."""

    def __init__(self, size: int, split="fp16"):
        mode = {"bf16": 1, "fp16": 2}[split]
        _plan.__init__(self, _call("kfr_dft_create_plan_tensor_f32", size, mode), "f32")


class dft_plan_md(dft_plan):
    """Multi-dimensional complex DFT over a row-major array (dft_plan_md<T>, include/kfr/dft/fft.hpp:568-702)."""

    def __init__(self, shape, dtype="f32"):
        sfx = _sfx(dtype)
        self.shape = tuple(int(v) for v in shape)
        arr = (ctypes.c_uint * len(self.shape))(*self.shape)
        _plan.__init__(self, _call(f"kfr_dft_create_md_plan_{sfx}", len(self.shape), ctypes.cast(arr, _P)), sfx)


class dft_plan_md_real(_plan):
    """Multi-dimensional real DFT (dft_plan_md_real<T>, include/kfr/dft/fft.hpp:704-924): real array of
    `shape` <-> CCs complex array whose last axis has shape[-1]//2 + 1 values."""

    _prefix = "kfr_dft_real"

    def __init__(self, shape, real_out_is_enough=False, dtype="f32"):
        sfx = _sfx(dtype)
        self.shape = tuple(int(v) for v in shape)
        self.complex_shape = self.shape[:-1] + (self.shape[-1] // 2 + 1,)
        arr = (ctypes.c_uint * len(self.shape))(*self.shape)
        super().__init__(_call(f"kfr_dft_real_create_md_plan_{sfx}", len(self.shape), ctypes.cast(arr, _P),
                               bool(real_out_is_enough)), sfx)

    def execute(self, out, inp, temp=None, inverse=False):
        op = "execute_inverse" if inverse else "execute"
        _call(self._fn(op), self.handle, _addr(out), _addr(inp), _addr(temp))

    def execute_batch(self, out, inp, batch, temp=None, inverse=False, stream=None):
        op = "execute_inverse_batch" if inverse else "execute_batch"
        _call(self._fn(op), self.handle, batch, _addr(out), _addr(inp), _addr(temp), _stream_addr(stream))


class dft_plan_real(_plan):
    """Real DFT of even length `size` (dft_plan_real<T>), CCs (N/2+1 bins) or Perm (N/2 bins) packing."""

    _prefix = "kfr_dft_real"

    def __init__(self, size: int, fmt="CCs", dtype="f32"):
        sfx = _sfx(dtype)
        self.fmt = CCs if fmt in ("CCs", CCs, "ccs") else Perm
        self.n = size
        super().__init__(_call(f"kfr_dft_real_create_plan_{sfx}", size, self.fmt), sfx)

    @property
    def complex_size(self):
        return self.n // 2 + 1 if self.fmt == CCs else self.n // 2

    @property
    def size(self):
        return _call(self._fn("get_size"), self.handle)

    @property
    def temp_size(self):
        return _call(self._fn("get_temp_size"), self.handle)

    def execute(self, out, inp, temp=None, inverse=False):
        op = "execute_inverse" if inverse else "execute"
        _call(self._fn(op), self.handle, _addr(out), _addr(inp), _addr(temp))

    def execute_batch(self, out, inp, batch, temp=None, inverse=False, stream=None):
        op = "execute_inverse_batch" if inverse else "execute_batch"
        _call(self._fn(op), self.handle, batch, _addr(out), _addr(inp), _addr(temp), _stream_addr(stream))

    def adjoint_batch(self, grad_in, grad_out, batch, inverse=False, stream=None):
        """Gradient of the input of execute_batch(inverse) from the gradient of its output."""
        op = "adjoint_inverse_batch" if inverse else "adjoint_batch"
        _call(self._fn(op), self.handle, batch, _addr(grad_in), _addr(grad_out), None, _stream_addr(stream))


class dct_plan(_plan):
    """DCT-II (forward) / DCT-III with X0 halved (inverse), unscaled (dct_plan<T>)."""

    _prefix = "kfr_dct"

    def __init__(self, size: int, dtype="f32"):
        sfx = _sfx(dtype)
        super().__init__(_call(f"kfr_dct_create_plan_{sfx}", size), sfx)

    @property
    def size(self):
        return _call(self._fn("get_size"), self.handle)

    @property
    def temp_size(self):
        return _call(self._fn("get_temp_size"), self.handle)

    def execute(self, out, inp, temp=None, inverse=False):
        op = "execute_inverse" if inverse else "execute"
        _call(self._fn(op), self.handle, _addr(out), _addr(inp), _addr(temp))

    def execute_batch(self, out, inp, batch, temp=None, inverse=False, stream=None):
        _call(self._fn("execute_batch"), self.handle, batch, _addr(out), _addr(inp), _addr(temp), bool(inverse),
              _stream_addr(stream))

    def adjoint_batch(self, grad_in, grad_out, batch, inverse=False, stream=None):
        """Gradient of the input of execute_batch(inverse) from the gradient of its output."""
        _call(self._fn("adjoint_batch"), self.handle, batch, _addr(grad_in), _addr(grad_out), None, bool(inverse),
              _stream_addr(stream))


def fir_backward(taps, x, grad_y, grad_x=None, grad_taps=None, channels=1, stream=None):
    """Gradients of the causal FIR convolution a convolution filter applies from a reset state (device tensors;
    x and grad_y hold `channels` signals back to back)."""
    n = _numel(x) // channels
    _call(f"kfr_fir_backward_{_conv_sfx(x)}", _addr(taps), _numel(taps), channels, n, _addr(x), _addr(grad_y),
          _addr(grad_x), _addr(grad_taps), _stream_addr(stream))


class dft_plan_uneven(_plan):
    """Many complex signals of uneven lengths stored back to back, one persistent launch (c32)."""

    _prefix = "kfr_dft_uneven"

    def __init__(self, lengths, autotune=True):
        arr = np.ascontiguousarray(np.asarray(lengths, dtype=np.uint64))
        self._lengths = arr
        h = _call("kfr_dft_create_uneven_plan_f32", arr.ctypes.data, len(arr), bool(autotune))
        super().__init__(h, "f32")

    def close(self):
        if getattr(self, "handle", None):
            lib().kfr_dft_uneven_delete_plan_f32(self.handle)
            self.handle = None

    @property
    def size(self):
        return _call("kfr_dft_uneven_get_size_f32", self.handle)

    def execute(self, out, inp, inverse=False, stream=None):
        _call("kfr_dft_uneven_execute_f32", self.handle, _addr(out), _addr(inp), bool(inverse), _stream_addr(stream))

    def execute_per_signal(self, out, inp, inverse=False, stream=None):
        _call("kfr_dft_uneven_execute_per_signal_f32", self.handle, _addr(out), _addr(inp), bool(inverse),
              _stream_addr(stream))

    def describe(self) -> str:
        buf = ctypes.create_string_buffer(512)
        _call("kfr_dft_uneven_describe_f32", self.handle, buf, 512)
        return buf.value.decode()


class convolve_filter(_plan):
    """Streaming FFT convolution filter (convolve_filter<T>); state persists across apply() until reset()."""

    _prefix = "kfr_filter"

    def __init__(self, taps, block_size: int = 1024, dtype=None, channels: int = 1):
        if dtype is None:
            dtype = getattr(taps, "dtype", "f32")
        sfx = _sfx(dtype)
        if isinstance(taps, np.ndarray):
            taps = np.ascontiguousarray(taps, dtype=np.float32 if sfx == "f32" else np.float64)
        self._taps = taps
        self.channels = channels
        n = taps.numel() if hasattr(taps, "numel") else len(taps)
        if channels == 1:
            h = _call(f"kfr_filter_create_convolution_plan_{sfx}", _addr(taps), n, block_size)
        else:
            h = _call(f"kfr_filter_create_convolution_plan_channels_{sfx}", _addr(taps), n, block_size, channels)
        super().__init__(h, sfx)

    def apply(self, out, inp, size=None):
        """size: samples per channel (default: all of inp over the plan's channels)."""
        if size is None:
            size = _numel(inp) // self.channels
        _call(self._fn("process"), self.handle, _addr(out), _addr(inp), size)

    def reset(self):
        _call(self._fn("reset"), self.handle)


class fir_filter(convolve_filter):
    """Streaming FIR filter (fir_filter<T>, include/kfr/dsp/fir.hpp; kfr_filter_create_fir_plan_*): y[n] =
    sum_k taps[k] x[n - k], state across apply() until reset(), computed through the FFT convolution path."""

    def __init__(self, taps, dtype=None):
        if dtype is None:
            dtype = getattr(taps, "dtype", "f32")
        sfx = _sfx(dtype)
        if isinstance(taps, np.ndarray):
            taps = np.ascontiguousarray(taps, dtype=np.float32 if sfx == "f32" else np.float64)
        self._taps = taps
        self.channels = 1
        n = taps.numel() if hasattr(taps, "numel") else len(taps)
        _plan.__init__(self, _call(f"kfr_filter_create_fir_plan_{sfx}", _addr(taps), n), sfx)


def _conv_sfx(x):
    d = str(getattr(x, "dtype", ""))
    table = {"float32": "f32", "float64": "f64", "complex64": "c32", "complex128": "c64", "torch.float32": "f32",
             "torch.float64": "f64", "torch.complex64": "c32", "torch.complex128": "c64"}
    if d not in table:
        raise ValueError(f"unsupported dtype {d}")
    return table[d]


def _numel(x):
    if isinstance(x, np.ndarray):
        return x.size
    return x.numel() if hasattr(x, "numel") else len(x)


def _like(x, n):
    if isinstance(x, np.ndarray):
        return np.zeros(n, dtype=x.dtype)
    import torch

    return torch.zeros(n, dtype=x.dtype, device=x.device)


def convolve(a, b):
    """Linear convolution (convolve, include/kfr/dft/convolution.hpp:53-58); complex inputs keep only the
    real part, as the reference does."""
    out = _like(a, _numel(a) + _numel(b) - 1)
    _call(f"kfr_convolve_{_conv_sfx(a)}", _addr(out), _addr(a), _numel(a), _addr(b), _numel(b))
    return out


def correlate(a, b):
    """Correlation: convolution with b reversed (not conjugated) (include/kfr/dft/convolution.hpp:61-66)."""
    out = _like(a, _numel(a) + _numel(b) - 1)
    _call(f"kfr_correlate_{_conv_sfx(a)}", _addr(out), _addr(a), _numel(a), _addr(b), _numel(b))
    return out


def autocorrelate(a):
    """Lags 0 .. n-1 of correlate(a, a) (include/kfr/dft/convolution.hpp:69-76); real inputs."""
    out = _like(a, _numel(a))
    _call(f"kfr_autocorrelate_{_conv_sfx(a)}", _addr(out), _addr(a), _numel(a))
    return out


def fft_multiply(dest, src1, src2, size, batch=1, fmt="CCs", accumulate_from=None, stream=None):
    """fft_multiply / fft_multiply_accumulate (include/kfr/dft/fft.hpp:983-1020) on device buffers: dest =
    [accumulate_from +] src1 * src2 over `batch` spectra of `size` elements; src2 holding `size` elements only
    is one spectrum shared by every signal.  fmt "Perm" multiplies element 0 part by part."""
    sfx = "f64" if "128" in str(getattr(dest, "dtype", "")) else "f32"
    shared = _numel(src2) == size and batch > 1
    f = 1 if fmt in ("CCs", 1) else 0
    if accumulate_from is None:
        _call(f"kfr_fft_multiply_{sfx}", _addr(dest), _addr(src1), _addr(src2), size, batch, shared, f,
              _stream_addr(stream))
    else:
        _call(f"kfr_fft_multiply_accumulate_{sfx}", _addr(dest), _addr(accumulate_from), _addr(src1), _addr(src2),
              size, batch, shared, f, _stream_addr(stream))
    return dest


def allocate(size: int, alignment: int = 64) -> int:
    """kfr_allocate_aligned: host memory, pinned when a GPU is present."""
    return _call("kfr_allocate_aligned", size, alignment)


def deallocate(ptr: int) -> None:
    _call("kfr_deallocate", ptr)


def version_string() -> str:
    return lib().kfr_version_string().decode()
