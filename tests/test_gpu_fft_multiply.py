"""Device fft_multiply / fft_multiply_accumulate (include/kfr/dft/fft.hpp:983-1020) through the C ABI
(kfr_fft_multiply_*, kfr_fft_multiply_accumulate_*) against the reference-generated fixtures and the oracle:
CCs and Perm packings, f32 and f64, one spectrum per signal or one shared by all, the two- and three-operand
accumulate forms.  Each output element is one complex product (and one sum), so the bound is a few units in
the last place of the element's magnitude."""
import numpy as np
import pytest

from conftest import load_golden

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu

EPS = {"f32": 2.0**-23, "f64": 2.0**-52}


def _close(got, want, scale, prec, ulps=4):
    err = np.abs(got - want)
    assert np.all(err <= ulps * EPS[prec] * np.maximum(scale, 1e-30)), float(np.max(err / scale))


@pytest.mark.parametrize("prec", ["f32", "f64"])
@pytest.mark.parametrize("fmt", ["ccs", "perm"])
def test_fft_multiply_matches_reference(prec, fmt):
    f = load_golden("fft_multiply.npz")
    a, b, c = f[f"a_{prec}"], f[f"b_{prec}"], f[f"c_{prec}"]
    m = a.shape[1] if fmt == "ccs" else a.shape[1] - 1
    a, b, c = (np.ascontiguousarray(v[:, :m]) for v in (a, b, c))
    da, db, dc = (torch.from_numpy(v).cuda() for v in (a, b, c))
    out = torch.empty_like(da)
    kfmt = "CCs" if fmt == "ccs" else "Perm"
    k.fft_multiply(out, da, db, m, batch=3, fmt=kfmt)
    scale = np.abs(a) * np.abs(b) + np.abs(a.real * b.real) + np.abs(a.imag * b.imag)
    _close(out.cpu().numpy(), f[f"mul_{fmt}_{prec}"], scale, prec)
    # three-operand accumulate: out = c + a * b
    k.fft_multiply(out, da, db, m, batch=3, fmt=kfmt, accumulate_from=dc)
    _close(out.cpu().numpy(), f[f"mac_{fmt}_{prec}"], scale + np.abs(c), prec, 8)
    # two-operand accumulate in place: dest = dest + a * b
    acc = dc.clone()
    k.fft_multiply(acc, da, db, m, batch=3, fmt=kfmt, accumulate_from=acc)
    _close(acc.cpu().numpy(), f[f"mac_{fmt}_{prec}"], scale + np.abs(c), prec, 8)


@pytest.mark.parametrize("perm", [False, True])
def test_fft_multiply_shared_filter_spectrum_on_a_stream(orc, perm):
    """One filter spectrum applied to a batch of 64 signal spectra, enqueued on a stream."""
    rng = np.random.default_rng(11)
    n, batch = 4097, 64
    x = (rng.standard_normal((batch, n)) + 1j * rng.standard_normal((batch, n))).astype(np.complex64)
    h = (rng.standard_normal(n) + 1j * rng.standard_normal(n)).astype(np.complex64)
    dx, dh = torch.from_numpy(x).cuda(), torch.from_numpy(h).cuda()
    out = torch.empty_like(dx)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        k.fft_multiply(out, dx, dh, n, batch=batch, fmt="Perm" if perm else "CCs", stream=s)
    s.synchronize()
    want = orc.fft_multiply(x, np.broadcast_to(h, x.shape), perm=perm)
    _close(out.cpu().numpy(), want, np.abs(x) * np.abs(h) + np.abs(x.real * h.real) + np.abs(x.imag * h.imag), "f32")


def test_fft_multiply_rejects_host_pointers():
    x = np.zeros(16, np.complex64)
    L = k.lib()
    L.kfr_fft_multiply_f32(x.ctypes.data, x.ctypes.data, x.ctypes.data, 16, 1, False, 1, None)
    assert b"device pointers" in L.kfr_last_error()


def test_fft_multiply_empty_is_a_no_op():
    """size 0 or batch 0: nothing runs and no error is reported (the reference's empty univectors)."""
    x = torch.ones(4, dtype=torch.complex64, device="cuda")
    L = k.lib()
    L.kfr_fft_multiply_f32(x.data_ptr(), x.data_ptr(), x.data_ptr(), 0, 1, False, 1, None)
    assert L.kfr_last_error() == b""
    L.kfr_fft_multiply_accumulate_f32(x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), 4, 0, False, 1, None)
    assert L.kfr_last_error() == b""
    assert torch.equal(x, torch.ones_like(x))
