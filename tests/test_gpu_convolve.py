"""Whole-signal convolve / correlate / autocorrelate on the GPU (kfr_convolve_*, kfr_correlate_*,
kfr_autocorrelate_*), against fixtures from KFR's own convolve / correlate and the reference's known answers
(tests/dft_test.cpp:107-167)."""
import numpy as np
import pytest

from conftest import load_golden
from oracle.oracle import c32_tolerance, c64_tolerance, rel_rms

torch = pytest.importorskip("torch")
import kfr_gb300 as k  # noqa: E402

pytestmark = pytest.mark.gpu


def test_known_answers():
    a = np.array([1, 2, 3, 4, 5], dtype=np.float32)
    b = np.array([0.25, 0.5, 1.0, -2.0, 1.5], dtype=np.float32)
    conv = np.array([0.25, 1.0, 2.75, 2.5, 3.75, 3.5, 1.5, -4.0, 7.5])
    corr = np.array([1.5, 1.0, 1.5, 2.5, 3.75, -4.0, 7.75, 3.5, 1.25])
    assert np.sqrt(np.mean((k.convolve(a, b) - conv) ** 2)) < 1e-4
    assert np.sqrt(np.mean((k.correlate(a, b) - corr) ** 2)) < 1e-4
    ca, cb = a.astype(np.complex64), b.astype(np.complex64)
    assert np.sqrt(np.mean(np.abs(k.convolve(ca, cb) - conv) ** 2)) < 1e-4
    assert np.sqrt(np.mean(np.abs(k.correlate(ca, cb) - corr) ** 2)) < 1e-4


@pytest.mark.parametrize("prec", ["f32", "f64"])
def test_reference_fixtures(prec):
    g = load_golden("convolution.npz")
    rdt, cdt = (np.float32, np.complex64) if prec == "f32" else (np.float64, np.complex128)
    # the per-transform tolerance at n = len(a) + len(b) (measured: at most 0.52 of it in f32, 0.42 in f64)
    tol = c32_tolerance if prec == "f32" else c64_tolerance
    for i in range(int(g["npairs"])):
        a, b = g[f"a_{i}"].astype(rdt), g[f"b_{i}"].astype(rdt)
        n = len(a) + len(b)
        assert rel_rms(k.convolve(a, b), g[f"real_0_{i}"]) <= tol(n), i
        assert rel_rms(k.correlate(a, b), g[f"real_1_{i}"]) <= tol(n), i
        ac, bc = g[f"ac_{i}"].astype(cdt), g[f"bc_{i}"].astype(cdt)
        # the reference keeps only the real part of a complex convolution
        got = k.convolve(ac, bc)
        assert np.all(got.imag == 0)
        assert rel_rms(got, g[f"cplx_0_{i}"]) <= tol(n), i
        assert rel_rms(k.correlate(ac, bc), g[f"cplx_1_{i}"]) <= tol(n), i


def test_long_signal_device_and_autocorrelate():
    rng = np.random.default_rng(8)
    a = rng.standard_normal(1 << 20).astype(np.float32)
    b = rng.standard_normal(1023).astype(np.float32)
    want = np.convolve(a.astype(np.float64), b.astype(np.float64))
    ad, bd = torch.from_numpy(a).cuda(), torch.from_numpy(b).cuda()
    got = k.convolve(ad, bd)
    assert got.is_cuda
    assert rel_rms(got.cpu().numpy(), want) <= c32_tolerance(len(want))  # measured 0.21 of it
    x = rng.standard_normal(5000)
    full = np.correlate(x, x, mode="full")
    assert rel_rms(k.autocorrelate(x), full[len(x) - 1:]) <= 1e-12
    assert k.lib().kfr_dft_cache_size() > 0
    k.lib().kfr_dft_cache_clear()
    assert k.lib().kfr_dft_cache_size() == 0
